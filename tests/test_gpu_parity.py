"""GPU parity: the C-ABI engine against the CPU oracle on identical inputs.

Tolerances (FP32): seismograms <= 1e-5 and gradients <= 1e-4 relative L2, the
bounds the engine is specified to meet against fd2dmpi.  Because the kernels
keep the reference's operation order and form no FMA, the FP32 results are
expected to be bit-identical to the oracle; that is asserted separately.
FP64 engine vs FP64 oracle: <= 1e-12.
"""
import numpy as np
import pytest

from oracle import oracle as O
from swit_gb300 import Engine, SwitError, survey

pytestmark = pytest.mark.gpu

SEIS_TOL = 1e-5
GRAD_TOL = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)


def case(**kw):
    s = survey.small(**kw)
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, free_surface=s.free_surface)
    return s, pb


def engine(s, **kw):
    return Engine(**s.engine_args(), **kw)


@pytest.fixture(scope="module")
def base():
    s, pb = case()
    src = s.source()
    rho = s.rho(s.vp_true)
    ref = O.forward(pb, s.vp_true, rho, src, store=True)
    obs = O.forward(pb, s.vp_init, rho, src, store=False)["seis"]
    adj = (ref["seis"] - obs).astype(np.float32)
    grad = O.adjoint(pb, s.vp_true, rho, src, adj, ref)
    return dict(s=s, pb=pb, src=src, rho=rho, ref=ref, obs=obs, adj=adj, grad=grad)


def test_forward_seismograms_match_oracle(base):
    s = base["s"]
    with engine(s) as e:
        e.set_model(s.vp_true, base["rho"])
        seis = e.forward(base["src"], save_boundary=True)
    assert rel(seis, base["ref"]["seis"]) <= SEIS_TOL
    np.testing.assert_array_equal(seis, base["ref"]["seis"])


@pytest.mark.parametrize("kernel", ["split", "walk", "vec", "cluster", "band"])
def test_boundary_strips_and_end_states_match_oracle(base, kernel):
    s = base["s"]
    with engine(s, kernel=kernel) as e:
        e.set_model(s.vp_true, base["rho"])
        e.forward(base["src"], save_boundary=True)
        snap = e.export_snapshot()
    for k in ("boundary", "p_end", "u_end", "w_end"):
        assert rel(snap[k], base["ref"][k]) <= SEIS_TOL, k
        np.testing.assert_array_equal(snap[k], base["ref"][k], err_msg=k)


def test_gradient_and_illumination_match_oracle(base):
    s = base["s"]
    with engine(s) as e:
        e.set_model(s.vp_true, base["rho"])
        e.forward(base["src"], save_boundary=True)
        g, fw, bk = e.backward(base["adj"])
    for mine, k in ((g, "g"), (fw, "fw"), (bk, "bk")):
        assert rel(mine, base["grad"][k]) <= GRAD_TOL, k
        np.testing.assert_array_equal(mine, base["grad"][k], err_msg=k)


def test_gradient_l2_single_call_matches_oracle(base):
    s, pb = base["s"], base["pb"]
    ref = O.gradient(pb, s.vp_true, base["rho"], base["src"], base["obs"])
    with engine(s) as e:
        e.set_model(s.vp_true, base["rho"])
        out = e.gradient_l2(base["src"], base["obs"], return_seis=True)
    np.testing.assert_array_equal(out["seis"], base["ref"]["seis"])
    for mine, k in ((out["grad"], "g"), (out["illum_fw"], "fw"), (out["illum_bk"], "bk")):
        np.testing.assert_array_equal(mine, ref[k], err_msg=k)
    r = (base["ref"]["seis"].astype(np.float64) - base["obs"])
    want = np.sum(np.sqrt(np.sum(r * r * s.dt, axis=-1)))
    assert abs(out["misfit"] - want) <= 1e-6 * want


@pytest.mark.parametrize("opts", [dict(path="plain"), dict(shots_per_batch=2), dict(kernel="walk", block_x=8),
                                  dict(kernel="walk", block_x=32), dict(kernel="walk", path="plain"),
                                  dict(kernel="split"), dict(kernel="split", block_x=8),
                                  dict(kernel="split", block_x=1), dict(kernel="split", path="plain"),
                                  dict(kernel="split", shots_per_batch=2), dict(kernel="vec"),
                                  dict(kernel="vec", path="plain"), dict(kernel="vec", shots_per_batch=2),
                                  dict(kernel="vec", block_x=1), dict(kernel="vec", block_x=2),
                                  dict(kernel="vec", block_x=32), dict(kernel="vec", block_x=64),
                                  dict(kernel="cluster"), dict(kernel="cluster", block_x=1),
                                  dict(kernel="cluster", block_x=2), dict(kernel="cluster", block_x=3),
                                  dict(kernel="cluster", block_x=7), dict(kernel="cluster", path="plain"),
                                  dict(kernel="cluster", shots_per_batch=2), dict(kernel="hybrid"),
                                  dict(kernel="hybrid", block_x=3, shots_per_batch=2),
                                  dict(kernel="hybrid", path="plain"), dict(kernel="band"),
                                  dict(kernel="band", block_x=1), dict(kernel="band", block_x=3),
                                  dict(kernel="band", block_x=7, shots_per_batch=2), dict(kernel="band", path="plain"),
                                  dict(kernel="vec", shots_per_batch=1, graph_branches=1),
                                  dict(kernel="vec", shots_per_batch=1, graph_branches=3),
                                  dict(kernel="vec", shots_per_batch=1, graph_branches=4),
                                  dict(kernel="split", shots_per_batch=1, graph_branches=3),
                                  dict(kernel="band", shots_per_batch=1, graph_branches=4)])
def test_launch_variants_are_identical(base, opts):
    s = base["s"]
    with engine(s, **opts) as e:
        e.set_model(s.vp_true, base["rho"])
        seis = e.forward(base["src"], save_boundary=True)
        g, fw, bk = e.backward(base["adj"])
        e.check()
    np.testing.assert_array_equal(seis, base["ref"]["seis"])
    np.testing.assert_array_equal(g, base["grad"]["g"])
    np.testing.assert_array_equal(bk, base["grad"]["bk"])


@pytest.mark.parametrize("kernel", ["walk", "split", "vec", "cluster", "band"])
def test_fp64_build_matches_fp64_oracle(base, kernel):
    s, pb = base["s"], base["pb"]
    ref = O.forward(pb, s.vp_true, base["rho"], base["src"], store=True, fp64=True)
    gref = O.adjoint(pb, s.vp_true, base["rho"], base["src"], base["adj"], ref, fp64=True)
    with engine(s, precision="fp64", kernel=kernel) as e:
        e.set_model(s.vp_true, base["rho"])
        seis = e.forward(base["src"], save_boundary=True)
        g, fw, bk = e.backward(base["adj"])
    assert seis.dtype == np.float64
    assert rel(seis, ref["seis"]) <= 1e-12
    assert rel(g, gref["g"]) <= 1e-12 and rel(fw, gref["fw"]) <= 1e-12 and rel(bk, gref["bk"]) <= 1e-12


def test_repeated_backward_after_one_forward(base):
    s = base["s"]
    with engine(s) as e:
        e.set_model(s.vp_true, base["rho"])
        e.forward(base["src"], save_boundary=True)
        g1 = e.backward(base["adj"])[0]
        g2 = e.backward(base["adj"])[0]
    np.testing.assert_array_equal(g1, base["grad"]["g"])
    np.testing.assert_array_equal(g2, base["grad"]["g"])


@pytest.mark.parametrize("kernel", ["walk", "split", "vec", "cluster", "band"])
def test_edge_geometry_surface_receivers_deep_source_uneven_traces(kernel):
    """Receivers on z = 0 (moved one node down), a source deep enough that the
    reconstruction subtracts it (fdcore.f90:250-256), shots with different
    receiver counts, a receiver shared by two grid-coincident positions."""
    s = survey.small(nx=40, nz=36, npml=8, nt=240, ns=3, zs=120.0, zr=0.0)
    rec = s.rec_xz.copy()
    rec[:, 5] = rec[:, 4] + np.array([3.0, 0.0], np.float32)  # same grid node as receiver 4
    s.rec_xz = rec
    ng = np.array([s.ng, s.ng - 7, 1], np.int32)
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, ng=ng)
    src = s.source()
    rho = s.rho(s.vp_true)
    ref = O.forward(pb, s.vp_true, rho, src, store=True)
    adj = np.random.default_rng(3).standard_normal(ref["seis"].shape).astype(np.float32)
    for i in range(3):
        adj[i, ng[i]:] = 0
    gref = O.adjoint(pb, s.vp_true, rho, src, adj, ref)
    with Engine(**s.engine_args(), ng=ng, kernel=kernel) as e:
        e.set_model(s.vp_true, rho)
        seis = e.forward(src, save_boundary=True)
        g, fw, bk = e.backward(adj)
    np.testing.assert_array_equal(seis, ref["seis"])
    np.testing.assert_array_equal(g, gref["g"])
    np.testing.assert_array_equal(fw, gref["fw"])
    np.testing.assert_array_equal(bk, gref["bk"])


@pytest.mark.parametrize("kernel", ["walk", "split", "vec", "cluster", "band"])
def test_no_free_surface(kernel):
    s, _ = case(nt=200)
    s.free_surface = 0
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, free_surface=0)
    src = s.source()
    rho = s.rho(s.vp_true)
    ref = O.forward(pb, s.vp_true, rho, src, store=True)
    adj = (ref["seis"] * 0.5).astype(np.float32)
    gref = O.adjoint(pb, s.vp_true, rho, src, adj, ref)
    with engine(s, kernel=kernel) as e:
        e.set_model(s.vp_true, rho)
        seis = e.forward(src, save_boundary=True)
        g, fw, bk = e.backward(adj)
    np.testing.assert_array_equal(seis, ref["seis"])
    np.testing.assert_array_equal(g, gref["g"])


def test_device_arrays_and_streams(base):
    import torch
    s = base["s"]
    with engine(s) as e:
        vp = torch.from_numpy(s.vp_true).cuda()
        rho = torch.from_numpy(base["rho"]).cuda()
        e.set_model(vp, rho)
        src = torch.from_numpy(base["src"]).cuda()
        seis = e.forward(src, save_boundary=True)
        g, fw, bk = e.backward(torch.from_numpy(base["adj"]).cuda())
        torch.cuda.synchronize()
    np.testing.assert_array_equal(seis.cpu().numpy(), base["ref"]["seis"])
    np.testing.assert_array_equal(g.cpu().numpy(), base["grad"]["g"])


def test_state_and_model_errors(base):
    s = base["s"]
    with engine(s) as e:
        with pytest.raises(SwitError, match="SWIT_E_STATE"):
            e.forward(base["src"])
        bad = s.vp_true.copy()
        bad[3, 4] = np.nan
        with pytest.raises(SwitError, match="SWIT_E_MODEL"):
            e.set_model(bad, base["rho"])
        with pytest.raises(SwitError, match="SWIT_E_CFL"):
            e.set_model(s.vp_true * 20, base["rho"])
        e.set_model(s.vp_true, base["rho"])
        with pytest.raises(SwitError, match="SWIT_E_STATE"):
            e.backward(base["adj"])


@pytest.mark.parametrize("kernel", ["walk", "vec", "cluster", "band"])
@pytest.mark.parametrize("npml", [8, 9, 10, 11])
def test_vec_kernels_every_mirror_alignment(npml, kernel):
    """The vectorised kernels own 4 rows per thread; npml mod 4 decides whether
    the free-surface mirror rows fs-1 and fs / fs+1 share a vector or not."""
    s = survey.small(nx=36, nz=28, npml=npml, nt=160, ns=2, zs=70.0, zr=0.0)
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz)
    src = s.source()
    rho = s.rho(s.vp_true)
    ref = O.forward(pb, s.vp_true, rho, src, store=True)
    adj = np.random.default_rng(npml).standard_normal(ref["seis"].shape).astype(np.float32)
    gref = O.adjoint(pb, s.vp_true, rho, src, adj, ref)
    with engine(s, kernel=kernel, **({"block_x": 5} if kernel == "cluster" else {})) as e:
        e.set_model(s.vp_true, rho)
        seis = e.forward(src, save_boundary=True)
        g, fw, bk = e.backward(adj)
    np.testing.assert_array_equal(seis, ref["seis"])
    np.testing.assert_array_equal(g, gref["g"])
    np.testing.assert_array_equal(fw, gref["fw"])
    np.testing.assert_array_equal(bk, gref["bk"])


@pytest.mark.parametrize("kernel", ["vec", "split", "walk", "cluster", "band"])
def test_import_snapshot_replaces_the_forward_run(base, kernel):
    """The adjoint job from saved files (fd2dmpi/solver.f90:212-228): export the
    strips and end states, load them into a fresh engine, run only the reverse loop."""
    s = base["s"]
    with engine(s, kernel=kernel) as e:
        e.set_model(s.vp_true, base["rho"])
        e.forward(base["src"], save_boundary=True)
        snap = e.export_snapshot()
    with engine(s, kernel=kernel) as e2:
        e2.set_model(s.vp_true, base["rho"])
        e2.import_snapshot(base["src"], snap["boundary"], snap["p_end"], snap["u_end"], snap["w_end"])
        g, fw, bk = e2.backward(base["adj"])
    np.testing.assert_array_equal(g, base["grad"]["g"])
    np.testing.assert_array_equal(fw, base["grad"]["fw"])
    np.testing.assert_array_equal(bk, base["grad"]["bk"])


def test_cluster_variant_rejects_a_grid_that_does_not_fit_on_chip():
    """3120 x 720 PML-grid columns need more than 16 CTAs' shared memory."""
    s = survey.small(nx=3000, nz=600, npml=60, nt=10, ns=1)
    with pytest.raises(SwitError, match="SWIT_E_LIMIT"):
        Engine(**s.engine_args(), kernel="cluster")


@pytest.mark.parametrize("opts", [dict(checkpoint_every=1), dict(checkpoint_every=7), dict(checkpoint_every=64),
                                  dict(checkpoint_every=298), dict(checkpoint_every=299),
                                  dict(checkpoint_every=1000), dict(checkpoint_every=13, shots_per_batch=2),
                                  dict(checkpoint_every=13, shots_per_batch=1, graph_branches=3),
                                  dict(checkpoint_every=13, path="plain"), dict(checkpoint_every=13, kernel="band"),
                                  dict(checkpoint_every=1, kernel="walk"), dict(checkpoint_every=13, kernel="walk"),
                                  dict(checkpoint_every=298, kernel="walk"),
                                  dict(checkpoint_every=13, kernel="walk", shots_per_batch=1, graph_branches=3)])
def test_checkpointed_recomputation_gives_the_boundary_saving_results(base, opts):
    """Checkpoints every k steps instead of strips; the reverse loop re-runs each
    segment to regenerate its strips, so every output is bit-identical to the
    boundary-saving run (and to the oracle), also on a second backward."""
    s = base["s"]
    with engine(s, **opts) as e:
        e.set_model(s.vp_true, base["rho"])
        seis = e.forward(base["src"], save_boundary=True)
        g, fw, bk = e.backward(base["adj"])
        g2, fw2, bk2 = e.backward(base["adj"])
        e.check()
    np.testing.assert_array_equal(seis, base["ref"]["seis"])
    for a, b in ((g, "g"), (fw, "fw"), (bk, "bk"), (g2, "g"), (fw2, "fw"), (bk2, "bk")):
        np.testing.assert_array_equal(a, base["grad"][b])


def test_checkpointed_gradient_l2_and_snapshot_refusal(base):
    s = base["s"]
    with engine(s) as e0:
        e0.set_model(s.vp_init, base["rho"])
        r0 = e0.gradient_l2(base["src"], base["ref"]["seis"])
    with engine(s, checkpoint_every=40) as e:
        e.set_model(s.vp_init, base["rho"])
        r = e.gradient_l2(base["src"], base["ref"]["seis"])
        with pytest.raises(SwitError, match="SWIT_E_STATE"):
            e.export_snapshot()
    for k in ("grad", "illum_fw", "illum_bk"):
        np.testing.assert_array_equal(r[k], r0[k])
    assert r["misfit"] == r0["misfit"]


@pytest.mark.parametrize("opts,launches", [(dict(kernel="vec", shots_per_batch=1, graph_branches=2), 3 * 256),
                                           (dict(kernel="vec", shots_per_batch=1, graph_branches=3), 3 * 256),
                                           (dict(kernel="vec", shots_per_batch=2, graph_branches=1), 2 * 256),
                                           (dict(kernel="split"), 299)])
def test_kernel_profile_counts_launches_and_leaves_results_intact(base, opts, launches):
    """swit_profile_kernels times the batched vec kernels each in a graph of
    min(nt-1, 256) steps of every batch (the split kernels: every launch of a
    forward and reverse loop, all shots per launch); the engine still computes the
    oracle's results afterwards."""
    s = base["s"]
    assert s.ns == 3 and s.nt == 300
    with engine(s, **opts) as e:
        e.set_model(s.vp_true, base["rho"])
        e.forward(base["src"], save_boundary=True)
        e.backward(base["adj"])
        prof = e.profile_kernels()
        seis = e.forward(base["src"], save_boundary=True)
        g, fw, bk = e.backward(base["adj"])
    assert set(prof) == {"fwd_p", "fwd_uw", "bwd_uw", "bwd_p"}
    for k, v in prof.items():
        assert v["launches"] == launches, k
        assert v["mean_ms"] > 0, k
    np.testing.assert_array_equal(seis, base["ref"]["seis"])
    np.testing.assert_array_equal(g, base["grad"]["g"])


@pytest.mark.parametrize("opts", [dict(shots_per_batch=1), dict(shots_per_batch=1, graph_branches=2),
                                  dict(shots_per_batch=1, checkpoint_every=40), dict(shots_per_batch=2)])
def test_loops_split_into_several_graphs_give_the_same_bits(base, opts, monkeypatch):
    """With a node bound of 1000 per graph every captured loop becomes one graph
    per batch (or per round of branches); results stay the oracle's."""
    monkeypatch.setenv("SWIT_GRAPH_NODES", "1000")
    s = base["s"]
    with engine(s, **opts) as e:
        e.set_model(s.vp_true, base["rho"])
        seis = e.forward(base["src"], save_boundary=True)
        g, fw, bk = e.backward(base["adj"])
        g2, _, _ = e.backward(base["adj"])
    np.testing.assert_array_equal(seis, base["ref"]["seis"])
    np.testing.assert_array_equal(g, base["grad"]["g"])
    np.testing.assert_array_equal(g2, base["grad"]["g"])
    np.testing.assert_array_equal(bk, base["grad"]["bk"])


@pytest.mark.parametrize("adjoint", ["fd2dmpi", "exact"])
def test_engine_calls_capture_into_a_cuda_graph(base, adjoint):
    """With device buffers the C-ABI calls are stream-ordered with no host
    synchronisation, so once an engine has built its own graphs a caller can
    capture forward + backward into a graph of its own and replay it."""
    import torch
    s = base["s"]
    with engine(s, adjoint=adjoint) as e:
        e.set_model(torch.from_numpy(s.vp_true).cuda(), torch.from_numpy(base["rho"]).cuda())
        src = torch.from_numpy(base["src"]).cuda()
        adj = torch.from_numpy(base["adj"]).cuda()
        seis = torch.zeros((s.ns, s.ng, s.nt), dtype=torch.float32, device="cuda")
        g = torch.zeros((s.nx, s.nz), dtype=torch.float32, device="cuda")
        fw, bk = torch.zeros_like(g), torch.zeros_like(g)

        def step():
            e.forward(src, save_boundary=True, seis=seis)
            if adjoint == "exact":
                e.backward_exact(adj, grad=g)
            else:
                e.backward(adj, grad=g, illum_fw=fw, illum_bk=bk)

        step()  # builds the engine's graphs
        torch.cuda.synchronize()
        want_seis, want_g = seis.clone(), g.clone()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, capture_error_mode="thread_local"):
            step()
        seis.zero_()
        g.zero_()
        for _ in range(2):
            graph.replay()
        torch.cuda.synchronize()
    torch.testing.assert_close(seis, want_seis, rtol=0, atol=0)
    torch.testing.assert_close(g, want_g, rtol=0, atol=0)
    if adjoint == "fd2dmpi":
        np.testing.assert_array_equal(g.cpu().numpy(), base["grad"]["g"])


@pytest.fixture(scope="module")
def vel():
    """Oracle runs with vx and vz receivers (dev/solver/fdcore.f90:154-177, 465-485)."""
    s = survey.small()
    src = s.source()
    rho = s.rho(s.vp_true)
    out = {}
    for comp in ("vx", "vz"):
        pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, free_surface=s.free_surface,
                       comp=comp)
        ref = O.forward(pb, s.vp_true, rho, src, store=True)
        adj = (ref["seis"] * 1e3).astype(np.float32)
        out[comp] = dict(ref=ref, adj=adj, grad=O.adjoint(pb, s.vp_true, rho, src, adj, ref))
    return dict(s=s, src=src, rho=rho, out=out)


@pytest.mark.parametrize("kernel", ["vec", "walk"])
@pytest.mark.parametrize("comp", ["vx", "vz"])
@pytest.mark.parametrize("opts", [dict(), dict(path="plain"), dict(shots_per_batch=1, graph_branches=3),
                                  dict(checkpoint_every=40), dict(precision="fp64")])
def test_velocity_receivers_match_oracle(vel, comp, opts, kernel):
    s, o = vel["s"], vel["out"][comp]
    with engine(s, kernel=kernel, receiver_component=comp, **opts) as e:
        e.set_model(s.vp_true, vel["rho"])
        seis = e.forward(vel["src"], save_boundary=True)
        g, fw, bk = e.backward(o["adj"])
    if opts.get("precision") == "fp64":
        assert rel(seis, o["ref"]["seis"]) <= SEIS_TOL and rel(g, o["grad"]["g"]) <= GRAD_TOL
        return
    np.testing.assert_array_equal(seis, o["ref"]["seis"])
    np.testing.assert_array_equal(g, o["grad"]["g"])
    np.testing.assert_array_equal(fw, o["grad"]["fw"])
    np.testing.assert_array_equal(bk, o["grad"]["bk"])


def test_automatic_batches_fit_the_l2():
    """481x141 (npml 40), 49 shots: the reverse loop's state is about 3.1 MB per
    shot, so 0.7 of the GB300's L2 holds 28 shots in flight: 6 batches of at
    most 9 shots on 3 graph branches."""
    s = survey.config(1)
    with Engine(**s.engine_args()) as e:
        q = e.query()
    import torch
    l2 = getattr(torch.cuda.get_device_properties(0), "L2_cache_size", None)
    if not l2:
        pytest.skip("L2 size not reported")
    state = (3 * (s.nx + 80) * (s.nz + 80) + 6 * s.nx * s.nz) * 4
    inflight = int(0.7 * l2 / state)
    per_branch = max(1, inflight // 3)
    k = 3 * -(-s.ns // (3 * per_branch))
    assert q["graph_branches"] == 3 and q["shots_per_batch"] == -(-s.ns // k)
    if 120e6 < l2 < 135e6:  # GB300
        assert q["shots_per_batch"] == 9


@pytest.mark.parametrize("idx,ns,nt", [(0, 5, 2000), (1, 4, 800)])
def test_benchmark_configurations_match_oracle(idx, ns, nt):
    """The plain small configuration (201x101, dx 25 m, nt 2000, 5 shots) in full
    and the Marmousi-like one (481x141, npml 40) with 4 of its shots and 800
    steps, through the C ABI against the FP32 oracle on the same seeded inputs:
    seismograms within 1e-5 and gradient and illuminations within 1e-4 relative
    L2, the engine's specified bounds."""
    s = survey.config(idx, ns=ns, nt=nt)
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, free_surface=s.free_surface)
    rho = s.rho(s.vp_true)
    src = s.source()
    obs = O.forward(pb, s.vp_true, rho, src, store=False)["seis"]
    ref = O.gradient(pb, s.vp_init, rho, src, obs, return_seis=True)
    with Engine(**s.engine_args()) as e:
        e.set_model(s.vp_init, rho)
        out = e.gradient_l2(src, obs, return_seis=True)
    assert rel(out["seis"], ref["seis"]) <= SEIS_TOL
    for mine, k in ((out["grad"], "g"), (out["illum_fw"], "fw"), (out["illum_bk"], "bk")):
        assert rel(mine, ref[k]) <= GRAD_TOL, k


@pytest.mark.parametrize("block_x", [2, 3, 5, 16, 64])
@pytest.mark.parametrize("nz,npml", [(28, 9), (210, 10)])
def test_walk_tiles_narrower_than_the_halo_and_tall_columns(block_x, nz, npml):
    """Walk kernels: tiles of 2..64 columns (narrower than the 3-column halo of
    the x-stencils, and wider than the grid) and columns of 56 or 64 vectors
    (two warps, or three warps in two warp groups with an idle fourth warp):
    seismograms, strips, end states and gradient equal the oracle's."""
    s = survey.small(nx=37, nz=nz, npml=npml, nt=150, ns=3, zs=60.0, zr=0.0)
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz)
    src = s.source()
    rho = s.rho(s.vp_true)
    ref = O.forward(pb, s.vp_true, rho, src, store=True)
    adj = np.random.default_rng(block_x).standard_normal(ref["seis"].shape).astype(np.float32)
    gref = O.adjoint(pb, s.vp_true, rho, src, adj, ref)
    with engine(s, kernel="walk", block_x=block_x) as e:
        e.set_model(s.vp_true, rho)
        seis = e.forward(src, save_boundary=True)
        snap = e.export_snapshot()
        g, fw, bk = e.backward(adj)
        e.check()
    np.testing.assert_array_equal(seis, ref["seis"])
    for k in ("boundary", "p_end", "u_end", "w_end"):
        np.testing.assert_array_equal(snap[k], ref[k], err_msg=k)
    np.testing.assert_array_equal(g, gref["g"])
    np.testing.assert_array_equal(fw, gref["fw"])
    np.testing.assert_array_equal(bk, gref["bk"])


def test_band_wait_timeout_is_reported_and_the_context_stays_usable(base, monkeypatch):
    """The band kernels' bounded mbarrier wait made to run out: with a poll
    limit of 0 (SWIT_BAND_WAIT_POLLS) every block gives up at once, records
    SWIT_E_TIMEOUT in the engine's error word, waits with the full bound for its
    own copies in flight and leaves without updating.  check() raises and clears
    the word; nothing faults or hangs, and an engine created afterwards on the
    same context computes the oracle's seismograms."""
    s = base["s"]
    monkeypatch.setenv("SWIT_BAND_WAIT_POLLS", "0")
    with engine(s, kernel="band") as e:
        e.set_model(s.vp_true, base["rho"])
        e.forward(base["src"], save_boundary=True)
        with pytest.raises(SwitError, match="SWIT_E_TIMEOUT"):
            e.check()
        e.check()  # the word was cleared
    monkeypatch.delenv("SWIT_BAND_WAIT_POLLS")
    with engine(s, kernel="band") as e:
        e.set_model(s.vp_true, base["rho"])
        seis = e.forward(base["src"], save_boundary=True)
        e.check()
    np.testing.assert_array_equal(seis, base["ref"]["seis"])


@pytest.mark.parametrize("opts", [dict(), dict(adjoint="exact")])
def test_tier0_rectangle_without_list_gives_the_same_bits(opts, monkeypatch):
    """The vec kernels map the deep-interior tier-0 rectangle arithmetically and
    take only the rest from their task lists; an engine with the rectangle
    switched off (SWIT_VEC_RECT=0: everything from the lists) computes the same
    bits, for fd2dmpi's adjoint and the exact adjoint."""
    s = survey.small(nx=60, nz=44, npml=10, nt=180, ns=3)
    src = s.source()
    rho = s.rho(s.vp_true)
    outs = []
    for flag in ("1", "0"):
        monkeypatch.setenv("SWIT_VEC_RECT", flag)
        with Engine(**s.engine_args(), kernel="vec", **opts) as e:
            e.set_model(s.vp_true, rho)
            seis = e.forward(src, save_boundary=True)
            adj = (seis * 0.25).astype(np.float32)
            if opts.get("adjoint") == "exact":
                g = e.backward_exact(adj)[0]
            else:
                g = e.backward(adj)[0]
        outs.append((seis, g))
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])
