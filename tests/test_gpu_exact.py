"""GPU parity of the exact discrete adjoint (adjoint_mode = 1) against the oracle.

The engine's two gather kernels per reverse step evaluate the oracle's
expressions (oracle_exact_*) in the same order without FMA, so the FP32 vp and
source gradients are expected to equal the FP32 oracle bit for bit; the FP64
build must match the FP64 oracle to 1e-12 and satisfy the dot-product identity
for the source and a finite-difference check for vp (the damping profile,
which follows vmin, held fixed: the vmin points are left unperturbed).
Every launch configuration and checkpoint interval gives the same bits.
"""
import numpy as np
import pytest

from oracle import oracle as O
from swit_gb300 import Engine, SwitError, survey

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def engine(s, **kw):
    kw.setdefault("adjoint", "exact")
    return Engine(**s.engine_args(), **kw)


@pytest.fixture(scope="module")
def base():
    s = survey.small()
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, free_surface=s.free_surface)
    src = s.source()
    rho = s.rho(s.vp_true)
    adj = np.random.default_rng(11).standard_normal((pb.ns, pb.ngmax, s.nt)).astype(np.float32)
    ref = O.exact(pb, s.vp_true, rho, src, adj)
    return dict(s=s, pb=pb, src=src, rho=rho, adj=adj, ref=ref)


def run(base, **kw):
    s = base["s"]
    with engine(s, **kw) as e:
        e.set_model(s.vp_true, base["rho"])
        seis = e.forward(base["src"], save_boundary=True)
        g, gs = e.backward_exact(base["adj"])
        g2, gs2 = e.backward_exact(base["adj"])
    np.testing.assert_array_equal(g2, g)
    np.testing.assert_array_equal(gs2, gs)
    return seis, g, gs


def test_exact_adjoint_matches_oracle_bit_for_bit(base):
    seis, g, gs = run(base)
    ref = base["ref"]
    np.testing.assert_array_equal(seis, ref["seis"])
    assert rel(g, ref["g"]) <= 1e-4 and rel(gs, ref["gsrc"]) <= 1e-4
    np.testing.assert_array_equal(g, ref["g"])
    np.testing.assert_array_equal(gs, ref["gsrc"])


@pytest.mark.parametrize("opts", [dict(shots_per_batch=1), dict(shots_per_batch=2), dict(path="plain"),
                                  dict(shots_per_batch=1, graph_branches=3), dict(block_x=2),
                                  dict(checkpoint_every=1), dict(checkpoint_every=7), dict(checkpoint_every=64),
                                  dict(checkpoint_every=299), dict(checkpoint_every=300),
                                  dict(checkpoint_every=1000), dict(checkpoint_every=13, shots_per_batch=1,
                                                                    graph_branches=2),
                                  dict(checkpoint_every=13, path="plain")])
def test_exact_adjoint_is_the_same_for_every_launch_configuration(base, opts):
    _, g, gs = run(base, **opts)
    np.testing.assert_array_equal(g, base["ref"]["g"])
    np.testing.assert_array_equal(gs, base["ref"]["gsrc"])


@pytest.mark.parametrize("fs", [1, 0])
def test_fp64_exact_adjoint_matches_fp64_oracle(base, fs):
    s = base["s"]
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, free_surface=fs)
    ref = O.exact(pb, s.vp_true, base["rho"], base["src"], base["adj"], fp64=True)
    args = dict(s.engine_args(), free_surface=fs)
    with Engine(**args, precision="fp64", adjoint="exact") as e:
        e.set_model(s.vp_true, base["rho"])
        seis = e.forward(base["src"], save_boundary=True)
        g, gs = e.backward_exact(base["adj"])
    assert g.dtype == np.float64
    assert rel(seis, ref["seis"]) <= 1e-12
    assert rel(g, ref["g"]) <= 1e-12 and rel(gs, ref["gsrc"]) <= 1e-12


def test_fp64_dot_product_and_finite_differences(base):
    """<F s, r> = <s, F^T r> for the source; d<seis(vp), r>/dvp . d against
    central differences for a perturbation d that leaves vmin unchanged."""
    s, r = base["s"], base["adj"].astype(np.float64)
    vp = s.vp_true.astype(np.float32)
    rho = base["rho"]
    with Engine(**s.engine_args(), precision="fp64", adjoint="exact") as e:
        e.set_model(vp, rho)
        seis = e.forward(base["src"], save_boundary=True)
        g, gs = e.backward_exact(base["adj"])
        a, b = np.sum(seis * r), np.sum(base["src"].astype(np.float64) * gs)
        assert abs(a - b) <= 1e-10 * abs(a)
        d = 0.5 * np.random.default_rng(4).standard_normal(vp.shape)  # the FP32 rounding of vp +- d is kept exactly
        vmin = vp[:, 1:].min()  # over interior rows 2..nz (math.f90:342-361)
        d[:, 1:][vp[:, 1:] < vmin + 50.0] = 0.0
        J = []
        for sgn in (1, -1):
            e.set_model((vp.astype(np.float64) + sgn * d).astype(np.float32), rho)
            J.append(np.sum(e.forward(base["src"], save_boundary=False) * r))
        dp = (vp.astype(np.float64) + d).astype(np.float32).astype(np.float64) - vp
        dm = vp - (vp.astype(np.float64) - d).astype(np.float32).astype(np.float64)
    fd = (J[0] - J[1])
    an = np.sum(g * (dp + dm))
    assert abs(fd - an) <= 5e-5 * abs(an)  # third-order truncation: 2.6e-4 measured with |d| 8x larger


def test_gradient_l2_in_exact_mode(base):
    """Forward, residual syn - obs and exact adjoint in one call: the same
    gradient as backward_exact of that residual, the same misfit as fd2dmpi's
    mode."""
    s = base["s"]
    obs = O.forward(base["pb"], s.vp_init, base["rho"], base["src"], store=False)["seis"]
    with engine(s) as e:
        e.set_model(s.vp_true, base["rho"])
        out = e.gradient_l2(base["src"], obs, return_seis=True)
        assert out["illum_fw"] is None and out["illum_bk"] is None
        g, gs = e.backward_exact((out["seis"] - obs).astype(np.float32))
    np.testing.assert_array_equal(out["grad"], g)
    with Engine(**s.engine_args()) as e:
        e.set_model(s.vp_true, base["rho"])
        assert e.gradient_l2(base["src"], obs)["misfit"] == out["misfit"]


def test_exact_and_fd2dmpi_calls_refuse_the_other_mode(base):
    s = base["s"]
    with engine(s) as e:
        e.set_model(s.vp_true, base["rho"])
        with pytest.raises(SwitError, match="SWIT_E_STATE"):
            e.backward_exact(base["adj"])  # no storing forward yet
        e.forward(base["src"], save_boundary=True)
        with pytest.raises(SwitError, match="SWIT_E_STATE"):
            e.backward(base["adj"])
        with pytest.raises(SwitError, match="SWIT_E_STATE"):
            e.export_snapshot()
        with pytest.raises(SwitError, match="SWIT_E_STATE"):
            e.profile_kernels()
    with Engine(**s.engine_args()) as e:
        e.set_model(s.vp_true, base["rho"])
        e.forward(base["src"], save_boundary=True)
        with pytest.raises(SwitError, match="SWIT_E_STATE"):
            e.backward_exact(base["adj"])


def test_autograd_uses_the_exact_adjoint(base):
    import torch
    from swit_gb300.autograd import propagate
    s = base["s"]
    rho = torch.from_numpy(base["rho"]).cuda()
    with engine(s) as e:
        vp = torch.from_numpy(s.vp_true).cuda().requires_grad_(True)
        src = torch.from_numpy(base["src"]).cuda().requires_grad_(True)
        r = torch.from_numpy(base["adj"]).cuda()
        (propagate(e, vp, rho, src) * r).sum().backward()
    np.testing.assert_array_equal(vp.grad.cpu().numpy(), base["ref"]["g"])
    np.testing.assert_array_equal(src.grad.cpu().numpy(), base["ref"]["gsrc"])


def test_gradcheck_with_the_fp64_exact_adjoint():
    """torch.autograd.gradcheck of seismogram samples with respect to vp at a few
    points (perturbations of 0.5 m/s: exact in the FP32 model input, away from
    vmin) and to the source samples."""
    import torch
    from swit_gb300.autograd import propagate
    s = survey.small(nx=24, nz=16, npml=6, nt=160, ns=2)
    rho = torch.from_numpy(s.rho(s.vp_true)).cuda()
    vp0 = torch.from_numpy(s.vp_true).cuda().double()
    vmin = float(vp0[:, 1:].min())
    rng = np.random.default_rng(8)
    cand = [(i, j) for i in range(2, s.nx - 2) for j in range(1, s.nz - 1) if s.vp_true[i, j] > vmin + 50]
    pts = [cand[k] for k in rng.choice(len(cand), 10, replace=False)]
    ii = torch.tensor([p[0] for p in pts], device="cuda")
    jj = torch.tensor([p[1] for p in pts], device="cuda")
    src0 = torch.from_numpy(s.source()).cuda().double()
    with Engine(**s.engine_args(), precision="fp64", adjoint="exact") as e:
        scale = float(propagate(e, vp0, rho, src0)[:, ::4, ::16].abs().max())  # outputs of order 1

        def f_vp(x):
            vp = vp0.index_put((ii, jj), vp0[ii, jj] + x)
            return propagate(e, vp, rho, src0)[:, ::4, ::16] / scale

        x = torch.zeros(len(pts), dtype=torch.float64, device="cuda", requires_grad=True)
        assert torch.autograd.gradcheck(f_vp, (x,), eps=0.5, atol=1e-7, rtol=1e-4, fast_mode=False)

        def f_src(sv):
            return propagate(e, vp0, rho, sv)[:, ::4, ::16] / scale

        sv = src0.clone().requires_grad_(True)
        assert torch.autograd.gradcheck(f_src, (sv,), eps=2.0 ** -6, atol=1e-7, rtol=1e-4, fast_mode=True)


def test_exact_loop_split_into_several_graphs(base, monkeypatch):
    monkeypatch.setenv("SWIT_GRAPH_NODES", "1000")
    _, g, gs = run(base, shots_per_batch=1)
    np.testing.assert_array_equal(g, base["ref"]["g"])
    np.testing.assert_array_equal(gs, base["ref"]["gsrc"])


@pytest.mark.parametrize("comp", ["vx", "vz"])
@pytest.mark.parametrize("opts", [dict(), dict(path="plain"), dict(checkpoint_every=40, shots_per_batch=1)])
def test_exact_adjoint_of_velocity_receivers_matches_oracle(base, comp, opts):
    s = base["s"]
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, free_surface=s.free_surface, comp=comp)
    ref = O.exact(pb, s.vp_true, base["rho"], base["src"], base["adj"])
    with engine(s, receiver_component=comp, **opts) as e:
        e.set_model(s.vp_true, base["rho"])
        seis = e.forward(base["src"], save_boundary=True)
        g, gs = e.backward_exact(base["adj"])
    np.testing.assert_array_equal(seis, ref["seis"])
    np.testing.assert_array_equal(g, ref["g"])
    np.testing.assert_array_equal(gs, ref["gsrc"])
