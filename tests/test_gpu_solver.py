"""GPU tests of the drop-in toolbox/solver.py replacement and the autograd path."""
import os
import types

import numpy as np
import pytest
import torch

from oracle import oracle as O
from swit_gb300 import Engine, misfit, solver, suio, survey
from swit_gb300.autograd import propagate

pytestmark = pytest.mark.gpu


def _simu(tmp_path, s, vp):
    """A toolbox `simulate` object with the fields toolbox/solver.py reads."""
    home = str(tmp_path) + "/"
    for d in ("data/obs", "data/syn", "parfile/forward_parfile", "parfile/forward_source",
              "parfile/adjoint_parfile", "parfile/adjoint_source", "parfile/model"):
        os.makedirs(home + d, exist_ok=True)
    wav = np.repeat(survey.ricker(s.nt, s.dt, s.f0)[None], s.ns, axis=0)
    model = types.SimpleNamespace(nx=s.nx, nz=s.nz, dx=s.dx, dt=s.dt, nt=s.nt, pml=s.npml, fs=True,
                                  vp=vp.astype(np.float64), rho=s.rho(vp).astype(np.float64), savestep=1)
    return types.SimpleNamespace(
        model=model, source=types.SimpleNamespace(n=s.ns, xz=s.src_xz.astype(np.float64), wavelet=wav, f0=s.f0),
        receiver=types.SimpleNamespace(n=s.ng, xz=s.rec_xz.astype(np.float64)),
        system=types.SimpleNamespace(homepath=home, mpiproc=4))


def test_dropin_forward_and_adjoint_files_match_oracle(tmp_path):
    s = survey.small(nt=250)
    simu = _simu(tmp_path, s, s.vp_true)
    solver.forward(simu, "obs", savesnap=0)
    simu.model.vp = s.vp_init.astype(np.float64)
    simu.model.rho = s.rho(s.vp_init).astype(np.float64)
    solver.forward(simu, "syn", savesnap=1)
    home = simu.system.homepath
    # oracle with the values fd2dmpi parses from the files
    src = np.fromfile(home + "parfile/forward_source/src1.bin", np.float32)
    srcs = np.stack([np.fromfile(home + "parfile/forward_source/src%d.bin" % (i + 1), np.float32)
                     for i in range(s.ns)])
    assert src.shape == (s.nt,)
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, suio.parfile_value("%f", s.dx), suio.parfile_value("%f", s.dt),
                   s.src_xz, s.rec_xz)
    rho = s.rho(s.vp_init)
    ref = O.forward(pb, s.vp_init, rho, srcs, store=True)
    for i in range(s.ns):
        h, d = suio.read_su(home + "data/syn/src%d_sg.su" % (i + 1))
        np.testing.assert_array_equal(d, ref["seis"][i])
        assert h["dt"][0] == 1000 and h["ns"][0] == s.nt

    def adjoint_source(simu_, misfit_type):
        obs = np.stack([suio.read_su(home + "data/obs/src%d_sg.su" % (i + 1))[1] for i in range(s.ns)])
        syn = np.stack([suio.read_su(home + "data/syn/src%d_sg.su" % (i + 1))[1] for i in range(s.ns)])
        return (syn - obs).astype(np.float64)

    seen = {}

    def grad_precond(simu_, optim_, grad, forw, back):
        seen.update(grad=grad, forw=forw, back=back)
        return grad

    optim = types.SimpleNamespace(misfit_type="Waveform")
    g = solver.adjoint(simu, optim, adjoint_source=adjoint_source, grad_precond=grad_precond)
    adj = adjoint_source(simu, "Waveform").astype(np.float32)
    gref = O.adjoint(pb, s.vp_init, rho, srcs, adj, ref)
    np.testing.assert_array_equal(g.reshape(s.nx, s.nz), gref["g"])
    np.testing.assert_array_equal(seen["forw"].reshape(s.nx, s.nz), gref["fw"])
    np.testing.assert_array_equal(np.fromfile(home + "data/syn/src0_illum_back.bin", np.float32).reshape(s.nx, s.nz),
                                  gref["bk"])


def test_dropin_adjoint_recomputes_strips_when_no_forward_kept(tmp_path):
    s = survey.small(nt=200)
    simu = _simu(tmp_path, s, s.vp_true)
    solver.forward(simu, "syn", savesnap=0)  # no strips kept
    optim = types.SimpleNamespace(misfit_type="Waveform")
    adj = np.ones((s.ns, s.ng, s.nt))
    g1 = solver.adjoint(simu, optim, adjoint_source=lambda a, b: adj, grad_precond=lambda a, b, g, f, k: g)
    solver.forward(simu, "syn", savesnap=1)
    g2 = solver.adjoint(simu, optim, adjoint_source=lambda a, b: adj, grad_precond=lambda a, b, g, f, k: g)
    np.testing.assert_array_equal(g1, g2)


def test_autograd_gradient_is_engine_gradient_over_dt():
    s = survey.small(nt=250)
    rho = torch.from_numpy(s.rho(s.vp_true)).cuda()
    src = torch.from_numpy(s.source()).cuda()
    with Engine(**s.engine_args()) as e:
        e.set_model(torch.from_numpy(s.vp_init).cuda(), rho)
        obs = e.forward(src, save_boundary=False).clone()
        vp = torch.from_numpy(s.vp_true).cuda().requires_grad_(True)
        seis = propagate(e, vp, rho, src)
        loss = misfit.waveform(seis, obs, s.dt)
        loss.backward()
        e.set_model(vp.detach(), rho)
        e.forward(src, save_boundary=True)
        g, _, _ = e.backward((seis.detach() - obs).contiguous())
    torch.testing.assert_close(vp.grad, g / s.dt, rtol=0, atol=0)


def test_autograd_recomputes_after_an_intervening_forward():
    s = survey.small(nt=200)
    rho = torch.from_numpy(s.rho(s.vp_true)).cuda()
    src = torch.from_numpy(s.source()).cuda()
    with Engine(**s.engine_args()) as e:
        v1 = torch.from_numpy(s.vp_true).cuda().requires_grad_(True)
        v2 = torch.from_numpy(s.vp_init).cuda().requires_grad_(True)
        y1 = propagate(e, v1, rho, src)
        y2 = propagate(e, v2, rho, src)   # overwrites the strips of y1
        (y1.square().sum() + y2.square().sum()).backward()
        g1 = v1.grad.clone()
        v1.grad = None
        propagate(e, v1, rho, src).square().sum().backward()
    torch.testing.assert_close(g1, v1.grad, rtol=0, atol=0)


def test_autograd_against_central_finite_differences():
    """Central differences of 1/2 ||seis - obs||^2 with the FP64 build; the
    reference's imaging gradient agrees in direction, not pointwise."""
    s = survey.small(nx=40, nz=30, npml=10, nt=400, ns=2, zs=60.0)
    vp0 = s.vp_true.astype(np.float64)
    rho = s.rho(vp0)
    src = s.source()
    with Engine(**s.engine_args(), precision="fp64") as e:
        e.set_model((vp0 * 0.97).astype(np.float32), rho)
        obs = e.forward(src, save_boundary=False)

        def L(v):
            e.set_model(v.astype(np.float32), rho)
            d = e.forward(src, save_boundary=False)
            return 0.5 * np.sum((d - obs) ** 2)
        e.set_model(vp0.astype(np.float32), rho)
        d0 = e.forward(src, save_boundary=True)
        g, _, _ = e.backward((d0 - obs).astype(np.float32))
        g = g / s.dt
        rng = np.random.default_rng(5)
        fd, gg = [], []
        for _ in range(20):
            i, j = rng.integers(12, s.nx - 12), rng.integers(4, s.nz - 4)
            h = 1e-3 * vp0[i, j]
            vpp, vpm = vp0.copy(), vp0.copy()
            vpp[i, j] += h
            vpm[i, j] -= h
            hh = float(np.float32(vpp[i, j]) - np.float32(vpm[i, j]))
            fd.append((L(vpp) - L(vpm)) / hh)
            gg.append(g[i, j])
    fd, gg = np.array(fd), np.array(gg)
    cos = fd @ gg / np.linalg.norm(fd) / np.linalg.norm(gg)
    scale = (fd @ gg) / (gg @ gg)
    print("autograd vs central FD: cosine %.4f, least-squares scale %.4f" % (cos, scale))
    assert cos > 0.95 and 0.7 < scale < 1.4


def _uneven_problems():
    """Three independent problems of different grids, spacings, shots and record lengths."""
    from swit_gb300 import survey
    out = []
    for (nx, nz, npml, nt, dx, ns, seed) in ((52, 30, 10, 260, 10.0, 3, 3), (40, 36, 8, 180, 12.0, 2, 4),
                                              (64, 24, 9, 320, 10.0, 4, 5)):
        s = survey.small(nx=nx, nz=nz, npml=npml, nt=nt, dx=dx, ns=ns, seed=seed)
        out.append(s)
    return out


@pytest.mark.parametrize("wave_bytes,graph_nodes", [(None, None), ("1", None), ("5e5", None), ("1", "0"),
                                                     ("5e5", "0"), ("1", "700")])
def test_multi_engine_matches_each_engine_bit_for_bit(wave_bytes, graph_nodes, monkeypatch):
    """All problems stepped by shared launches give each problem's own engine's
    seismogram misfit, gradient and illuminations exactly, twice in a row.
    Wave layouts: the three small problems in one shared wave (default); one
    (problem, shot) pair per wave (wave budget 1 byte); a wave of one problem
    beside a wave shared by two (5e5 bytes); and waves launched step by step
    instead of as graphs (all of them, or those beyond a small graph node
    budget)."""
    import torch
    from swit_gb300 import MultiEngine
    if wave_bytes:
        monkeypatch.setenv("SWIT_MULTI_WAVE_BYTES", wave_bytes)
    if graph_nodes:
        monkeypatch.setenv("SWIT_MULTI_GRAPH_NODES", graph_nodes)
    surveys = _uneven_problems()
    ref = []
    for s in surveys:
        rho = s.rho(s.vp_true)
        with Engine(**s.engine_args()) as e:
            e.set_model(s.vp_true, rho)
            obs = e.forward(s.source(), save_boundary=False)
            e.set_model(s.vp_init, rho)
            ref.append((obs, e.gradient_l2(s.source(), obs)))
    with MultiEngine([s.engine_args() for s in surveys]) as me:
        for e, s in zip(me.engines, surveys):
            e.set_model(s.vp_init, s.rho(s.vp_true))
        srcs = [s.source() for s in surveys]
        obss = [r[0] for r in ref]
        for _ in range(2):
            outs = me.gradient_l2(srcs, obss)
            for o, (_, r) in zip(outs, ref):
                for k in ("grad", "illum_fw", "illum_bk"):
                    np.testing.assert_array_equal(o[k], r[k])
                assert o["misfit"] == r["misfit"]
        mis = me.misfit_l2(srcs, obss)
        assert mis == [r[1]["misfit"] for r in ref]
        mis = me.misfit_l2(srcs, obss, active=[False, True, False])
        assert mis == [0.0, ref[1][1]["misfit"], 0.0]
        outs = me.gradient_l2(srcs, obss)  # every instance again after a partial call
        for o, (_, r) in zip(outs, ref):
            np.testing.assert_array_equal(o["grad"], r["grad"])
        # device inputs
        outs = me.gradient_l2([torch.from_numpy(x).cuda() for x in srcs], [torch.from_numpy(x).cuda() for x in obss])
        torch.cuda.synchronize()
        for o, (_, r) in zip(outs, ref):
            np.testing.assert_array_equal(o["grad"].cpu().numpy(), r["grad"])


def test_misfit_only_call_matches_the_gradient_call():
    s = survey.small()
    rho = s.rho(s.vp_true)
    with Engine(**s.engine_args()) as e:
        e.set_model(s.vp_true, rho)
        obs = e.forward(s.source(), save_boundary=False)
        e.set_model(s.vp_init, rho)
        m = e.misfit_l2(s.source(), obs)
        r = e.gradient_l2(s.source(), obs)
    assert m == r["misfit"] and m > 0
