"""The differentiable path with correlation misfits on the thrust-fold model of
the 501x171 configuration, at a reduced size (121x51, nt 1500, 4 shots).

Seismograms come from autograd.propagate, the misfits from swit_gb300.misfit
(the reference's global-correlation and traveltime adjoint sources), and the
vp gradient from loss.backward() through the engine.  Checks:
* central finite differences at 20 random grid points, h = 1e-3 vp, with the
  FP64 build: the exact adjoint for a normalised-correlation misfit written in
  torch, and the reference's global-correlation misfit, whose adjoint source
  (misfit.py:219-242) leaves out the mean removal of its value (338-355), so it
  is checked in direction only, as is fd2dmpi's continuous-adjoint gradient;
* the FP32 exact gradient against the FP64 exact gradient, and the FP64 engine
  against the FP64 oracle with the same adjoint source;
* the traveltime misfit is piecewise constant in vp (integer cross-correlation
  lags), so it enters only through its adjoint source (golden-tested in
  test_misfit.py) and the FP32/FP64 comparison.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from swit_gb300 import Engine, misfit, survey
from swit_gb300.autograd import propagate

pytestmark = pytest.mark.gpu


def make():
    nx, nz, dx = 121, 51, 20.0
    vp = survey.thrust_fold(nx, nz, dx, seed=1002)
    src, rec = survey._line_geometry(nx, dx, 4, 20.0, 20.0)
    return survey.Survey(name="thrust-fold 121x51", nx=nx, nz=nz, dx=dx, dt=0.0015, nt=1500, npml=20, f0=5.0,
                         vp_true=vp, vp_init=survey.smooth(vp, 250.0, dx), src_xz=src, rec_xz=rec)


def cos_loss(seis, obs):
    """-sum over traces of the normalised correlation, differentiated by torch."""
    s = seis / torch.linalg.vector_norm(seis, dim=-1, keepdim=True).clamp_min(1e-300)
    o = obs / torch.linalg.vector_norm(obs, dim=-1, keepdim=True).clamp_min(1e-300)
    return -(s * o).sum()


def cosine(a, b):
    return float(a @ b / np.linalg.norm(a) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def setup():
    s = make()
    rho = torch.from_numpy(s.rho(s.vp_true)).cuda()
    src = torch.from_numpy(s.source()).cuda()
    with Engine(**s.engine_args(), precision="fp64") as e:
        e.set_model(torch.from_numpy(s.vp_true).cuda(), rho)
        obs = e.forward(src, save_boundary=False).clone()
    vp = s.vp_init.astype(np.float32)
    vmin = vp[:, 1:].min()
    rng = np.random.default_rng(20)
    cand = [(i, j) for i in range(3, s.nx - 3) for j in range(2, s.nz - 2) if vp[i, j] > vmin + 50]
    pts = [cand[k] for k in rng.choice(len(cand), 20, replace=False)]
    return dict(s=s, rho=rho, src=src, obs=obs, vp=vp, pts=pts)


def grad_and_fd(st, loss_fn, adjoint):
    s, rho, src, obs, vp = st["s"], st["rho"], st["src"], st["obs"], st["vp"]
    with Engine(**s.engine_args(), precision="fp64", adjoint=adjoint) as e:
        v = torch.from_numpy(vp).cuda().double().requires_grad_(True)
        loss_fn(propagate(e, v, rho, src), obs).backward()
        g = v.grad.cpu().numpy()
        fd, an = [], []
        for (i, j) in st["pts"]:
            h = 1e-3 * float(vp[i, j])
            vals = []
            for sgn in (1, -1):
                w = vp.copy()
                w[i, j] = np.float32(float(vp[i, j]) + sgn * h)
                e.set_model(torch.from_numpy(w).cuda(), rho)
                vals.append(float(loss_fn(e.forward(src, save_boundary=False), obs)))
            hh = float(np.float32(float(vp[i, j]) + h)) - float(np.float32(float(vp[i, j]) - h))
            fd.append((vals[0] - vals[1]) / hh)
            an.append(g[i, j])
    return np.array(fd), np.array(an)


def test_exact_gradient_matches_finite_differences(setup):
    fd, an = grad_and_fd(setup, cos_loss, "exact")
    err = np.linalg.norm(fd - an) / np.linalg.norm(fd)
    print("exact adjoint vs central FD (20 points, h = 1e-3 vp): rel. L2 %.2e" % err)
    assert err <= 2e-3


def test_reference_misfit_gradients_against_finite_differences(setup):
    def gc(seis, obs):
        return misfit.global_correlation(seis, obs, setup["s"].dt)

    fd, an = grad_and_fd(setup, gc, "exact")
    c_exact = cosine(fd, an)
    fd2, an2 = grad_and_fd(setup, gc, "fd2dmpi")
    c_ref = cosine(fd2, an2)
    print("global correlation vs central FD: exact adjoint cosine %.4f, fd2dmpi adjoint cosine %.4f"
          % (c_exact, c_ref))
    assert c_exact >= 0.99 and c_ref >= 0.9


def test_fp32_exact_gradient_against_fp64_and_the_oracle(setup):
    s, rho, src, obs = setup["s"], setup["rho"], setup["src"], setup["obs"]

    def loss(seis, o):
        return misfit.global_correlation(seis, o, s.dt) + misfit.traveltime(seis, o, s.dt)

    out = {}
    for prec in ("fp32", "fp64"):
        with Engine(**s.engine_args(), precision=prec, adjoint="exact") as e:
            v = torch.from_numpy(setup["vp"]).cuda().double().requires_grad_(True)  # gradient kept in FP64
            seis = propagate(e, v, rho, src)
            sd = seis.detach().clone().requires_grad_(True)
            (adj,) = torch.autograd.grad(loss(sd, obs), sd)
            loss(seis, obs).backward()
            out[prec] = (v.grad.double().cpu().numpy(), adj.float().cpu().numpy())
    g32, g64 = out["fp32"][0], out["fp64"][0]
    assert np.linalg.norm(g32 - g64) / np.linalg.norm(g64) <= 1e-4
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz)
    ref = O.exact(pb, setup["vp"], rho.cpu().numpy(), src.cpu().numpy(), out["fp64"][1], fp64=True)
    assert np.linalg.norm(g64 - ref["g"]) / np.linalg.norm(ref["g"]) <= 1e-12
