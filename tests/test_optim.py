"""The device optimiser against search directions made by the reference's own
toolbox/inversion.py (tests/golden/make_optim_golden.py), on CPU tensors and
(marked gpu) on CUDA tensors."""
import importlib.util
import os

import numpy as np
import pytest
import torch

from swit_gb300 import optim as O

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "optim_golden.npz"))
_spec = importlib.util.spec_from_file_location("_mk", os.path.join(os.path.dirname(__file__), "golden",
                                                                   "make_optim_golden.py"))
_mk = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(_mk)
DEVICES = [pytest.param("cpu", id="cpu"), pytest.param("cuda", id="cuda", marks=pytest.mark.gpu)]


@pytest.mark.parametrize("device", DEVICES)
@pytest.mark.parametrize("scheme,key", [("LBFGS", "d_lbfgs"), ("NLCG", "d_nlcg")])
def test_directions_match_reference(scheme, key, device):
    A, b, v0 = _mk.problem()
    A, b = torch.from_numpy(A).to(device), torch.from_numpy(b).to(device)
    st = O.init_state(scheme, v0.size, device=device)
    st["v_now"] = torch.from_numpy(v0.copy()).to(device)
    st["v_old"] = torch.from_numpy(v0.copy()).to(device)
    for i in range(4):
        st["g_now"] = A @ st["v_now"] - b
        st = O.nlcg_direction(st) if scheme == "NLCG" else O.lbfgs_direction(st)
        ref = G[key][i]
        assert st["d_now"].device.type == device
        np.testing.assert_allclose(st["d_now"].cpu().numpy(), ref, rtol=0, atol=2e-5 * np.abs(ref).max())
        if scheme == "NLCG":
            st["g_old"], st["d_old"] = st["g_now"], st["d_now"]
        else:
            st["g_old"], st["v_old"] = st["g_now"], st["v_now"]
        st["v_now"] = st["v_now"] + 0.5 * st["d_now"]


@pytest.mark.parametrize("device", DEVICES)
@pytest.mark.parametrize("scheme", ["LBFGS", "NLCG"])
def test_fwi_loop_decreases_a_quadratic(scheme, device):
    A, b, v0 = _mk.problem()
    A, b = torch.from_numpy(A).to(device), torch.from_numpy(b).to(device)

    def f(v):
        return 0.5 * v @ (A @ v) - b @ v

    st, hist = O.fwi(torch.from_numpy(v0).to(device), lambda v: (f(v), A @ v - b), f, scheme=scheme, maxiter=5,
                     step_length=0.5, vpmax=1e9, vpmin=-1e9)
    fs = [h["f"] for h in hist]
    assert all(h["ls_status"] == 0 for h in hist)
    assert fs == sorted(fs, reverse=True) and fs[-1] < float(f(torch.from_numpy(v0).to(device)))
    assert st["v_now"].device.type == device


def test_model_update_clips_to_bounds():
    v = torch.tensor([1000.0, 2000.0, 4900.0])
    out = O.model_update(v, torch.tensor([-500.0, 10.0, 500.0]), 5000.0, 1000.0)
    assert out.tolist() == [1000.0, 2010.0, 5000.0]


@pytest.mark.parametrize("scheme", ["LBFGS", "NLCG"])
def test_lockstep_fwi_follows_each_problem_alone(scheme):
    """Three independent quadratic problems run through fwi_lockstep take the same
    iterates, line-search steps and misfits as fwi runs each alone."""
    rng = np.random.default_rng(5)
    probs = []
    for n in (30, 45, 20):
        Q = rng.standard_normal((n, n))
        A = torch.tensor(Q @ Q.T / n + np.eye(n))
        b = torch.tensor(rng.standard_normal(n))
        v0 = torch.tensor(2000.0 + 100.0 * rng.standard_normal(n))
        probs.append((A, b, v0))

    def f_of(A, b, v):
        return float(0.5 * v @ (A @ v) - b @ v)

    def g_of(A, b, v):
        return A @ v - b

    alone = []
    for A, b, v0 in probs:
        st, h = O.fwi(v0, lambda v, A=A, b=b: (f_of(A, b, v), g_of(A, b, v)), lambda v, A=A, b=b: f_of(A, b, v),
                          scheme=scheme, maxiter=4, vpmax=5000.0, vpmin=1000.0)
        alone.append((st, h))
    sts, hists = O.fwi_lockstep(
        [p[2] for p in probs],
        lambda vs: [(f_of(A, b, v), g_of(A, b, v)) for (A, b, _), v in zip(probs, vs)],
        lambda vs, act: [f_of(A, b, v) if a else None for (A, b, _), v, a in zip(probs, vs, act)],
        scheme=scheme, maxiter=4, vpmax=5000.0, vpmin=1000.0)
    for (st, h), st2, h2 in zip(alone, sts, hists):
        assert h == h2
        assert torch.equal(st["v_now"], st2["v_now"])
