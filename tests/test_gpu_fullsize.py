"""Parity at the benchmark configurations' own sizes (full grid, full nt).

Each case runs the engine's FP32 Waveform gradient through the C ABI and
compares it with
  * the FP32 oracle on the same inputs: bit-for-bit (same statements, same
    order, no FMA on either side) and within the specified bounds
    (seismograms <= 1e-5, gradient and illuminations <= 1e-4 relative L2);
  * the FP64 build of the same kernels: the error FP32 arithmetic itself adds
    over the full record, which the specification bounds by the same figures.

The shot counts are what the CPU oracle finishes in seconds on the host cores
(one shot per thread); the timed 49-shot run repeats both comparisons for all
shots (bench.py's ``parity`` key).
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from swit_gb300 import Engine, survey

pytestmark = pytest.mark.gpu

SEIS_TOL = 1e-5
GRAD_TOL = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))


def subset(s, keep):
    """The survey s with only the shots in keep (same grid, model and nt)."""
    import dataclasses
    return dataclasses.replace(s, src_xz=s.src_xz[keep].copy(), rec_xz=s.rec_xz[keep].copy())


def run_case(s):
    threads = os.cpu_count() or 1
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, free_surface=s.free_surface)
    rho = s.rho(s.vp_true)
    src = s.source()
    obs = O.forward(pb, s.vp_true, rho, src, store=False, nthreads=threads)["seis"]
    ref = O.gradient(pb, s.vp_init, rho, src, obs, return_seis=True, nthreads=threads)
    outs = {}
    for prec in ("fp32", "fp64"):
        with Engine(**s.engine_args(), precision=prec) as e:
            e.set_model(s.vp_init, rho)
            outs[prec] = e.gradient_l2(src, obs, return_seis=True)
    return ref, outs["fp32"], outs["fp64"]


def check(ref, mine, r64):
    names = (("seis", "seis", SEIS_TOL), ("grad", "g", GRAD_TOL), ("illum_fw", "fw", GRAD_TOL),
             ("illum_bk", "bk", GRAD_TOL))
    errs = {}
    for k, rk, tol in names:
        e_or = rel(mine[k], ref[rk])
        e64 = rel(mine[k], r64[k])
        errs[k] = (e_or, e64)
        assert e_or <= tol, (k, e_or)
        assert np.array_equal(np.asarray(mine[k]), ref[rk]), (k, "not bit-identical to the FP32 oracle", e_or)
        assert e64 <= tol, (k, "FP32 vs FP64 build", e64)
    print("rel L2 (vs FP32 oracle, vs FP64 build):", errs)


def test_marmousi_like_full_record_matches_oracle_and_fp64_build():
    """481x141 at 25 m, npml 40, nt 4000: 16 of the 49 shots (every third,
    spanning the whole line)."""
    s = subset(survey.config(1), np.arange(0, 48, 3))
    assert s.nt == 4000 and s.ns == 16
    check(*run_case(s))


def test_thrust_fold_full_record_matches_oracle_and_fp64_build():
    """501x171 at 20 m, npml 40, dt 1.5 ms, nt 5000 (the correlation-misfit
    configuration's grid and record): 8 of its 51 shots."""
    s = subset(survey.config(2), np.arange(0, 51, 7)[:8])
    assert s.nt == 5000 and (s.nx, s.nz) == (501, 171)
    check(*run_case(s))
