"""swit_forward_shot_static: forward modeling of one shot with no device
allocation, for callers that cannot call cudaMalloc (a framework or plugin host
that owns all device memory through its own pool, or a loop that cannot afford
the device-wide synchronisation cudaMalloc and cudaFree imply).

The GPU test calls it through the C ABI and checks its seismograms against the
batched entry point swit_forward on the same shots, with the seismogram
tolerance of the parity tests (1e-5 relative L2), on consecutive calls -- the
calls share one static scratch array, so the second call must not see the
first call's wavefields.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from swit_gb300 import Engine, _lib, survey

SEIS_TOL = 1e-5


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_static_entry_rejects_problems_beyond_its_capacity():
    lib = _lib.load()
    rx = np.zeros(4, np.float32)
    # 5000 columns exceed SWIT_STATIC_MAX_COLUMNS; the device arguments are never touched
    rc = lib.swit_forward_shot_static(5000, 100, 40, 10, 10.0, 0.001, 1, 0.0, 0.0, 4, rx.ctypes.data,
                                      rx.ctypes.data, 1, 1, 1, 1, None)
    assert rc == -8
    assert "at most" in lib.swit_last_error().decode()
    rc = lib.swit_forward_shot_static(100, 100, 40, 10, 10.0, 0.001, 1, 0.0, 0.0, 5000, rx.ctypes.data,
                                      rx.ctypes.data, 1, 1, 1, 1, None)
    assert rc == -8


def _static_call(lib, s, shot, vp_d, rho_d, src, free_surface, seis_d):
    import torch
    src_d = torch.from_numpy(np.ascontiguousarray(src[shot])).cuda()
    rx = np.ascontiguousarray(s.rec_xz[shot, :, 0])
    rz = np.ascontiguousarray(s.rec_xz[shot, :, 1])
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.swit_forward_shot_static(s.nx, s.nz, s.npml, s.nt, float(np.float32(s.dx)), float(np.float32(s.dt)),
                                      free_surface, float(s.src_xz[shot, 0]), float(s.src_xz[shot, 1]), s.ng,
                                      rx.ctypes.data, rz.ctypes.data, vp_d.data_ptr(), rho_d.data_ptr(),
                                      src_d.data_ptr(), seis_d.data_ptr(), stream)
    assert rc == 0, lib.swit_last_error().decode()
    torch.cuda.synchronize()
    return seis_d.cpu().numpy()


@pytest.mark.gpu
def test_static_entry_matches_swit_forward_on_consecutive_calls():
    """Three calls on the benchmark grid (free surface on, 481 receivers), then
    two on a smaller grid with the free surface off and 37 receivers, then the
    benchmark grid again: each call's seismogram equals swit_forward's bit for
    bit (both run the same update expressions in the same order; SEIS_TOL is
    the bound the parity tests would accept), so no call sees the previous
    call's grid layout, receiver table or wavefields."""
    import torch
    lib = _lib.load()
    big = survey.config(1, ns=2, nt=600)  # 561 x 224 padded points fit the scratch
    small = survey.small(nx=90, nz=47, npml=12, nt=500, ns=2, ng=37)
    small.free_surface = 0
    cases = []
    for s in (big, small):
        rho = s.rho(s.vp_true)
        src = s.source()
        with Engine(**s.engine_args()) as e:
            e.set_model(s.vp_true, rho)
            ref = e.forward(src, save_boundary=False)
        cases.append((s, torch.from_numpy(s.vp_true).cuda(), torch.from_numpy(rho).cuda(), src, ref))
    for ci, shot in ((0, 0), (0, 1), (0, 0), (1, 1), (1, 0), (0, 1)):
        s, vp_d, rho_d, src, ref = cases[ci]
        seis_d = torch.full((s.ng, s.nt), float("nan"), dtype=torch.float32, device="cuda")
        got = _static_call(lib, s, shot, vp_d, rho_d, src, s.free_surface, seis_d)
        assert np.isfinite(got).all()
        err = _rel(got, ref[shot])
        assert err <= SEIS_TOL, (ci, shot, err)
        assert np.array_equal(got, ref[shot]), (ci, shot, err)


@pytest.mark.gpu
def test_static_entry_marks_a_bad_model_with_nan_then_recovers():
    """A model value that is not positive cannot be reported by return code
    (the model never leaves the device), so the whole seismogram is NaN; the
    next call with a good model is unaffected."""
    import torch
    lib = _lib.load()
    s = survey.small(nx=60, nz=40, npml=10, nt=200, ns=1, ng=20)
    rho = s.rho(s.vp_true)
    src = s.source()
    bad = s.vp_true.copy()
    bad[7, 9] = 0.0
    seis_d = torch.zeros((s.ng, s.nt), dtype=torch.float32, device="cuda")
    got = _static_call(lib, s, 0, torch.from_numpy(bad).cuda(), torch.from_numpy(rho).cuda(), src, 1, seis_d)
    assert np.isnan(got).all()
    with Engine(**s.engine_args()) as e:
        e.set_model(s.vp_true, rho)
        ref = e.forward(src, save_boundary=False)
    got = _static_call(lib, s, 0, torch.from_numpy(s.vp_true).cuda(), torch.from_numpy(rho).cuda(), src, 1,
                       seis_d)
    assert np.array_equal(got, ref[0])
