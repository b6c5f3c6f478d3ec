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


@pytest.mark.gpu
def test_static_entry_matches_swit_forward_on_consecutive_calls():
    import torch
    lib = _lib.load()
    s = survey.config(1, ns=2, nt=600)  # the benchmark grid: 561 x 224 padded points fit the scratch
    rho = s.rho(s.vp_true)
    src = s.source()
    with Engine(**s.engine_args()) as e:
        e.set_model(s.vp_true, rho)
        ref = e.forward(src, save_boundary=False)
    vp_d = torch.from_numpy(s.vp_true).cuda()
    rho_d = torch.from_numpy(rho).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    for shot in (0, 1, 0):
        src_d = torch.from_numpy(np.ascontiguousarray(src[shot])).cuda()
        seis_d = torch.full((s.ng, s.nt), float("nan"), dtype=torch.float32, device="cuda")
        rx = np.ascontiguousarray(s.rec_xz[shot, :, 0])
        rz = np.ascontiguousarray(s.rec_xz[shot, :, 1])
        rc = lib.swit_forward_shot_static(s.nx, s.nz, s.npml, s.nt, float(np.float32(s.dx)),
                                          float(np.float32(s.dt)), 1, float(s.src_xz[shot, 0]),
                                          float(s.src_xz[shot, 1]), s.ng, rx.ctypes.data, rz.ctypes.data,
                                          vp_d.data_ptr(), rho_d.data_ptr(), src_d.data_ptr(), seis_d.data_ptr(),
                                          stream)
        assert rc == 0, lib.swit_last_error().decode()
        torch.cuda.synchronize()
        got = seis_d.cpu().numpy()
        assert np.isfinite(got).all()
        err = _rel(got, ref[shot])
        assert err <= SEIS_TOL, (shot, err)
