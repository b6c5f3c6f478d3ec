"""Launch-configuration autotuner.

Times a short Waveform-gradient run (the full geometry and shot count, a few
dozen time steps) for each candidate (kernel variant, columns per CTA, shots
per launch, concurrent graph branches) and returns the fastest.  Every candidate computes bit-identical
results, so the choice only affects speed.  Results are cached per process
by problem shape.
"""
import time

import numpy as np

from ._lib import SwitError
from .engine import Engine

_cache = {}


FUSED = False  # the fused kernels are slower on GB300 at every measured shape


def candidates(ns, nz_pml):
    """Launch configurations to time for ns shots (nz_pml: padded rows, for the fused kernels' limit)."""
    out = []
    batches = sorted({ns, max(1, (ns + 1) // 2), max(1, (ns + 3) // 4)}, reverse=True)
    if FUSED and nz_pml <= 1024:
        for tx in (8, 16, 32):
            for b in batches:
                out.append(dict(kernel="fused", block_x=tx, shots_per_batch=b))
    # vec: the engine's automatic choice (L2-sized batches on three branches), then
    # 1..8 batches on 1..4 concurrent graph branches (no more branches than batches)
    out.append(dict(kernel="vec", block_x=4, shots_per_batch=0, graph_branches=0))
    vb = sorted({-(-ns // k) for k in range(1, 9)}, reverse=True)
    for br in (1, 2, 3, 4):
        for b in vb:
            if br == 1 or br <= -(-ns // b):
                out.append(dict(kernel="vec", block_x=4, shots_per_batch=b, graph_branches=br))
    out.append(dict(kernel="split", block_x=4, shots_per_batch=ns))
    out.append(dict(kernel="cluster", block_x=8, shots_per_batch=ns))
    out.append(dict(kernel="hybrid", block_x=8, shots_per_batch=max(1, (ns + 1) // 2)))
    return out


def tune(nx, nz, npml, dx, dt, src_xz, rec_xz, vp, rho, free_surface=1, trial_steps=48, repeats=2,
         cands=None, verbose=False, adjoint="fd2dmpi"):
    """Returns (best options, [(options, seconds per trial gradient), ...])."""
    import torch
    src_xz = np.asarray(src_xz, np.float32)
    rec_xz = np.asarray(rec_xz, np.float32)
    ns = src_xz.shape[0]
    key = (nx, nz, npml, ns, rec_xz.shape[-2], trial_steps, free_surface, adjoint)
    if key in _cache and cands is None:
        return _cache[key]
    cands = cands or candidates(ns, nz + 2 * npml)
    if adjoint == "exact":  # the exact adjoint runs on the vec kernels
        cands = [c for c in cands if c["kernel"] == "vec"]
    nt = trial_steps
    rng = np.random.default_rng(0)
    src = torch.from_numpy(rng.standard_normal((ns, nt)).astype(np.float32)).cuda()
    times = []
    for c in cands:
        try:
            eng = Engine(nx, nz, npml, nt, dx, dt, src_xz, rec_xz, free_surface=free_surface, adjoint=adjoint, **c)
        except SwitError as err:  # e.g. a cluster variant whose wavefields do not fit on chip
            if verbose:
                print("autotune", c, "unavailable:", err)
            continue
        with eng as e:
            e.set_model(vp, rho)
            obs = torch.zeros((ns, e.ngmax, nt), dtype=torch.float32, device="cuda")
            e.gradient_l2(src, obs)  # graphs captured here
            torch.cuda.synchronize()
            best = float("inf")
            for _ in range(repeats):
                t0 = time.perf_counter()
                e.gradient_l2(src, obs)
                torch.cuda.synchronize()
                best = min(best, time.perf_counter() - t0)
            times.append((dict(c), best))
            if verbose:
                print("autotune", c, "%.3f ms" % (best * 1e3))
    best = min(times, key=lambda t: t[1])[0]
    _cache[key] = (best, times)
    return best, times
