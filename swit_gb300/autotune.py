"""Launch-configuration autotuner.

Times a short Waveform-gradient run (the full geometry and shot count, a few
dozen time steps) for each candidate (shots per launch, concurrent graph
branches of the vec kernels) and returns the fastest.  Every candidate computes bit-identical
results, so the choice only affects speed.  Results are cached per process
by problem shape.
"""
import time

import numpy as np

from ._lib import SwitError
from .engine import Engine

_cache = {}


def candidates(ns):
    """Launch configurations to time for ns shots: the vec kernels with the
    engine's automatic choice (L2-sized batches on three branches), then 1..8
    batches on 1..4 concurrent graph branches (no more branches than batches).
    The other variants compute the same bits but measured slower at every shape
    timed on GB300 (481x141, 49 shots: split 40.8, walk 70.8, cluster 77.7,
    hybrid 88.3, band 52.2 shot-gradients/s against 125-128 for vec), so they
    are not timed; name one in Engine(kernel=...) to use it."""
    out = [dict(kernel="vec", block_x=4, shots_per_batch=0, graph_branches=0)]
    vb = sorted({-(-ns // k) for k in range(1, 9)}, reverse=True)
    for br in (1, 2, 3, 4):
        for b in vb:
            if br == 1 or br <= -(-ns // b):
                out.append(dict(kernel="vec", block_x=4, shots_per_batch=b, graph_branches=br))
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
    cands = cands or candidates(ns)
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
