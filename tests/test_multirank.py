"""Multi-rank host logic on CPU (gloo, world size 2): the shot split of
fd2dmpi/mmi_mpi.f90:52-80 and the gradient sum of fd2dmpi/solver.f90:263-265.
Each rank computes its block's gradient with the oracle; the all-reduced sum
must equal the single-process gradient of all shots."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from swit_gb300 import shots


@pytest.mark.parametrize("ns,world", [(49, 1), (49, 2), (49, 4), (49, 16), (5, 8), (10, 3)])
def test_assigned_blocks_cover_every_shot_once(ns, world):
    seen = []
    for r in range(world):
        b, e = shots.assigned(ns, r, world)
        seen.extend(range(b, e))
    assert sorted(seen) == list(range(ns))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    from swit_gb300 import survey
    s = survey.small(nx=32, nz=24, npml=8, nt=150, ns=5)
    rho = s.rho(s.vp_true)
    src = s.source()
    b, e = shots.assigned(s.ns, rank, world)
    pb_all = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz)
    obs = O.forward(pb_all, s.vp_init, rho, src, store=False, nthreads=1)["seis"]
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz[b:e], s.rec_xz[b:e])
    r = O.gradient(pb, s.vp_true, rho, src[b:e], obs[b:e], nthreads=1)
    # the oracle applies -2/c per block; the sum of blocks is the sum of shots
    ts = [torch.from_numpy(r[k].copy()) for k in ("g", "fw", "bk")]
    shots.allreduce_sum(ts)
    if rank == 0:
        full = O.gradient(pb_all, s.vp_true, rho, src, obs, nthreads=1)
        errs = [float(np.linalg.norm(t.numpy() - full[k]) / np.linalg.norm(full[k]))
                for t, k in zip(ts, ("g", "fw", "bk"))]
        out.put(errs)
    dist.destroy_process_group()


def test_two_gloo_ranks_sum_to_the_single_process_gradient():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    errs = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert max(errs) < 1e-6, errs
