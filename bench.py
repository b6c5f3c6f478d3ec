#!/usr/bin/env python
"""FWI shot-gradient throughput of the GB300 engine (one JSON line on rank 0).

Workload: the batched Marmousi-like gradient -- 481 x 141 grid at 25 m, 40-point
PML, nt = 4000, dt = 2 ms, 49 shots at z = 25 m, 481 surface receivers, 5 Hz
Ricker -- on a seeded synthetic faulted-layer model (no public model is read).
One step = one Waveform-misfit gradient of every shot: forward with boundary
strips, adjoint source syn - obs, reconstruction + adjoint + imaging, shot sum.

  value  shot-gradients/s with inputs resident in device memory
  e2e    the same through the C ABI with host (pinned) buffers: model, sources and
         observed data copied in, gradient + illuminations + misfit copied out
         every step
Under torchrun (N > 1) every rank runs its own 49-shot block of a 49 N-shot
survey and the gradients are summed with one all-reduce (weak scaling).
``--impl reference`` times the CPU restatement of fd2dmpi (the reference's
Fortran cannot be built here) on the host cores instead.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FWI shot-gradients/s (481x141, nt=4000) batched vs plain GPU; GPts/s, % HBM roof"
UNIT = "shot-gradients/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mine", choices=["mine", "reference"])
    ap.add_argument("--shots", type=int, default=None, help="shots per rank (default 49)")
    ap.add_argument("--nt", type=int, default=None, help="time steps (default 4000)")
    ap.add_argument("--batch", type=int, default=0, help="shots per launch (0 = engine default)")
    ap.add_argument("--block-x", type=int, default=0)
    ap.add_argument("--branches", type=int, default=0, help="concurrent graph branches (0 = engine default)")
    ap.add_argument("--adjoint", default="fd2dmpi", choices=["fd2dmpi", "exact"],
                    help="fd2dmpi's adjoint (the reference's gradient) or the exact discrete adjoint")
    ap.add_argument("--kernel", default="auto", choices=["auto", "walk", "split", "vec", "cluster", "hybrid", "band"])
    ap.add_argument("--no-tune", action="store_true", help="skip the launch-configuration autotuner")
    ap.add_argument("--no-extras", action="store_true", help="skip plain path, CPU baseline and kernel profile")
    ap.add_argument("--workload", default="marmousi", choices=["marmousi", "small", "large", "multi", "correlation"],
                    help="marmousi: 481x141 nt 4000 49 shots (the headline); small: 201x101 nt 2000 5 shots; "
                         "large: 2001x601 nt 6000 200 shots; "
                         "multi: uneven independent FWI problems, L-BFGS on all at once vs one after another; "
                         "correlation: 501x171 nt 5000 51 shots, global-correlation + traveltime misfits "
                         "through torch.autograd")
    ap.add_argument("--instances", type=int, default=64, help="multi: problems")
    ap.add_argument("--iters", type=int, default=5, help="multi: L-BFGS iterations")
    ap.add_argument("--scale", type=float, default=1.0, help="multi: factor on shot counts and record lengths")
    ap.add_argument("--parity-shots", type=int, default=16,
                    help="large: shots of the full-size comparison with the FP64 build and the oracle (0: none)")
    ap.add_argument("--plain-lbfgs", action="store_true",
                    help="multi: run the plain path's L-BFGS in full (default: one plain gradient of every problem)")
    ap.add_argument("--checkpoint", default="0",
                    help="memory strategy: 0 = boundary saving, k = checkpoints every k steps, auto = the interval "
                         "that minimises memory, budget = boundary saving if the engine fits 150 GB, else the "
                         "interval that minimises memory")
    return ap.parse_args()


# --------------------------------------------------------------------- units
def work_units(nx, nz, npml, nt, ng):
    """Grid-point updates U and algorithmic bytes B per shot-gradient.

    U = (nt-1) (2 N_pml + N_int); B = (nt-1) [64 N_pml + 56 N_int + 8 S] + 8 nt ng
    with N_pml = (nx+2 npml)(nz+2 npml), N_int = nx nz, S = 9 nx + 6 nz: state
    p, u, w read and written once per step on the PML grid forward and adjoint,
    two coefficient arrays, the interior reconstruction and three imaging sums,
    strips written and read, seismograms written and adjoint sources read.
    """
    npml_pts = (nx + 2 * npml) * (nz + 2 * npml)
    nint = nx * nz
    S = 9 * nx + 6 * nz
    U = (nt - 1) * (2 * npml_pts + nint)
    B = (nt - 1) * (64 * npml_pts + 56 * nint + 8 * S) + 8 * nt * ng
    return U, B


def kernel_bytes_per_shot(nx, nz, npml, ng, nt):
    """Compulsory bytes one launch of each stencil kernel moves per shot (each
    array it touches read or written once per time step, neighbours not counted
    again).  The cluster kernels run the whole time loop in one launch."""
    npts = (nx + 2 * npml) * (nz + 2 * npml)
    nint = nx * nz
    step = {
        "fwd_p": 20 * npts,                                   # p r/w, u, w, A
        "fwd_uw": 24 * npts + 4 * (9 * nx + 6 * nz) + 4 * ng,  # u, w r/w, p, B; strips, trace samples
        "bwd_uw": 24 * npts + 24 * nint + 4 * (nx + 2 * nz),   # adjoint u, w; reconstruction u, w; strips
        "bwd_p": 20 * npts + 44 * nint + 4 * (5 * nx + 4 * nz) + 4 * ng,  # adjoint p; reco p; imaging; strips
        # walk: p, u, w, A, B read and p, u, w written once; the interior adds the
        # reconstruction state and the three imaging sums
        "fwd_step": 32 * npts + 4 * (9 * nx + 6 * nz) + 4 * ng,
        "bwd_step": 32 * npts + 48 * nint + 4 * (6 * nx + 6 * nz) + 4 * ng,
    }
    step["fwd_loop"] = (nt - 1) * (step["fwd_p"] + step["fwd_uw"])
    step["bwd_loop"] = (nt - 1) * (step["bwd_uw"] + step["bwd_p"])
    return step


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# DRAM traffic of k_bwd_p_v per shot and launch with the L2 warm: 51,527 B (the average of two steady 9-shot
# launches, 464 KB each), from
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum --clock-control none \
#       -k regex:k_bwd_p_v -s 600 -c 3 --csv \
#       python bench.py --shots 27 --nt 300 --steps 1 --warmup 1 --no-extras --no-tune --kernel vec
# (profiles/stencil_traffic.txt keeps the capture's summary).  It is a stored figure, not measured by this run.
BWD_P_TRAFFIC_PER_SHOT = 51527


def l2_bandwidth():
    """L2 read+write bandwidth (GB/s) measured now on this GPU (swit_l2_bandwidth), or None."""
    import ctypes as C

    import torch

    from swit_gb300 import _lib
    g = C.c_double(0.0)
    rc = _lib.load().swit_l2_bandwidth(64 << 20, 200, C.byref(g), torch.cuda.current_stream().cuda_stream)
    return g.value if rc == 0 else None


# --------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------- arms
def rel_l2(a, b):
    """||a - b|| / ||b|| in float64 (0 when b is all zero and a equals it)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a))


def _np(x):
    return x.detach().cpu().numpy() if hasattr(x, "detach") else np.asarray(x)


def oracle_gradient(sv, rho, src, obs, threads):
    """All shots' Waveform gradient on the CPU oracle (FP32, one shot per thread,
    fd2dmpi's static split); returns (result, wall seconds)."""
    from oracle import oracle as O
    pb = O.Problem(sv.nx, sv.nz, sv.npml, sv.nt, sv.dx, sv.dt, sv.src_xz, sv.rec_xz)
    t0 = time.perf_counter()
    ref = O.gradient(pb, sv.vp_init, rho, src, obs, return_seis=True, nthreads=threads)
    return ref, time.perf_counter() - t0


def full_size_parity(sv, rho, src_d, obs_d, mine, ref32=None):
    """Error of the timed FP32 result at the benchmark's own size: against the
    FP64 build of the same kernels (the error FP32 arithmetic adds) and, when
    given, against the FP32 oracle (bit-for-bit agreement expected: the same
    statements in the same order, no FMA)."""
    from swit_gb300 import Engine
    e64 = Engine(sv.nx, sv.nz, sv.npml, sv.nt, sv.dx, sv.dt, sv.src_xz, sv.rec_xz, free_surface=sv.free_surface,
                 precision="fp64")
    e64.set_model(sv.vp_init, rho)
    r64 = e64.gradient_l2(src_d, obs_d, return_seis=True)
    e64.close()
    m = {k: _np(mine[k]) for k in ("seis", "grad", "illum_fw", "illum_bk")}
    out = {"shots": int(sv.ns), "nt": int(sv.nt),
           "vs_fp64_build": {k + "_rel_l2": rel_l2(m[k], _np(r64[k])) for k in m},
           "tolerance": {"seis_rel_l2": 1e-5, "grad_rel_l2": 1e-4}}
    if ref32 is not None:
        names = {"seis": "seis", "grad": "g", "illum_fw": "fw", "illum_bk": "bk"}
        o = {}
        for k, rk in names.items():
            o[k + "_rel_l2"] = rel_l2(m[k], ref32[rk])
            o[k + "_bit_exact"] = bool(np.array_equal(m[k], ref32[rk]))
        out["vs_fp32_oracle"] = o
        out["oracle_vs_fp64_build"] = {k + "_rel_l2": rel_l2(ref32[rk], _np(r64[k])) for k, rk in names.items()}
    v = out["vs_fp64_build"]
    out["within_tolerance"] = bool(v["seis_rel_l2"] <= 1e-5 and v["grad_rel_l2"] <= 1e-4)
    return out


def subset_parity(sv, rho, n):
    """The full-size comparison on n of the workload's shots, evenly spread
    (full grid and nt): FP32 engine against the FP64 build and the FP32 oracle."""
    import dataclasses

    import torch

    from swit_gb300 import Engine
    keep = np.linspace(0, sv.ns - 1, min(n, sv.ns)).round().astype(int)
    sub = dataclasses.replace(sv, src_xz=sv.src_xz[keep].copy(), rec_xz=sv.rec_xz[keep].copy())
    src_d = torch.from_numpy(sub.source()).cuda()
    with Engine(**sub.engine_args()) as e:
        e.set_model(sub.vp_true, rho)
        obs_d = e.forward(src_d, save_boundary=False)
        e.set_model(sub.vp_init, rho)
        mine = e.gradient_l2(src_d, obs_d, return_seis=True)
    ref32, wall = oracle_gradient(sub, rho, sub.source(), obs_d.cpu().numpy(), os.cpu_count() or 1)
    out = full_size_parity(sub, rho, src_d, obs_d, mine, ref32)
    out["shot_indices"] = [int(k) for k in keep]
    out["oracle_wall_s"] = wall
    return out


def cpu_with_strip_io(sv, rho, src, obs, threads):
    """The same sample as cpu_baseline, but with fd2dmpi's file round trip: the
    forward job writes each shot's boundary strips and final wavefields to files
    (fdcore.f90:130-166, one file set per shot, srcN_snapshot/), the adjoint job
    reads them back (solver.f90:213-228).  Files go to a temporary directory,
    written and read by one thread per shot."""
    import shutil
    import tempfile
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O
    n = min(sv.ns, threads)
    pb = O.Problem(sv.nx, sv.nz, sv.npml, sv.nt, sv.dx, sv.dt, sv.src_xz[:n], sv.rec_xz[:n])
    keys = ("boundary", "p_end", "u_end", "w_end")
    tmp = tempfile.mkdtemp(prefix="swit_strips_")
    try:
        t0 = time.perf_counter()
        f = O.forward(pb, sv.vp_init, rho, src[:n], store=True, nthreads=threads)
        shapes = {k: f[k].shape[1:] for k in keys}

        def write(i):
            for k in keys:
                f[k][i].tofile(os.path.join(tmp, "src%d_%s.bin" % (i + 1, k)))

        def read(i):
            return [np.fromfile(os.path.join(tmp, "src%d_%s.bin" % (i + 1, k)), np.float32).reshape(shapes[k])
                    for k in keys]

        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(write, range(n)))
            for k in keys:
                del f[k]
            parts = list(ex.map(read, range(n)))
        fwd = {k: np.stack([p[j] for p in parts]) for j, k in enumerate(keys)}
        adj = (f["seis"] - obs[:n]).astype(np.float32)
        O.adjoint(pb, sv.vp_init, rho, src[:n], adj, fwd, nthreads=threads)
        wall = time.perf_counter() - t0
        nbytes = sum(os.path.getsize(os.path.join(tmp, x)) for x in os.listdir(tmp))
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return {"value": n / wall, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d of %d shots at full nt=%d with the strips and final wavefields written to and read from "
                      "files (%.2f GB), %.1f s wall" % (n, sv.ns, sv.nt, nbytes / 1e9, wall)}


def workload_config(sv, shots):
    """The workload as both arms name it (identical keys and values)."""
    strips = shots * sv.nt * (9 * sv.nx + 6 * sv.nz) * 4
    traces = 2 * shots * sv.ng * sv.nt * 4
    l2 = ("inputs larger than L2" if strips + traces > 126e6 else "inputs smaller than L2, no flush between steps")
    return {"workload": sv.name, "grid": [sv.nx, sv.nz], "npml": sv.npml, "nt": sv.nt, "shots_per_gpu": shots,
            "receivers": sv.ng, "dx_m": sv.dx, "dt_s": sv.dt,
            "l2": "%s: each step streams %.2f GB of boundary strips and %.2f GB of traces"
                  % (l2, strips / 1e9, traces / 1e9)}


def run_reference(args):
    """The reference arm: the CPU restatement of fd2dmpi (FP32, g++ -O3) on the
    host cores, one shot per thread with fd2dmpi's static shot split, every
    step the full workload (all shots, full nt) -- the same work as one step of
    the GPU arm.  Rank 0 alone runs under torchrun."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    from swit_gb300 import survey
    sv = survey.config(1, ns=args.shots, nt=args.nt)
    threads = os.cpu_count() or 1
    rho = sv.rho(sv.vp_true)
    src = sv.source()
    pb = O.Problem(sv.nx, sv.nz, sv.npml, sv.nt, sv.dx, sv.dt, sv.src_xz, sv.rec_xz)
    obs = O.forward(pb, sv.vp_true, rho, src, store=False, nthreads=threads)["seis"]
    walls = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        O.gradient(pb, sv.vp_init, rho, src, obs, nthreads=threads)
        if i >= args.warmup:
            walls.append(time.perf_counter() - t0)
    ms_per_step = 1000.0 * float(np.mean(walls))
    v = sv.ns / (ms_per_step / 1000.0)
    U, B = work_units(sv.nx, sv.nz, sv.npml, sv.nt, sv.ng)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(sv, sv.ns),
            "engine": {"path": "CPU restatement of fd2dmpi (oracle/fd2d_oracle.cpp, FP32, g++ -O3), one shot per "
                               "thread; fd2dmpi itself needs gfortran + MPI, absent"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "all %d shots per step at full nt=%d, one shot per thread" % (sv.ns, sv.nt)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpts_per_s": v * U / 1e9}
    if not args.no_extras:
        # fd2dmpi keeps the strips on disk between its forward and adjoint jobs: one timing with that round trip
        line["cpu_baseline_with_strip_io"] = cpu_with_strip_io(sv, rho, src, obs, threads)
    print(json.dumps(line), flush=True)


def run_mine(args):
    import torch
    import torch.distributed as dist

    from swit_gb300 import Engine, shots, survey

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    large = args.workload == "large"
    if large:  # no autotune (each trial engine would hold the full survey) and no CPU-side extras
        args.no_tune = args.no_extras = True
    exact = args.adjoint == "exact"
    if exact:  # the kernel profile, plain path and CPU baseline time fd2dmpi's adjoint
        args.no_extras = True
    small = args.workload == "small"
    per_rank = args.shots or (200 if large else (5 if small else 49))
    full = survey.config(3 if large else (0 if small else 1), ns=per_rank * world, nt=args.nt)
    # rank r owns a contiguous block of shots (fd2dmpi/mmi_mpi.f90:52-80)
    lo, hi = shots.assigned(per_rank * world, rank, world)
    sv = full
    src_xz, rec_xz = full.src_xz[lo:hi], full.rec_xz[lo:hi]
    rho = sv.rho(sv.vp_true)
    src = sv.source()[lo:hi].copy()
    from swit_gb300.engine import checkpoint_interval
    if args.checkpoint in ("auto", "budget"):
        budget = 150e9 if args.checkpoint == "budget" else 0
        ckpt = checkpoint_interval(sv.nx, sv.nz, sv.npml, sv.nt, per_rank, budget, ng=sv.ng,
                                   exact=args.adjoint == "exact")
    else:
        ckpt = int(args.checkpoint)
    opts = dict(shots_per_batch=args.batch, block_x=args.block_x, kernel=args.kernel, checkpoint_every=ckpt,
                graph_branches=args.branches, adjoint=args.adjoint)
    tuned = None
    if not args.no_tune and args.batch == 0 and args.block_x == 0 and args.kernel == "auto" and args.branches == 0:
        from swit_gb300 import autotune
        best, trials = autotune.tune(sv.nx, sv.nz, sv.npml, sv.dx, sv.dt, src_xz, rec_xz, sv.vp_init, rho,
                                     free_surface=sv.free_surface, adjoint=args.adjoint)
        opts.update(best)
        tuned = [dict(c, ms=round(t * 1e3, 3)) for c, t in trials]
    eng = Engine(sv.nx, sv.nz, sv.npml, sv.nt, sv.dx, sv.dt, src_xz, rec_xz, **opts)
    q = eng.query()
    # observed data from the true model, synthetics from the smoothed model
    eng.set_model(sv.vp_true, rho)
    src_d = torch.from_numpy(src).cuda()
    obs_d = eng.forward(src_d, save_boundary=False)
    eng.set_model(sv.vp_init, rho)
    torch.cuda.synchronize()

    def step_device():
        out = eng.gradient_l2(src_d, obs_d)
        shots.allreduce_sum([out[k] for k in ("grad", "illum_fw", "illum_bk") if out[k] is not None])
        return out

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        last = step_device()
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    ms_per_step = ms / args.steps
    value = per_rank * world / (ms_per_step / 1000.0)

    # ---- e2e: the same step through the C ABI with host buffers
    src_h = torch.from_numpy(src).pin_memory()
    obs_h = obs_d.cpu().pin_memory()
    vp_h = torch.from_numpy(sv.vp_init).pin_memory()
    rho_h = torch.from_numpy(rho).pin_memory()

    def step_host():
        eng.set_model(vp_h, rho_h)
        out = eng.gradient_l2(src_h, obs_h)
        if world > 1:
            g = torch.from_numpy(np.stack([out[k] for k in ("grad", "illum_fw", "illum_bk")
                                           if out[k] is not None])).cuda()
            shots.allreduce_sum([g])
            g.cpu()
        return out

    for _ in range(max(1, args.warmup // 2)):
        step_host()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    NX, LD = sv.nx + 2 * sv.npml, ((sv.nz + 2 * sv.npml + 31) // 32) * 32
    LDI = ((sv.nz + 31) // 32) * 32
    h2d = (2 * sv.nx * sv.nz * 4 + src.nbytes + obs_h.numel() * 4 + 2 * NX * LD * 4 + sv.nx * LDI * 4
           + (sv.npml + 1) * 4)
    d2h = (1 if exact else 3) * sv.nx * sv.nz * 4 + per_rank * sv.ng * 8

    U, B = work_units(sv.nx, sv.nz, sv.npml, sv.nt, sv.ng)
    peak, peak_kind = measured_peak()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(sv, per_rank),
            "engine": {"path": "batched, CUDA graph", "kernel": q["kernel"], "shots_per_launch": q["shots_per_batch"],
                       "block_x": q["block_x"], "graph_branches": q["graph_branches"], "adjoint": args.adjoint,
                       "parallelism": "shots" + ("" if world == 1 else " x%d ranks" % world)},
            "autotune": {"trial_steps": 48, "candidates": tuned} if tuned else None,
            "gpts_per_s": value * U / 1e9,
            "hbm_roof_frac_step": (value / world) * B / 1e9 / peak,
            "algorithmic_gb_per_shot_gradient": B / 1e9,
            "e2e": {"value": per_rank * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "clocks": clk,
            "gpu_launches": int(args.steps * (q["kernels_per_forward"] + q["kernels_per_backward"] + 5))}
    import hashlib
    gh = last["grad"].detach().float().cpu().numpy()
    line["engine"]["memory"] = {
        "strategy": "checkpoints every %d steps" % ckpt if ckpt else "boundary saving",
        "device_bytes": q["device_bytes"],
        "gradient_sha256": hashlib.sha256(gh.tobytes()).hexdigest()[:16],
        "gradient_l2": float(np.linalg.norm(gh.astype(np.float64)))}

    if not args.no_extras:
        # per-kernel cost under graph conditions (swit_profile_kernels: each vec kernel alone in a graph of
        # the loop's batches and branches), the L2 roof, and the dominant kernel against both roofs
        prof = eng.profile_kernels()
        kb = kernel_bytes_per_shot(sv.nx, sv.nz, sv.npml, sv.ng, sv.nt)
        nbatch = -(-per_rank // q["shots_per_batch"])
        shots_launch = per_rank / nbatch  # mean shots per launch (the last batch may be smaller)
        vec = q["kernel"] == "vec"
        kern = {}
        for k, v in prof.items():
            per_step = v["mean_ms"] * (nbatch if vec else v["launches"] / (sv.nt - 1))
            kern[k] = dict(v, ms_per_time_step=per_step, ms_per_gradient=per_step * (sv.nt - 1))
        tot = sum(x["ms_per_gradient"] for x in kern.values())
        for k in kern:
            kern[k]["share"] = kern[k]["ms_per_gradient"] / tot
        top = max(kern, key=lambda k: kern[k]["ms_per_gradient"])
        alg = kb[top] * shots_launch
        achieved = alg / (prof[top]["mean_ms"] / 1000.0) / 1e9
        l2 = l2_bandwidth()
        traffic = BWD_P_TRAFFIC_PER_SHOT * shots_launch if (top == "bwd_p" and vec) else None
        line["roofline"] = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "peak_kind": peak_kind,
                            "traffic": traffic,
                            "traffic_source": "stored: ncu dram__bytes_read.sum + dram__bytes_write.sum of k_bwd_p_v, "
                                              "%d B per shot and launch (warm L2), scaled by shots per launch"
                                              % BWD_P_TRAFFIC_PER_SHOT if traffic else None,
                            "l2_peak": l2, "l2_frac": achieved / l2 if l2 else None,
                            "l2_peak_source": "measured in this run: swit_l2_bandwidth, read-modify-write sweeps "
                                              "over 64 MiB through L2",
                            "algorithmic_bytes_per_launch": alg, "mean_launch_ms": prof[top]["mean_ms"],
                            "shots_per_launch": shots_launch,
                            "timing": ("each kernel alone in a CUDA graph of every batch on the loop's %d branches, "
                                       "events around one replay" % q["graph_branches"]) if vec else
                                      "events around every launch",
                            "kernels": kern, "kernels_ms_per_gradient": tot,
                            "ms_per_step": ms_per_step}
        # plain one-shot-per-launch path on a bounded sample
        nplain = min(4, per_rank)
        pe = Engine(sv.nx, sv.nz, sv.npml, sv.nt, sv.dx, sv.dt, src_xz[:nplain], rec_xz[:nplain], path="plain",
                    kernel=q["kernel"], block_x=q["block_x"])
        pe.set_model(sv.vp_init, rho)
        src_p, obs_p = src_d[:nplain].contiguous(), obs_d[:nplain].contiguous()
        pe.gradient_l2(src_p, obs_p)
        torch.cuda.synchronize()
        ev0.record(stream)
        pe.gradient_l2(src_p, obs_p)
        ev1.record(stream)
        torch.cuda.synchronize()
        plain = nplain / (ev0.elapsed_time(ev1) / 1000.0)
        pe.close()
        line["plain"] = {"value": plain, "unit": UNIT,
                         "sample": "%d shots, one shot per launch, no graph; shots run one after another, so all %d "
                                   "take %.2f s at this rate" % (nplain, per_rank, per_rank / plain)}
        line["batched_over_plain"] = (value / world) / plain
        if rank == 0 and world == 1:
            # every shot of the workload on the oracle: the timed CPU baseline and the FP32 parity target
            threads = os.cpu_count() or 1
            ref32, wall = oracle_gradient(sv, rho, src, obs_d.cpu().numpy(), threads)
            line["cpu_baseline"] = {"value": sv.ns / wall, "unit": UNIT, "cores": threads, "kind": "port",
                                    "sample": "all %d shots at full nt=%d, one shot per thread, %.1f s wall"
                                              % (sv.ns, sv.nt, wall)}
            fin = eng.gradient_l2(src_d, obs_d, return_seis=True)
            line["parity"] = full_size_parity(sv, rho, src_d, obs_d, fin, ref32)
            del ref32, fin
    eng.close()
    if large and rank == 0 and world == 1 and args.parity_shots > 0:
        line["parity"] = subset_parity(sv, rho, args.parity_shots)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_multi(args):
    """Uneven multi-instance batch: L-BFGS (swit_gb300.optim) on every problem,
    (a) all problems stepped together by one MultiEngine (fwi_lockstep), (b) one
    problem after another on its own batched engine, (c) one after another on the
    plain path (one shot per launch, no graph).  Reports L-BFGS iterations per
    second of each and the largest difference between their final models."""
    import torch

    from swit_gb300 import Engine, MultiEngine, optim, precond, survey
    probs = survey.config4_instances(args.instances, args.scale, args.scale)
    srcs = [torch.from_numpy(p.source()).cuda() for p in probs]
    vpmax = 5000.0

    def prec(p, o):
        return precond.grad_precond(o["grad"], o["illum_fw"], o["illum_bk"], p.nx, p.nz, vpmax, "Land", 0, 0.0, 0)

    def model(p, v):
        return v.reshape(p.nx, p.nz).float().contiguous()

    me = MultiEngine([p.engine_args() for p in probs])
    obss = []
    for e, p, s in zip(me.engines, probs, srcs):
        e.set_model(torch.from_numpy(p.vp_true).cuda(), torch.from_numpy(p.rho(p.vp_true)).cuda())
        obss.append(e.forward(s, save_boundary=False))
    rhos = [torch.from_numpy(p.rho(p.vp_true)).cuda() for p in probs]
    v0s = [torch.from_numpy(p.vp_init).cuda().double().reshape(-1) for p in probs]

    def set_all(vs):
        for e, p, v, r in zip(me.engines, probs, vs, rhos):
            e.set_model(model(p, v), r)

    def objective_all(vs):
        set_all(vs)
        return [(o["misfit"], prec(p, o)) for p, o in zip(probs, me.gradient_l2(srcs, obss))]

    def misfit_all(vs, active):
        for e, p, v, r, a in zip(me.engines, probs, vs, rhos, active):
            if a:
                e.set_model(model(p, v), r)
        return me.misfit_l2(srcs, obss, active)

    # one gradient of every problem: together vs one engine after another (kernel efficiency alone);
    # the first pass also warms the libraries the preconditioning uses, so no timed run pays for that
    set_all(v0s)
    for p, o in zip(probs, me.gradient_l2(srcs, obss)):
        prec(p, o)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    me.gradient_l2(srcs, obss)
    torch.cuda.synchronize()
    t_grad_multi = time.perf_counter() - t0
    t_grad_seq = 0.0
    for p, s, o, r, v0 in zip(probs, srcs, obss, rhos, v0s):
        with Engine(**p.engine_args()) as e:
            e.set_model(model(p, v0), r)
            e.gradient_l2(s, o)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            e.gradient_l2(s, o)
            torch.cuda.synchronize()
            t_grad_seq += time.perf_counter() - t1
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sts, hists = optim.fwi_lockstep(v0s, objective_all, misfit_all, maxiter=args.iters, vpmax=vpmax, vpmin=1000.0)
    torch.cuda.synchronize()
    t_multi = time.perf_counter() - t0
    me.close()

    def one_by_one(path):
        finals, t = [], 0.0
        for p, s, o, r, v0 in zip(probs, srcs, obss, rhos, v0s):
            with Engine(**p.engine_args(), path=path) as e:
                def obj(v, e=e, p=p, s=s, o=o, r=r):
                    e.set_model(model(p, v), r)
                    out = e.gradient_l2(s, o)
                    return out["misfit"], prec(p, out)

                def mis(v, e=e, p=p, s=s, o=o, r=r):
                    e.set_model(model(p, v), r)
                    return e.misfit_l2(s, o)

                torch.cuda.synchronize()
                t1 = time.perf_counter()
                st, _ = optim.fwi(v0, obj, mis, maxiter=args.iters, vpmax=vpmax, vpmin=1000.0)
                torch.cuda.synchronize()
                t += time.perf_counter() - t1
                finals.append(st["v_now"])
        return finals, t

    fin_b, t_batched = one_by_one("batched")
    diff = max(float((a["v_now"] - b).abs().max()) for a, b in zip(sts, fin_b))
    # the plain path (one shot per launch, no graph): one gradient of every problem, and the full L-BFGS
    # only on request (about 14x the batched time); otherwise its L-BFGS time is the batched one scaled by
    # the plain / batched ratio of one gradient of every problem
    t_grad_plain = 0.0
    for p, s, o, r, v0 in zip(probs, srcs, obss, rhos, v0s):
        with Engine(**p.engine_args(), path="plain") as e:
            e.set_model(model(p, v0), r)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            e.gradient_l2(s, o)
            torch.cuda.synchronize()
            t_grad_plain += time.perf_counter() - t1
    if args.plain_lbfgs:
        fin_p, t_plain = one_by_one("plain")
        diff_p = max(float((a["v_now"] - b).abs().max()) for a, b in zip(sts, fin_p))
        plain_kind = "measured"
    else:
        t_plain, diff_p = t_batched * t_grad_plain / t_grad_seq, None
        plain_kind = "estimated: sequential batched L-BFGS time x (plain / batched time of one gradient of every problem)"
    n_it = args.instances * args.iters
    line = {"metric": "multi-instance FWI: L-BFGS iterations/s over all problems", "value": n_it / t_multi,
            "unit": "iterations/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "uneven multi-instance batch", "instances": args.instances, "iters": args.iters,
                       "shot_and_nt_scale": args.scale,
                       "grids": [[p.nx, p.nz] for p in probs], "shots": [p.ns for p in probs],
                       "nt": [p.nt for p in probs]},
            "seconds": {"multi": t_multi, "sequential_batched": t_batched, "sequential_plain": t_plain,
                        "sequential_plain_kind": plain_kind,
                        "one_gradient_each_multi": t_grad_multi, "one_gradient_each_sequential": t_grad_seq,
                        "one_gradient_each_sequential_plain": t_grad_plain},
            "shots_total": int(sum(p.ns for p in probs)),
            "speedup": {"vs_sequential_batched": t_batched / t_multi, "vs_sequential_plain": t_plain / t_multi},
            "max_model_difference_m_s": {"vs_sequential_batched": diff, "vs_sequential_plain": diff_p},
            "final_misfit_ratio": [h[-1]["f"] / h[0]["f"] if h[0]["f"] else None for h in hists]}
    print(json.dumps(line), flush=True)


def run_correlation(args):
    """The differentiable path with correlation misfits at 501x171, nt 5000, 51
    shots: seismograms from autograd.propagate, normalised global-correlation
    plus cross-correlation traveltime misfit (swit_gb300.misfit, the reference's
    adjoint sources), loss.backward() through the engine's reverse loop (fd2dmpi's
    adjoint, or the exact adjoint with --adjoint exact).  A step is one such
    gradient of every shot."""
    import torch

    from swit_gb300 import Engine, misfit, survey
    from swit_gb300.autograd import propagate
    sv = survey.config(2, ns=args.shots, nt=args.nt)
    ckpt = int(args.checkpoint) if args.checkpoint != "auto" else 0
    opts = dict(shots_per_batch=args.batch, block_x=args.block_x, graph_branches=args.branches, adjoint=args.adjoint,
                checkpoint_every=ckpt)
    eng = Engine(**sv.engine_args(), kernel="vec" if args.kernel == "auto" else args.kernel, **opts)
    q = eng.query()
    rho = torch.from_numpy(sv.rho(sv.vp_true)).cuda()
    src = torch.from_numpy(sv.source()).cuda()
    eng.set_model(torch.from_numpy(sv.vp_true).cuda(), rho)
    obs = eng.forward(src, save_boundary=False).clone()
    vp0 = torch.from_numpy(sv.vp_init).cuda()

    def step(vp_in, src_in, obs_in):
        vp = vp_in.clone().requires_grad_(True)
        seis = propagate(eng, vp, rho, src_in)
        loss = misfit.global_correlation(seis, obs_in, sv.dt) + misfit.traveltime(seis, obs_in, sv.dt)
        loss.backward()
        return vp.grad, loss.detach()

    for _ in range(args.warmup):
        step(vp0, src, obs)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        g, loss = step(vp0, src, obs)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms_per_step = ev0.elapsed_time(ev1) / args.steps
    value = sv.ns / (ms_per_step / 1000.0)
    # end to end: model, sources and observed data from pinned host memory, gradient and misfit back
    vp_h, src_h, obs_h = vp0.cpu().pin_memory(), src.cpu().pin_memory(), obs.cpu().pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gg, ll = step(vp_h.cuda(non_blocking=True), src_h.cuda(non_blocking=True), obs_h.cuda(non_blocking=True))
        gg.cpu(), ll.cpu()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    U, B = work_units(sv.nx, sv.nz, sv.npml, sv.nt, sv.ng)
    peak, peak_kind = measured_peak()
    gh = g.double().cpu().numpy()
    line = {"metric": "FWI shot-gradients/s (501x171, nt=5000) global-correlation + traveltime misfits through "
                      "torch.autograd", "value": value, "unit": "shot-gradients/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": sv.name, "grid": [sv.nx, sv.nz], "npml": sv.npml, "nt": sv.nt, "shots": sv.ns,
                       "receivers": sv.ng, "dx_m": sv.dx, "dt_s": sv.dt, "adjoint": args.adjoint,
                       "kernel": q["kernel"], "shots_per_launch": q["shots_per_batch"],
                       "graph_branches": q["graph_branches"],
                       "memory": {"strategy": "checkpoints every %d steps" % ckpt if ckpt else "stored per step",
                                  "device_bytes": q["device_bytes"]},
                       "l2": "inputs larger than L2: each step streams the per-step records of every shot",
                       "gradient_l2": float(np.linalg.norm(gh)), "loss": float(loss)},
            "gpts_per_s": value * U / 1e9, "hbm_roof_frac_step": value * B / 1e9 / peak, "peak_kind": peak_kind,
            "e2e": {"value": sv.ns / e2e_s, "unit": "shot-gradients/s",
                    "h2d_bytes_per_step": int(vp_h.numel() * 4 + src_h.numel() * 4 + obs_h.numel() * 4),
                    "d2h_bytes_per_step": int(sv.nx * sv.nz * 4 + 4)},
            "clocks": clk,
            "gpu_launches": int(args.steps * (q["kernels_per_forward"] + q["kernels_per_backward"] + 5))}
    if not args.no_extras and args.adjoint == "fd2dmpi":
        # the engine's Waveform gradient of every shot at this size against the FP64 build and the oracle
        rho_h = sv.rho(sv.vp_true)
        eng.set_model(vp0, rho)
        mine = eng.gradient_l2(src, obs, return_seis=True)
        ref32, wall = oracle_gradient(sv, rho_h, sv.source(), obs.cpu().numpy(), os.cpu_count() or 1)
        line["parity"] = full_size_parity(sv, rho_h, src, obs, mine, ref32)
        line["parity"]["misfit"] = "Waveform (the correlation misfits' gradients run the same reverse loop)"
        line["cpu_baseline"] = {"value": sv.ns / wall, "unit": "shot-gradients/s", "cores": os.cpu_count() or 1,
                                "kind": "port", "sample": "Waveform gradient of all %d shots at full nt=%d, one shot "
                                                          "per thread, %.1f s wall" % (sv.ns, sv.nt, wall)}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "multi":
        run_multi(args)
    elif args.workload == "correlation":
        run_correlation(args)
    else:
        run_mine(args)


if __name__ == "__main__":
    main()
