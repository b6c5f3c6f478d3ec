"""Python front end of the GB300 engine (one object per model geometry).

``Engine`` owns a ``swit_engine`` from the C ABI (include/swit_gb300.h).  Arrays
may be numpy arrays (host buffers, copied inside the call) or CUDA torch
tensors (device buffers; the call is ordered on torch's current stream).
Layouts follow SWIT's Python side: model and gradients (nx, nz), sources
(ns, nt), seismograms and adjoint sources (ns, ng_max, nt).
"""
import ctypes as C

import numpy as np

from . import _lib


def _is_torch(a):
    return type(a).__module__.split(".")[0] == "torch"


class Engine:
    """Batched forward / adjoint / imaging engine for one model geometry.

    Parameters mirror the fd2dmpi parfile (NX, NZ, DX, NPML, NT_WORK, DT_WORK,
    FREESURFACE; fd2dmpi/io.f90:74-96) and coord.txt (toolbox/solver.py:171-180).
    ``src_xz`` is (ns, 2) and ``rec_xz`` is (ns, ng_max, 2) or (ng, 2) shared by
    all shots, in metres.
    """

    def __init__(self, nx, nz, npml, nt, dx, dt, src_xz, rec_xz, free_surface=1, ng=None, precision="fp32",
                 path="batched", shots_per_batch=0, block_x=0, kernel="auto", checkpoint_every=0, graph_branches=0,
                 adjoint="fd2dmpi", receiver_component="p", _borrow=None):
        lib = _lib.load()
        src_xz = np.asarray(src_xz, dtype=np.float32).reshape(-1, 2)
        rec_xz = np.asarray(rec_xz, dtype=np.float32)
        if rec_xz.ndim == 2:
            rec_xz = np.broadcast_to(rec_xz, (src_xz.shape[0],) + rec_xz.shape)
        if rec_xz.ndim != 3 or rec_xz.shape[0] != src_xz.shape[0] or rec_xz.shape[2] != 2:
            raise ValueError("rec_xz must be (ns, ng_max, 2) or (ng, 2)")
        self.nx, self.nz, self.npml, self.nt = int(nx), int(nz), int(npml), int(nt)
        self.dx, self.dt = float(np.float32(dx)), float(np.float32(dt))
        self.ns, self.ngmax = src_xz.shape[0], rec_xz.shape[1]
        self.precision = precision
        self.fp64 = precision == "fp64"
        if precision not in ("fp32", "fp64"):
            raise ValueError("precision must be 'fp32' or 'fp64'")
        if path not in ("batched", "plain"):
            raise ValueError("path must be 'batched' or 'plain'")
        self.path = path
        variants = {"auto": 0, "split": 1, "walk": 2, "vec": 3, "cluster": 4, "hybrid": 5, "band": 6}
        if adjoint not in ("fd2dmpi", "exact"):
            raise ValueError("adjoint must be 'fd2dmpi' or 'exact'")
        self.adjoint = adjoint
        comps = {"p": 0, "vx": 1, "vz": 2}
        if receiver_component not in comps:
            raise ValueError("receiver_component must be 'p', 'vx' or 'vz'")
        self.receiver_component = receiver_component
        if kernel not in variants:
            raise ValueError("kernel must be one of %s" % ", ".join(sorted(variants)))
        self._keep = dict(
            ng=np.ascontiguousarray(np.full(self.ns, self.ngmax) if ng is None else ng, dtype=np.int32),
            xs=np.ascontiguousarray(src_xz[:, 0]), zs=np.ascontiguousarray(src_xz[:, 1]),
            xg=np.ascontiguousarray(rec_xz[:, :, 0]).reshape(-1), zg=np.ascontiguousarray(rec_xz[:, :, 1]).reshape(-1))
        k = self._keep
        d = _lib.SwitDesc(self.nx, self.nz, self.npml, self.nt, self.dx, self.dt, int(free_surface), self.ns,
                          self.ngmax, k["ng"].ctypes.data, k["xs"].ctypes.data, k["zs"].ctypes.data,
                          k["xg"].ctypes.data, k["zg"].ctypes.data, 1 if self.fp64 else 0,
                          1 if path == "plain" else 0, int(shots_per_batch), int(block_x), variants[kernel],
                          int(checkpoint_every), int(graph_branches), 1 if adjoint == "exact" else 0,
                          comps[receiver_component])
        self.checkpoint_every = int(checkpoint_every)
        self._desc = d
        self._lib = lib
        self._owned = _borrow is None
        if _borrow is not None:  # an instance of a MultiEngine, which owns the handle
            self._h = _borrow
            return
        h = C.c_void_p()
        _lib.check(lib.swit_create(C.byref(d), C.byref(h)))
        self._h = h

    # ------------------------------------------------------------------ utils
    @property
    def out_dtype(self):
        return np.float64 if self.fp64 else np.float32

    def _ptr(self, a, dtype):
        """Returns (pointer, on_device) for a numpy array or CUDA tensor input."""
        if a is None:
            return None, None
        if _is_torch(a):
            import torch
            if not a.is_cuda:
                a = a.detach().numpy()
            else:
                want = torch.float32 if dtype == np.float32 else torch.float64
                if a.dtype != want or not a.is_contiguous():
                    raise ValueError("device arrays must be contiguous %s" % want)
                return a.data_ptr(), 1
        if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
            raise ValueError("host arrays must be C-contiguous %s" % np.dtype(dtype).name)
        return a.ctypes.data, 0

    @staticmethod
    def _stream(on_device):
        if on_device:
            import torch
            return torch.cuda.current_stream().cuda_stream
        return None

    def _new(self, shape, like_device):
        if like_device:
            import torch
            return torch.zeros(shape, dtype=torch.float64 if self.fp64 else torch.float32, device="cuda")
        return np.zeros(shape, self.out_dtype)

    @staticmethod
    def _f32(a):
        """float32, C-contiguous; host inputs that already are keep their buffer (a
        pinned torch tensor stays pinned, so the engine's copy is a direct DMA)."""
        if _is_torch(a):
            if a.is_cuda:
                return a.contiguous().float()
            return np.ascontiguousarray(a.detach().numpy(), dtype=np.float32)
        return np.ascontiguousarray(a, dtype=np.float32)

    # ------------------------------------------------------------------ API
    def set_model(self, vp, rho):
        """vp, rho: (nx, nz) float32."""
        vp, rho = self._f32(vp), self._f32(rho)
        if tuple(vp.shape) != (self.nx, self.nz) or tuple(rho.shape) != (self.nx, self.nz):
            raise ValueError("vp/rho must be (nx, nz) = (%d, %d)" % (self.nx, self.nz))
        pv, dev = self._ptr(vp, np.float32)
        pr, dev2 = self._ptr(rho, np.float32)
        if dev != dev2:
            raise ValueError("vp and rho must both be host or both be device arrays")
        _lib.check(self._lib.swit_set_model(self._h, pv, pr, dev, self._stream(dev)))

    def forward(self, src, save_boundary=True, seis=None):
        """Seismograms (ns, ng_max, nt) of source functions src (ns, nt)."""
        src = self._f32(src)
        if tuple(src.shape) != (self.ns, self.nt):
            raise ValueError("src must be (ns, nt) = (%d, %d)" % (self.ns, self.nt))
        ps, dev = self._ptr(src, np.float32)
        if seis is None:
            seis = self._new((self.ns, self.ngmax, self.nt), dev)
        po, _ = self._ptr(seis, self.out_dtype)
        _lib.check(self._lib.swit_forward(self._h, ps, po, 1 if save_boundary else 0, dev, self._stream(dev)))
        return seis

    def backward(self, adj, grad=None, illum_fw=None, illum_bk=None):
        """(grad, illum_fw, illum_bk), each (nx, nz), for adjoint sources adj (ns, ng_max, nt)."""
        adj = self._f32(adj)
        if tuple(adj.shape) != (self.ns, self.ngmax, self.nt):
            raise ValueError("adj must be (ns, ng_max, nt)")
        pa, dev = self._ptr(adj, np.float32)
        outs = [x if x is not None else self._new((self.nx, self.nz), dev) for x in (grad, illum_fw, illum_bk)]
        ptrs = [self._ptr(x, self.out_dtype)[0] for x in outs]
        _lib.check(self._lib.swit_backward(self._h, pa, ptrs[0], ptrs[1], ptrs[2], dev, self._stream(dev)))
        return tuple(outs)

    def backward_exact(self, adj, grad=None, src_grad=None):
        """Exact discrete adjoint (engines with adjoint="exact") of adjoint sources
        adj (ns, ng_max, nt) = dJ/dseis after forward(save_boundary=True): returns
        (grad (nx, nz) = dJ/dvp with the damping profile held fixed,
        src_grad (ns, nt) = dJ/dsrc)."""
        adj = self._f32(adj)
        if tuple(adj.shape) != (self.ns, self.ngmax, self.nt):
            raise ValueError("adj must be (ns, ng_max, nt)")
        pa, dev = self._ptr(adj, np.float32)
        grad = grad if grad is not None else self._new((self.nx, self.nz), dev)
        src_grad = src_grad if src_grad is not None else self._new((self.ns, self.nt), dev)
        _lib.check(self._lib.swit_backward_exact(self._h, pa, self._ptr(grad, self.out_dtype)[0],
                                                 self._ptr(src_grad, self.out_dtype)[0], dev, self._stream(dev)))
        return grad, src_grad

    def gradient_l2(self, src, obs, return_seis=False):
        """Waveform-misfit gradient: returns dict(grad, illum_fw, illum_bk, misfit[, seis])
        (exact-adjoint engines: the exact gradient and no illumination)."""
        src, obs = self._f32(src), self._f32(obs)
        ps, dev = self._ptr(src, np.float32)
        po, dev2 = self._ptr(obs, np.float32)
        if dev != dev2:
            raise ValueError("src and obs must both be host or both be device arrays")
        outs = [self._new((self.nx, self.nz), dev) if k == 0 or self.adjoint == "fd2dmpi" else None for k in range(3)]
        seis = self._new((self.ns, self.ngmax, self.nt), dev) if return_seis else None
        m = C.c_double(0.0)
        _lib.check(self._lib.swit_gradient_l2(self._h, ps, po, *[self._ptr(x, self.out_dtype)[0] for x in outs],
                                              self._ptr(seis, self.out_dtype)[0], C.byref(m), dev,
                                              self._stream(dev)))
        out = dict(grad=outs[0], illum_fw=outs[1], illum_bk=outs[2], misfit=m.value)
        if return_seis:
            out["seis"] = seis
        return out

    def misfit_l2(self, src, obs):
        """Waveform misfit only (a forward run without strips; swit_misfit_l2)."""
        src, obs = self._f32(src), self._f32(obs)
        ps, dev = self._ptr(src, np.float32)
        po, dev2 = self._ptr(obs, np.float32)
        if dev != dev2:
            raise ValueError("src and obs must both be host or both be device arrays")
        m = C.c_double(0.0)
        _lib.check(self._lib.swit_misfit_l2(self._h, ps, po, C.byref(m), dev, self._stream(dev)))
        return m.value

    def export_snapshot(self):
        """Boundary strips (ns, nt, 9nx+6nz) and p_end/u_end/w_end (ns, nx, nz) of the last saved forward."""
        b = np.zeros((self.ns, self.nt, 9 * self.nx + 6 * self.nz), self.out_dtype)
        ends = [np.zeros((self.ns, self.nx, self.nz), self.out_dtype) for _ in range(3)]
        _lib.check(self._lib.swit_export_snapshot(self._h, b.ctypes.data, *[x.ctypes.data for x in ends], 0, None))
        return dict(boundary=b, p_end=ends[0], u_end=ends[1], w_end=ends[2])

    def import_snapshot(self, src, boundary, p_end, u_end, w_end):
        """Loads a saved forward run (see swit_import_snapshot): src (ns, nt), boundary
        (ns, nt, 9nx+6nz), p_end/u_end/w_end (ns, nx, nz), all float32 host arrays."""
        arrs = [self._f32(a) for a in (src, boundary, p_end, u_end, w_end)]
        ptrs = [self._ptr(a, np.float32)[0] for a in arrs]
        _lib.check(self._lib.swit_import_snapshot(self._h, *ptrs, 0, None))

    def profile_kernels(self):
        """Mean launch duration (ms) and launch count of the four stencil kernels,
        timed with CUDA events on torch's current stream (see swit_profile_kernels)."""
        import torch
        n = (C.c_int32 * 4)()
        ms = (C.c_double * 4)()
        _lib.check(self._lib.swit_profile_kernels(self._h, n, ms, torch.cuda.current_stream().cuda_stream))
        names = ("fwd_p", "fwd_uw", "bwd_uw", "bwd_p")
        kind = self.query()["kernel"]
        if kind == "walk":
            names = ("fwd_step", None, "bwd_step", None)
        elif kind == "cluster":
            names = ("fwd_loop", None, "bwd_loop", None)
        elif kind == "hybrid":
            names = ("fwd_loop", None, "bwd_uw", "bwd_p")
        return {k: dict(launches=int(n[i]), mean_ms=float(ms[i])) for i, k in enumerate(names) if k}

    def query(self):
        by = C.c_int64()
        sb, bx, kf, kb, kv, br = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        _lib.check(self._lib.swit_query(self._h, C.byref(by), C.byref(sb), C.byref(bx), C.byref(kf), C.byref(kb),
                                        C.byref(kv), C.byref(br)))
        return dict(device_bytes=by.value, shots_per_batch=sb.value, block_x=bx.value, graph_branches=br.value,
                    kernels_per_forward=kf.value,
                    kernels_per_backward=kb.value, kernel={1: "split", 2: "walk", 3: "vec", 4: "cluster", 5: "hybrid", 6: "band"}.get(kv.value, "?"))

    def check(self):
        """Waits for torch's current stream and raises SwitError if a kernel gave
        up waiting on an in-kernel copy since the last check (swit_check)."""
        import torch
        _lib.check(self._lib.swit_check(self._h, torch.cuda.current_stream().cuda_stream))

    def close(self):
        if getattr(self, "_h", None):
            if getattr(self, "_owned", True):
                self._lib.swit_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class MultiEngine:
    """Many independent problems (grids, shot counts, record lengths may all
    differ) stepped together: (problem, shot) pairs in L2-sized waves (a
    problem's own shots, or several small problems) on concurrent branches, per
    wave one launch of each phase kernel per time step over the pairs still
    running (swit_multi_*).  ``problems`` is a list
    of Engine keyword dicts (nx, nz, npml, nt, dx, dt, src_xz, rec_xz[, ng,
    free_surface, block_x]); ``engines[i]`` is problem i's Engine (set_model,
    forward, ... work on it alone)."""

    def __init__(self, problems):
        lib = _lib.load()
        views = [Engine(**p, _borrow=C.c_void_p(1)) for p in problems]  # descriptions only
        for v in views:
            if v.fp64 or v.path != "batched" or v.checkpoint_every:
                raise ValueError("a MultiEngine runs FP32 problems on the batched path with boundary saving")
        descs = (_lib.SwitDesc * len(views))(*[v._desc for v in views])
        h = C.c_void_p()
        _lib.check(lib.swit_multi_create(descs, len(views), C.byref(h)))
        self._h, self._lib = h, lib
        self.engines = []
        for i, (v, p) in enumerate(zip(views, problems)):
            e = C.c_void_p()
            _lib.check(lib.swit_multi_engine(h, i, C.byref(e)))
            v._h = e
            self.engines.append(v)

    def __len__(self):
        return len(self.engines)

    def _inputs(self, srcs, obss):
        if len(srcs) != len(self) or len(obss) != len(self):
            raise ValueError("one src and one obs per problem")
        ps, po, keep, devs = [], [], [], set()
        for e, s, o in zip(self.engines, srcs, obss):
            s, o = e._f32(s), e._f32(o)
            if tuple(s.shape) != (e.ns, e.nt) or tuple(o.shape) != (e.ns, e.ngmax, e.nt):
                raise ValueError("src (ns, nt) and obs (ns, ng_max, nt) per problem")
            a, d1 = e._ptr(s, np.float32)
            b, d2 = e._ptr(o, np.float32)
            ps.append(a)
            po.append(b)
            keep += [s, o]
            devs |= {d1, d2}
        if len(devs) != 1:
            raise ValueError("all inputs must be host arrays or all device arrays")
        dev = devs.pop()
        return (C.c_void_p * len(self))(*ps), (C.c_void_p * len(self))(*po), dev, keep

    def gradient_l2(self, srcs, obss):
        """Waveform-misfit gradients of every problem: a list of dict(grad, illum_fw, illum_bk, misfit)."""
        ps, po, dev, keep = self._inputs(srcs, obss)
        outs = [[e._new((e.nx, e.nz), dev) for _ in range(3)] for e in self.engines]
        arr = [(C.c_void_p * len(self))(*[e._ptr(o[j], e.out_dtype)[0] for e, o in zip(self.engines, outs)])
               for j in range(3)]
        m = (C.c_double * len(self))()
        _lib.check(self._lib.swit_multi_gradient_l2(self._h, ps, po, arr[0], arr[1], arr[2], m, dev,
                                                    Engine._stream(dev)))
        return [dict(grad=o[0], illum_fw=o[1], illum_bk=o[2], misfit=m[i]) for i, o in enumerate(outs)]

    def misfit_l2(self, srcs, obss, active=None):
        """Waveform misfit of every problem with active[i] true (all by default;
        the others do no work and get 0): forward runs only."""
        ps, po, dev, keep = self._inputs(srcs, obss)
        act = None if active is None else (C.c_int32 * len(self))(*[1 if a else 0 for a in active])
        m = (C.c_double * len(self))()
        _lib.check(self._lib.swit_multi_misfit_l2(self._h, ps, po, act, m, dev, Engine._stream(dev)))
        return list(m)

    def close(self):
        if getattr(self, "_h", None):
            for e in self.engines:
                e._h = None
            self._lib.swit_multi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def checkpoint_interval(nx, nz, npml, nt, ns, budget_bytes, ng=None, fp64=False, exact=False):
    """Memory strategy for a survey: 0 (boundary saving, fd2dmpi's own) when the
    engine with the strips of all shots fits in ``budget_bytes`` (wavefields,
    imaging sums and trace staging included; ng receivers per shot, default nx),
    else the checkpoint interval k that minimises checkpoints + strip buffer,
    ns * (ceil(nt/k) * 3 * NX * LD + k * (9 nx + 6 nz)) values (the allocation of
    swit_create with checkpoint_every = k).  exact: an exact-adjoint engine,
    whose per-step record is a whole NX * LD divergence field instead of the
    strips."""
    esz = 8 if fp64 else 4
    NX, NZ = nx + 2 * npml, nz + 2 * npml
    fsz = NX * ((NZ + 31) // 32) * 32
    sl = fsz if exact else 9 * nx + 6 * nz
    ng = nx if ng is None else ng
    rest = 12 * ns * fsz * esz + ns * ng * nt * (3 * esz + 4)  # fields and sums; seis, adjoint, staging, input
    if ns * nt * sl * esz + rest <= budget_bytes:
        return 0

    def mem(k):
        return ns * (-(-nt // k) * 3 * fsz + k * sl) * esz

    k0 = max(1, int(round(((nt - 1) * 3 * fsz / sl) ** 0.5)))
    return min(range(max(1, k0 // 2), min(nt, 2 * k0) + 1), key=mem)


def damp_profile(nx, nz, npml, dx, vmin):
    """Closed-form damping profile damp_global (NX, NZ) the kernels evaluate (host-side, no GPU)."""
    lib = _lib.load()
    out = np.zeros((nx + 2 * npml, nz + 2 * npml), np.float32)
    _lib.check(lib.swit_damp_profile(int(nx), int(nz), int(npml), float(np.float32(dx)), float(np.float32(vmin)),
                                     out.ctypes.data))
    return out
