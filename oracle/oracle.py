"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module.  It wraps ``libfd2d_oracle.so`` (built by ``oracle/build.py``), a
statement-by-statement C++ restatement of fd2dmpi's forward
(fd2dmpi/fdcore.f90:30-198), reconstruction (fdcore.f90:202-289), adjoint
(fdcore.f90:293-375) and imaging/shot-sum (fd2dmpi/solver.f90:230-270), plus
the exact discrete adjoint of that forward (``exact``; pinned by
``oracle/exact.py``).

Array conventions (all z-fastest, as SWIT's Python side):
  vp, rho            (nx, nz) float32
  src                (ns, nt) float32            forward source, already integrated
  seismograms, adj   (ns, ngmax, nt)             one trace per receiver
  boundary           (ns, nt, 9nx+6nz)           reference boundary(S, nt) layout
  p/u/w_end, g, fw, bk (ns or 1, nx, nz)
"""
import ctypes as C
import os

import numpy as np

from . import build as _build


class _Desc(C.Structure):
    _fields_ = [("nx", C.c_int32), ("nz", C.c_int32), ("npml", C.c_int32), ("nt", C.c_int32),
                ("dx", C.c_float), ("dt", C.c_float), ("free_surface", C.c_int32),
                ("ns", C.c_int32), ("ngmax", C.c_int32),
                ("ng", C.POINTER(C.c_int32)), ("xs", C.POINTER(C.c_float)), ("zs", C.POINTER(C.c_float)),
                ("xg", C.POINTER(C.c_float)), ("zg", C.POINTER(C.c_float)), ("comp", C.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.build())
    return _lib


def _p(a, ct=C.c_float):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


class Problem:
    """Model + acquisition in the units of SWIT's parfile and coord.txt."""

    def __init__(self, nx, nz, npml, nt, dx, dt, src_xz, rec_xz, free_surface=1, ng=None, comp="p"):
        if comp not in ("p", "vx", "vz"):
            raise ValueError("comp must be 'p', 'vx' or 'vz'")
        self.comp = {"p": 0, "vx": 1, "vz": 2}[comp]
        self.nx, self.nz, self.npml, self.nt = int(nx), int(nz), int(npml), int(nt)
        self.dx, self.dt = np.float32(dx), np.float32(dt)
        self.free_surface = int(free_surface)
        src_xz = np.asarray(src_xz, dtype=np.float32).reshape(-1, 2)
        rec_xz = np.asarray(rec_xz, dtype=np.float32)
        if rec_xz.ndim == 2:
            rec_xz = np.broadcast_to(rec_xz, (src_xz.shape[0],) + rec_xz.shape)
        self.ns = src_xz.shape[0]
        self.ngmax = rec_xz.shape[1]
        self.ng = (np.full(self.ns, self.ngmax, np.int32) if ng is None else np.asarray(ng, np.int32))
        self.xs = np.ascontiguousarray(src_xz[:, 0])
        self.zs = np.ascontiguousarray(src_xz[:, 1])
        self.xg = np.ascontiguousarray(rec_xz[:, :, 0]).reshape(-1)
        self.zg = np.ascontiguousarray(rec_xz[:, :, 1]).reshape(-1)

    def desc(self):
        d = _Desc(self.nx, self.nz, self.npml, self.nt, self.dx, self.dt, self.free_surface, self.ns, self.ngmax,
                  _p(self.ng, C.c_int32), _p(self.xs), _p(self.zs), _p(self.xg), _p(self.zg), self.comp)
        return d

    @property
    def strip_len(self):
        return 9 * self.nx + 6 * self.nz


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _check(rc, what):
    if rc != 0:
        raise ValueError("oracle %s failed with code %d" % (what, rc))


def forward(pb: Problem, vp, rho, src, store=True, fp64=False, nthreads=None):
    """Forward modeling of every shot.  Returns dict(seis, boundary, p_end, u_end, w_end)."""
    nthreads = nthreads or os.cpu_count()
    R = np.float64 if fp64 else np.float32
    seis = np.zeros((pb.ns, pb.ngmax, pb.nt), R)
    out = dict(seis=seis)
    if store:
        out["boundary"] = np.zeros((pb.ns, pb.nt, pb.strip_len), R)
        for k in ("p_end", "u_end", "w_end"):
            out[k] = np.zeros((pb.ns, pb.nx, pb.nz), R)
    ct = C.c_double if fp64 else C.c_float
    fn = lib().oracle_forward_f64 if fp64 else lib().oracle_forward_f32
    vp, rho, src = _f32(vp), _f32(rho), _f32(src)
    d = pb.desc()
    rc = fn(C.byref(d), _p(vp), _p(rho), _p(src), C.c_int(1 if store else 0), _p(seis, ct),
            _p(out.get("boundary"), ct), _p(out.get("p_end"), ct), _p(out.get("u_end"), ct),
            _p(out.get("w_end"), ct), C.c_int(nthreads))
    _check(rc, "forward")
    return out


def adjoint(pb: Problem, vp, rho, src, adj, fwd, fp64=False, record_adjoint=False, nthreads=None):
    """Reverse loop (reconstruction + adjoint + imaging) of every shot, summed.

    Returns dict(g, fw, bk[, adj_seis]) with g already scaled by -2/c.
    """
    nthreads = nthreads or os.cpu_count()
    R = np.float64 if fp64 else np.float32
    ct = C.c_double if fp64 else C.c_float
    g = np.zeros((pb.nx, pb.nz), R)
    fw = np.zeros_like(g)
    bk = np.zeros_like(g)
    adj_seis = np.zeros((pb.ns, pb.ngmax, pb.nt), R) if record_adjoint else None
    fn = lib().oracle_adjoint_f64 if fp64 else lib().oracle_adjoint_f32
    vp, rho, src, adj = _f32(vp), _f32(rho), _f32(src), _f32(adj)
    bnd = np.ascontiguousarray(fwd["boundary"], R)
    pe, ue, we = (np.ascontiguousarray(fwd[k], R) for k in ("p_end", "u_end", "w_end"))
    d = pb.desc()
    rc = fn(C.byref(d), _p(vp), _p(rho), _p(src), _p(adj), _p(bnd, ct), _p(pe, ct), _p(ue, ct), _p(we, ct),
            _p(g, ct), _p(fw, ct), _p(bk, ct), _p(adj_seis, ct), C.c_int(nthreads))
    _check(rc, "adjoint")
    out = dict(g=g, fw=fw, bk=bk)
    if record_adjoint:
        out["adj_seis"] = adj_seis
    return out


def gradient(pb: Problem, vp, rho, src, obs, fp64=False, return_seis=False, nthreads=None):
    """Waveform-misfit shot-gradient of every shot (forward + syn-obs + reverse loop)."""
    nthreads = nthreads or os.cpu_count()
    R = np.float64 if fp64 else np.float32
    ct = C.c_double if fp64 else C.c_float
    g = np.zeros((pb.nx, pb.nz), R)
    fw = np.zeros_like(g)
    bk = np.zeros_like(g)
    seis = np.zeros((pb.ns, pb.ngmax, pb.nt), R) if return_seis else None
    fn = lib().oracle_gradient_f64 if fp64 else lib().oracle_gradient_f32
    vp, rho, src, obs = _f32(vp), _f32(rho), _f32(src), _f32(obs)
    d = pb.desc()
    rc = fn(C.byref(d), _p(vp), _p(rho), _p(src), _p(obs), _p(g, ct), _p(fw, ct), _p(bk, ct), _p(seis, ct),
            C.c_int(nthreads))
    _check(rc, "gradient")
    out = dict(g=g, fw=fw, bk=bk)
    if return_seis:
        out["seis"] = seis
    return out


def exact(pb: Problem, vp, rho, src, adj, fp64=False, nthreads=None):
    """Exact discrete adjoint of the forward map (oracle_exact_*): the forward
    of every shot, then the transpose of its recursion for adjoint sources adj
    (ns, ngmax, nt).  Returns dict(g = dJ/dvp (nx, nz), gsrc = dJ/dsrc (ns, nt),
    seis)."""
    nthreads = nthreads or os.cpu_count()
    R = np.float64 if fp64 else np.float32
    ct = C.c_double if fp64 else C.c_float
    g = np.zeros((pb.nx, pb.nz), R)
    gsrc = np.zeros((pb.ns, pb.nt), R)
    seis = np.zeros((pb.ns, pb.ngmax, pb.nt), R)
    fn = lib().oracle_exact_f64 if fp64 else lib().oracle_exact_f32
    vp, rho, src, adj = _f32(vp), _f32(rho), _f32(src), _f32(adj)
    d = pb.desc()
    rc = fn(C.byref(d), _p(vp), _p(rho), _p(src), _p(adj), _p(g, ct), _p(gsrc, ct), _p(seis, ct), C.c_int(nthreads))
    _check(rc, "exact")
    return dict(g=g, gsrc=gsrc, seis=seis)


def damp_profile(pb: Problem, vp, rho):
    NX, NZ = pb.nx + 2 * pb.npml, pb.nz + 2 * pb.npml
    out = np.zeros((NX, NZ), np.float32)
    vp, rho = _f32(vp), _f32(rho)
    d = pb.desc()
    _check(lib().oracle_damp_profile_f32(C.byref(d), _p(vp), _p(rho), _p(out)), "damp_profile")
    return out
