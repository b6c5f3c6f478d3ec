"""Drop-in for SWIT's toolbox/solver.py: forward() and adjoint() with the same
signatures, arguments and file side effects, computed by the GB300 engine
instead of `mpirun fd2dmpi` (toolbox/solver.py:54 and :79).

    forward(simu, simu_type='obs', savesnap=0)   toolbox/solver.py:24-58
    adjoint(simu, optim)                         toolbox/solver.py:61-92
    write_parfile(simu, simu_type, src, savesnap) toolbox/solver.py:95-180
    source_wavelet(nt, dt, f0, srctype)          toolbox/solver.py:183-197

forward() writes homepath/data/{obs,syn}/srcN_sg.su (N = 1..ns) exactly as
fd2dmpi does and, like the reference, the parfile, model, source and geometry
files.  With savesnap=1 the boundary strips and final wavefields stay in device
memory for the following adjoint(); they are written to
data/syn/srcN_snapshot/{boundary,p_end,u_end,w_end}.bin only when the
environment variable SWIT_GB300_WRITE_SNAPSHOTS=1 is set, because only
fd2dmpi's adjoint job reads those files.  adjoint() computes the adjoint
sources with the toolbox's own misfit.adjoint_source, runs the reverse loop,
writes data/syn/src0_kernel_vp.bin, src0_illum_forw.bin and
src0_illum_back.bin, and returns the toolbox's grad_precond of them.

Numbers reach the engine exactly as fd2dmpi would read them from the files:
DX and DT_WORK through '%f', coordinates through '%10.1f', the source through
float32 (toolbox/solver.py:113, 145-148, 178).

Errors: an engine failure raises ValueError('Forward solver crash') or
ValueError('Adjoint solver crash') like toolbox/solver.py:56-58 and :81-82,
chained to the engine's SwitError.
"""
import hashlib
import os

import numpy as np
from scipy import integrate

from . import suio
from ._lib import SwitError
from .engine import Engine

_cache = {"key": None, "engine": None, "state": None}


def source_wavelet(nt, dt, f0, srctype):
    """toolbox/solver.py:183-197."""
    t = np.linspace(0, dt * nt, num=nt, endpoint=False)
    if srctype.lower() in ["ricker"]:
        t0 = 1.2 / f0
        temp = (np.pi * f0) ** 2
        return (1 - 2 * temp * (t - t0) ** 2) * np.exp(- temp * (t - t0) ** 2)
    raise ValueError('Other wavelets can be implemented here.')


def _integrate(wavelet):
    # toolbox/solver.py:47 calls integrate.cumtrapz, renamed cumulative_trapezoid
    return integrate.cumulative_trapezoid(wavelet, axis=-1, initial=0)


def _geometry(simu):
    """Acquisition as fd2dmpi parses it from coord.txt (float32 of '%10.1f')."""
    src = np.asarray(simu.source.xz, np.float64).reshape(-1, 2)
    rec = np.asarray(simu.receiver.xz, np.float64)
    if rec.ndim == 2:
        rec = np.broadcast_to(rec, (src.shape[0],) + rec.shape)
    f = np.vectorize(lambda v: float("%10.1f" % v))
    return f(src).astype(np.float32), f(rec).astype(np.float32)


def _engine_for(simu):
    m = simu.model
    dx = suio.parfile_value("%f", m.dx)
    dt = suio.parfile_value("%f", m.dt)
    src_xz, rec_xz = _geometry(simu)
    key = (int(m.nx), int(m.nz), int(m.pml), int(m.nt), float(dx), float(dt), bool(m.fs),
           hashlib.sha1(src_xz.tobytes() + rec_xz.tobytes()).hexdigest())
    if _cache["key"] != key:
        if _cache["engine"] is not None:
            _cache["engine"].close()
        _cache["engine"] = Engine(int(m.nx), int(m.nz), int(m.pml), int(m.nt), dx, dt, src_xz, rec_xz,
                                  free_surface=1 if m.fs else 0)
        _cache["key"] = key
        _cache["state"] = None
    return _cache["engine"], src_xz, rec_xz


def write_parfile(simu, simu_type, src, savesnap=0):
    """toolbox/solver.py:95-180: parfile, vel.bin, rho.bin, coord.txt and the
    per-shot source files, with the same names and formats."""
    path = simu.system.homepath
    if simu_type in ['obs', 'syn']:
        parpath = path + 'parfile/forward_parfile/parfile'
        srcpath = path + 'parfile/forward_source/'
        job = 'forward_modeling'
    elif simu_type in ['adj']:
        parpath = path + 'parfile/adjoint_parfile/parfile'
        srcpath = path + 'parfile/adjoint_source/'
        job = 'adjoint_modeling'
    else:
        raise ValueError('write_parfile: unsupported simulation type %s' % simu_type)
    for d in (os.path.dirname(parpath), srcpath, path + 'parfile/model/'):
        suio.ensure_dir(d)
    for isrc in range(simu.source.n):
        suio.save_bin(srcpath + 'src%d.bin' % (isrc + 1), src[isrc, :])
    suio.save_bin(path + 'parfile/model/vel.bin', simu.model.vp)
    suio.save_bin(path + 'parfile/model/rho.bin', simu.model.rho)
    m = simu.model
    suio.write_parfile(parpath, job, path, simu_type if simu_type != 'adj' else 'syn', m.nx, m.nz, m.dx, m.pml,
                       m.nt, m.dt, m.fs, savesnap, m.savestep)
    src_xz = np.asarray(simu.source.xz, np.float64).reshape(-1, 2)
    rec_xz = np.asarray(simu.receiver.xz, np.float64)
    if rec_xz.ndim == 2:
        rec_xz = np.broadcast_to(rec_xz, (src_xz.shape[0],) + rec_xz.shape)
    suio.write_coord(path + 'parfile/model/coord.txt', src_xz, rec_xz)


def _model32(simu):
    vp = np.ascontiguousarray(simu.model.vp, np.float32)
    rho = np.ascontiguousarray(simu.model.rho, np.float32)
    return vp, rho


def forward(simu, simu_type='obs', savesnap=0):
    """forward solver (toolbox/solver.py:24-58) on the GB300 engine."""
    if simu_type not in ['obs', 'syn']:
        raise ValueError('Forward: unsupport simulation tyep.')
    homepath = simu.system.homepath
    srcn = simu.source.n
    outdir = homepath + 'data/%s/' % simu_type
    if simu_type in ['syn']:
        _clean(outdir)
    suio.ensure_dir(outdir)
    src = _integrate(simu.source.wavelet)
    write_parfile(simu, simu_type, src, savesnap=savesnap)
    src32 = np.ascontiguousarray(src, np.float32)
    try:
        eng, src_xz, rec_xz = _engine_for(simu)
        vp, rho = _model32(simu)
        eng.set_model(vp, rho)
        seis = eng.forward(src32, save_boundary=bool(savesnap))
    except SwitError as err:
        print(str(err))
        raise ValueError('Forward solver crash') from err
    dt32 = suio.parfile_value("%f", simu.model.dt)
    for isrc in range(srcn):
        suio.write_su(outdir + 'src%d_sg.su' % (isrc + 1), seis[isrc], dt32, src_xz[isrc, 0], rec_xz[isrc, :, 0])
    if savesnap:
        _cache["state"] = dict(vp=vp.copy(), rho=rho.copy(), src=src32.copy())
        if os.environ.get("SWIT_GB300_WRITE_SNAPSHOTS") == "1":
            snap = eng.export_snapshot()
            for isrc in range(srcn):
                d = outdir + 'src%d_snapshot/' % (isrc + 1)
                suio.ensure_dir(d)
                for k in ("boundary", "p_end", "u_end", "w_end"):
                    suio.save_bin(d + k + '.bin', snap[k][isrc])
    else:
        _cache["state"] = None


def _clean(folder):
    """toolbox/tools.py cleandata: empty the folder, keep it."""
    if os.path.isdir(folder):
        for name in os.listdir(folder):
            p = os.path.join(folder, name)
            if os.path.isdir(p):
                for root, dirs, files in os.walk(p, topdown=False):
                    for f in files:
                        os.remove(os.path.join(root, f))
                    for d in dirs:
                        os.rmdir(os.path.join(root, d))
                os.rmdir(p)
            else:
                os.remove(p)


def adjoint(simu, optim, adjoint_source=None, grad_precond=None):
    """adjoint solver (toolbox/solver.py:61-92) on the GB300 engine.

    adjoint_source / grad_precond default to the toolbox's own
    misfit.adjoint_source and postprocess.grad_precond.
    """
    if adjoint_source is None:
        from misfit import adjoint_source  # the toolbox module (toolbox/misfit.py:74-88)
    if grad_precond is None:
        from postprocess import grad_precond  # toolbox/postprocess.py:20-85
    homepath = simu.system.homepath
    src_adj = np.asarray(adjoint_source(simu, optim.misfit_type))
    write_parfile(simu, 'adj', src_adj, savesnap=0)
    try:
        eng, _, _ = _engine_for(simu)
        vp, rho = _model32(simu)
        st = _cache["state"]
        src = np.ascontiguousarray(_integrate(simu.source.wavelet), np.float32)
        if st is None or not (np.array_equal(st["vp"], vp) and np.array_equal(st["rho"], rho)
                              and np.array_equal(st["src"], src)):
            # no strips from a matching forward(savesnap=1) in this process:
            # recompute them (identical to what fd2dmpi reads back from disk)
            eng.set_model(vp, rho)
            eng.forward(src, save_boundary=True)
            _cache["state"] = dict(vp=vp.copy(), rho=rho.copy(), src=src.copy())
        adj = np.zeros((eng.ns, eng.ngmax, eng.nt), np.float32)
        adj[:, :src_adj.shape[1], :] = src_adj.astype(np.float32)
        grad, forw, back = eng.backward(adj)
    except SwitError as err:
        raise ValueError('Adjoint solver crash') from err
    suio.ensure_dir(homepath + 'data/syn/')
    suio.save_bin(homepath + 'data/syn/src0_kernel_vp.bin', grad)
    suio.save_bin(homepath + 'data/syn/src0_illum_forw.bin', forw)
    suio.save_bin(homepath + 'data/syn/src0_illum_back.bin', back)
    grad = suio.load_bin(homepath + 'data/syn/src0_kernel_vp.bin')
    forw = suio.load_bin(homepath + 'data/syn/src0_illum_forw.bin')
    back = suio.load_bin(homepath + 'data/syn/src0_illum_back.bin')
    return grad_precond(simu, optim, grad, forw, back)
