"""fd2dmpi-compatible command line on the GB300 engine.

    python -m swit_gb300.fd2dmpi par=<parfile>        (or swit_gb300/bin/fd2dmpi par=<parfile>)

reads the same parfile, coordinate file, model files and per-shot source files
as fd2dmpi (fd2dmpi/fd2dmpi.f90:16-34, io.f90:60-300, solver.f90:95, 213-228)
and writes the same outputs:

  jobtype=forward_modeling   <DATA_OUT>N_sg.su (or _sg.bin when FILEFORMAT is not su)
                             and, with STORE_SNAP=1, <DATA_OUT>N_snapshot/{boundary,p_end,
                             u_end,w_end}.bin                       (fdcore.f90:162-188)
  jobtype=adjoint_modeling   <DATA_OUT>0_kernel_vp.bin, 0_illum_forw.bin, 0_illum_back.bin
                                                                    (solver.f90:263-279)

so toolbox/solver.py runs unchanged with this program in place of fd2dmpi.
The dev solver's DATA_COMP key (p, vx or vz; dev/solver/io.f90:77) selects the
recorded component.
The adjoint job reads the saved strips and end states when they exist and
otherwise recomputes them on the GPU.  Under mpirun every rank but rank 0
exits at once: all shots run batched on one GPU.  The exit status is 0 on
success and 1 on failure (toolbox/solver.py:55-58 turns that into its
'solver crash' errors).
"""
import os
import sys

import numpy as np

from . import suio

NLINE = 1000  # fd2dmpi/parser.f90: only the first 1000 lines are searched


def read_par(path, key, default=None):
    """fd2dmpi/parser.f90 readParFile*: the first line that STARTS with `key`
    (a plain prefix test) gives the value, which begins one character after the key."""
    with open(path) as f:
        for i, line in enumerate(f):
            if i >= NLINE:
                break
            line = line.rstrip("\n")
            if line[:len(key)] == key:
                return line[len(key) + 1:].strip()
    return default


def read_coord(path):
    """fd2dmpi/io.f90:126-228: seven columns per line; a new shot starts where the
    source index changes.  Returns (src_xz (ns, 2), rec_xz (ns, ngmax, 2), ng (ns,))."""
    rows = []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 7:
                rows.append([float(x) for x in parts[:7]])
    if not rows:
        raise ValueError("coordinate file %s has no geometry" % path)
    shots = []
    for r in rows:
        if not shots or r[0] != shots[-1][0]:
            shots.append([r[0], []])
        shots[-1][1].append(r)
    ns = len(shots)
    ng = np.array([len(s[1]) for s in shots], np.int32)
    ngmax = int(ng.max())
    src = np.zeros((ns, 2), np.float32)
    rec = np.zeros((ns, ngmax, 2), np.float32)
    for i, (_, lines) in enumerate(shots):
        src[i] = (lines[-1][2], lines[-1][3])   # io.f90:206-207 keep the last line's source
        for j, r in enumerate(lines):
            rec[i, j] = (r[4], r[5])
        if len(lines) < ngmax:                  # padded receivers: any point inside the model
            rec[i, len(lines):] = rec[i, 0]
    return src, rec, ng


def _rank():
    for k in ("OMPI_COMM_WORLD_RANK", "PMI_RANK", "PMIX_RANK", "SLURM_PROCID"):
        if k in os.environ:
            return int(os.environ[k])
    return 0


class Job:
    """The parfile of one fd2dmpi run (fd2dmpi/io.f90:74-96 keys and defaults)."""

    def __init__(self, parfile):
        self.parfile = parfile
        self.jobtype = read_par(parfile, "jobtype", "")
        self.coordfile = read_par(parfile, "COORD_FILE", "n/a")
        self.data_out = read_par(parfile, "DATA_OUT", "src")
        self.velfile = read_par(parfile, "VEL_IN", "n/a")
        self.densityfile = read_par(parfile, "DENSITYFILE", "n/a")
        self.fileformat = read_par(parfile, "FILEFORMAT", "su")
        self.nx = int(read_par(parfile, "NX", "-1"))
        self.nz = int(read_par(parfile, "NZ", "-1"))
        self.nt = int(read_par(parfile, "NT_WORK", "-1"))
        self.free_surface = int(read_par(parfile, "FREESURFACE", "1"))
        self.npml = int(read_par(parfile, "NPML", "40"))
        self.store_snap = int(read_par(parfile, "STORE_SNAP", "0"))
        # the dev solver's recorded component (dev/solver/io.f90:77, fdcore.f90:155-177): p, vx or vz
        comp = read_par(parfile, "DATA_COMP", "p")
        if comp[:1] == "p":
            self.data_comp = "p"
        elif comp[:2] in ("vx", "vz"):
            self.data_comp = comp[:2]
        else:
            raise ValueError("data comp not recognized: %s" % comp)
        self.dx = np.float32(float(read_par(parfile, "DX", "-1.0")))
        self.dt = np.float32(float(read_par(parfile, "DT_WORK", "-1.0")))
        if self.nx <= 0 or self.nz <= 0 or self.nt <= 0 or self.dx <= 0 or self.dt <= 0:
            raise ValueError("parfile %s lacks NX, NZ, NT_WORK, DX or DT_WORK" % parfile)

    def out(self, num, suffix):
        return "%s%d%s" % (self.data_out, num, suffix)  # fd2dmpi/string.f90 filename()


def _engine(job, src_xz, rec_xz, ng):
    from .engine import Engine
    return Engine(job.nx, job.nz, job.npml, job.nt, float(job.dx), float(job.dt), src_xz, rec_xz,
                  free_surface=job.free_surface, ng=ng, receiver_component=job.data_comp)


def _model(job):
    n = job.nx * job.nz
    vp = np.fromfile(job.velfile, np.float32, count=n).reshape(job.nx, job.nz)
    rho = np.fromfile(job.densityfile, np.float32, count=n).reshape(job.nx, job.nz)
    return vp, rho


def _sources(job, ns, folder):
    return np.stack([np.fromfile("./parfile/%s/src%d.bin" % (folder, i + 1), np.float32, count=job.nt)
                     for i in range(ns)])


def forward_modeling(job):
    """jobtype=forward_modeling (fd2dmpi/solver.f90:36-116): seismograms, and strips with STORE_SNAP=1."""
    src_xz, rec_xz, ng = read_coord(job.coordfile)
    ns = src_xz.shape[0]
    vp, rho = _model(job)
    src = _sources(job, ns, "forward_source")
    for i in range(ns):
        print(" Process 0, shot %d source max value = %g" % (i + 1, float(src[i].max())), flush=True)
    with _engine(job, src_xz, rec_xz, ng) as e:
        e.set_model(vp, rho)
        seis = e.forward(src, save_boundary=job.store_snap == 1)
        snap = e.export_snapshot() if job.store_snap == 1 else None
    for i in range(ns):
        traces = seis[i, :ng[i]]
        if job.fileformat[:2] == "su":
            suio.write_su(job.out(i + 1, "_sg.su"), traces, job.dt, src_xz[i, 0], rec_xz[i, :ng[i], 0])
        else:
            suio.save_bin(job.out(i + 1, "_sg.bin"), traces)
        if snap is not None:
            d = job.out(i + 1, "_snapshot/")
            suio.ensure_dir(d)
            for k in ("boundary", "p_end", "u_end", "w_end"):
                suio.save_bin(d + k + ".bin", snap[k][i])


def adjoint_modeling(job):
    """jobtype=adjoint_modeling (fd2dmpi/solver.f90:120-289): vp kernel and illuminations."""
    src_xz, rec_xz, ng = read_coord(job.coordfile)
    ns, ngmax = src_xz.shape[0], rec_xz.shape[1]
    vp, rho = _model(job)
    src = _sources(job, ns, "forward_source")
    adj = np.zeros((ns, ngmax, job.nt), np.float32)
    for i in range(ns):
        a = np.fromfile("./parfile/adjoint_source/src%d.bin" % (i + 1), np.float32)
        a = a[:(a.size // job.nt) * job.nt].reshape(-1, job.nt)
        adj[i, :min(a.shape[0], ng[i])] = a[:ng[i]]
    S = 9 * job.nx + 6 * job.nz
    names = ("boundary", "p_end", "u_end", "w_end")
    files = [[job.out(i + 1, "_snapshot/%s.bin" % k) for k in names] for i in range(ns)]
    have = all(os.path.exists(f) for fs in files for f in fs)
    with _engine(job, src_xz, rec_xz, ng) as e:
        e.set_model(vp, rho)
        if have:
            b = np.stack([np.fromfile(f[0], np.float32, count=job.nt * S).reshape(job.nt, S) for f in files])
            ends = [np.stack([np.fromfile(f[q], np.float32, count=job.nx * job.nz).reshape(job.nx, job.nz)
                              for f in files]) for q in (1, 2, 3)]
            e.import_snapshot(src, b, *ends)
        else:
            print(" no saved boundary strips: recomputing the forward run", flush=True)
            e.forward(src, save_boundary=True)
        g, fw, bk = e.backward(adj)
    suio.save_bin(job.out(0, "_kernel_vp.bin"), g)
    suio.save_bin(job.out(0, "_illum_forw.bin"), fw)
    suio.save_bin(job.out(0, "_illum_back.bin"), bk)


def main(argv=None):
    """fd2dmpi par=<parfile> (fd2dmpi/fd2dmpi.f90:16-34); returns the exit status."""
    argv = sys.argv[1:] if argv is None else argv
    parfile = "fdparfile"  # fd2dmpi.f90:22 default of readCmd('par', ...)
    for a in argv:
        if a.startswith("par="):
            parfile = a[4:]
    if _rank() != 0:
        return 0
    try:
        job = Job(parfile)
        if job.jobtype[:16] == "forward_modeling":
            print(" Forward modeling ---- time-domain staggered-42-FD (GB300)", flush=True)
            forward_modeling(job)
        elif job.jobtype[:16] == "adjoint_modeling":
            print(" Adjoint modeling ---- time-domain staggered-42-FD (GB300)", flush=True)
            adjoint_modeling(job)
        else:
            print(" unknown jobtype %r in %s" % (job.jobtype, parfile), file=sys.stderr)
            return 1
    except Exception as err:  # the toolbox only sees the exit status
        print(" fd2dmpi (GB300) failed: %s" % err, file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
