"""File formats of the fd2dmpi contract: SU seismograms, raw float32 binaries,
the parfile and coord.txt.

write_su() produces the bytes fd2dmpi's write_sufile_2d_coord writes
(fd2dmpi/io.f90:522-571): per trace a 240-byte SU header (fd2dmpi/su.f90,
nhead = 60 words, native byte order) followed by nt float32 samples, with
  ns = nt, ep = 1, fldr = 1, dt = int(dt * 1e6) microseconds, d1 = dt, d2 = 1,
  f1 = 0, f2 = 1, tracl = tracr = trace number, sx = nint(xs), gx = nint(xg),
  cdp = cdpt = nint(0.5 (xs + xg)), offset = gx - sx
and every other field zero (clean_suheader, io.f90:690-774).  read_su() reads it
back without obspy.
"""
import os

import numpy as np

# 240-byte SU trace header: the field order and widths of fd2dmpi/su.f90
_HDR = np.dtype([
    ("tracl", "<i4"), ("tracr", "<i4"), ("fldr", "<i4"), ("tracf", "<i4"), ("ep", "<i4"), ("cdp", "<i4"),
    ("cdpt", "<i4"), ("trid", "<i2"), ("nvs", "<i2"), ("nhs", "<i2"), ("duse", "<i2"), ("offset", "<i4"),
    ("gelev", "<i4"), ("selev", "<i4"), ("sdepth", "<i4"), ("gdel", "<i4"), ("sdel", "<i4"), ("swdep", "<i4"),
    ("gwdep", "<i4"), ("scalel", "<i2"), ("scalco", "<i2"), ("sx", "<i4"), ("sy", "<i4"), ("gx", "<i4"),
    ("gy", "<i4"), ("counit", "<i2"), ("wevel", "<i2"), ("swevel", "<i2"), ("sut", "<i2"), ("gut", "<i2"),
    ("sstat", "<i2"), ("gstat", "<i2"), ("tstat", "<i2"), ("laga", "<i2"), ("lagb", "<i2"), ("delrt", "<i2"),
    ("muts", "<i2"), ("mute", "<i2"), ("ns", "<u2"), ("dt", "<u2"), ("gain", "<i2"), ("igc", "<i2"),
    ("igi", "<i2"), ("corr", "<i2"), ("sfs", "<i2"), ("sfe", "<i2"), ("slen", "<i2"), ("styp", "<i2"),
    ("stas", "<i2"), ("stae", "<i2"), ("tatyp", "<i2"), ("afilf", "<i2"), ("afils", "<i2"), ("nofilf", "<i2"),
    ("nofils", "<i2"), ("lcf", "<i2"), ("hcf", "<i2"), ("lcs", "<i2"), ("hcs", "<i2"), ("year", "<i2"),
    ("day", "<i2"), ("hour", "<i2"), ("minute", "<i2"), ("sec", "<i2"), ("timbas", "<i2"), ("trwf", "<i2"),
    ("grnors", "<i2"), ("grnofr", "<i2"), ("grnlof", "<i2"), ("gaps", "<i2"), ("otrav", "<i2"),
    ("d1", "<f4"), ("f1", "<f4"), ("d2", "<f4"), ("f2", "<f4"), ("ungpow", "<f4"), ("unscale", "<f4"),
    ("mark", "<i2"), ("unass", "<i2", (17,))])
assert _HDR.itemsize == 240


def fortran_nint(x):
    """Fortran NINT on float32 values: round half away from zero."""
    x = np.asarray(x, np.float32)
    return np.where(x >= 0, np.floor(x + np.float32(0.5)), np.ceil(x - np.float32(0.5))).astype(np.int64)


def su_headers(nt, dt, xs, xg):
    """Headers of one shot gather (fd2dmpi/io.f90:522-571)."""
    xg = np.asarray(xg, np.float32)
    xs32 = np.float32(xs)
    n2 = xg.shape[0]
    h = np.zeros(n2, _HDR)
    h["tracl"] = np.arange(1, n2 + 1)
    h["tracr"] = np.arange(1, n2 + 1)
    h["fldr"] = 1
    h["ep"] = 1
    h["ns"] = np.uint16(nt & 0xFFFF)
    h["dt"] = np.uint16(int(np.float32(dt) * np.float32(1.0e6)) & 0xFFFF)
    h["d1"] = np.float32(dt)
    h["d2"] = np.float32(1.0)
    h["f1"] = np.float32(0.0)
    h["f2"] = np.float32(1.0)
    sx = int(fortran_nint(xs32))
    h["sx"] = sx
    gx = fortran_nint(xg)
    h["gx"] = gx
    cdp = fortran_nint(np.float32(0.5) * (xs32 + xg))
    h["cdp"] = cdp
    h["cdpt"] = cdp
    h["offset"] = gx - sx
    return h


def write_su(path, traces, dt, xs, xg):
    """traces (ng, nt) float32 -> SU file, byte-compatible with fd2dmpi."""
    traces = np.ascontiguousarray(traces, np.float32)
    n2, nt = traces.shape
    rec = np.zeros(n2, np.dtype([("h", _HDR), ("d", "<f4", (nt,))]))
    rec["h"] = su_headers(nt, dt, xs, xg)
    rec["d"] = traces
    with open(path, "wb") as f:
        rec.tofile(f)


def read_su(path, nt=None):
    """Reads an SU file written by write_su / fd2dmpi: returns (headers, traces (ng, nt))."""
    raw = np.fromfile(path, np.uint8)
    if nt is None:
        nt = int(raw[:240].view(_HDR)["ns"][0])
    rec = raw.view(np.dtype([("h", _HDR), ("d", "<f4", (nt,))]))
    return rec["h"].copy(), rec["d"].copy()


def save_bin(path, a):
    """toolbox/tools.py:72-77: raw float32, C order."""
    np.asarray(a, np.float32).tofile(path)


def load_bin(path):
    return np.fromfile(path, np.float32)


def parfile_value(fmt, v):
    """The float32 value fd2dmpi parses from a parfile or coord.txt field written
    with the given printf format (toolbox/solver.py:145-148, 178)."""
    return np.float32(float(fmt % v))


def write_parfile(path, jobtype, homepath, simu_type, nx, nz, dx, npml, nt, dt, fs, savesnap, savestep):
    """toolbox/solver.py:121-155, the same keys and formats."""
    out = "data/obs/src" if simu_type == "obs" else "data/syn/src"
    with open(path, "w") as fp:
        fp.write("######################################### \n")
        fp.write("#                                         \n")
        fp.write("#     fd2dmpi input parameter file        \n")
        fp.write("#                                         \n")
        fp.write("######################################### \n")
        fp.write("                                          \n")
        fp.write("jobtype=%s\n" % jobtype)
        fp.write("COORD_FILE=%s\n" % (homepath + "parfile/model/coord.txt"))
        fp.write("DATA_OUT=%s\n" % (homepath + out))
        fp.write("VEL_IN=%s\n" % (homepath + "parfile/model/vel.bin"))
        fp.write("DENSITYFILE=%s\n" % (homepath + "parfile/model/rho.bin"))
        fp.write("FILEFORMAT=su\n")
        fp.write("NX=%d\n" % nx)
        fp.write("NZ=%d\n" % nz)
        fp.write("DX=%f\n" % dx)
        fp.write("NPML=%d\n" % npml)
        fp.write("NT_WORK=%d\n" % nt)
        fp.write("DT_WORK=%f\n" % dt)
        fp.write("FREESURFACE=%d\n" % (1 if fs else 0))
        fp.write("STORE_SNAP=%d\n" % savesnap)
        fp.write("STORE_STEP=%d\n" % savestep)


def write_coord(path, src_xz, rec_xz):
    """toolbox/solver.py:166-180: '%6i %6i %10.1f %10.1f %10.1f %10.1f %10.1f' per source-receiver pair."""
    with open(path, "w") as fp:
        for isrc in range(src_xz.shape[0]):
            for irec in range(rec_xz.shape[1]):
                fp.write("%6i %6i %10.1f %10.1f %10.1f %10.1f %10.1f\n" % (
                    isrc + 1, irec + 1, src_xz[isrc, 0], src_xz[isrc, 1], rec_xz[isrc, irec, 0],
                    rec_xz[isrc, irec, 1], 1))


def read_parfile(path):
    """KEY=value pairs of the first 1000 lines (fd2dmpi/parser.f90); '#' lines skipped."""
    out = {}
    with open(path) as f:
        for i, line in enumerate(f):
            if i >= 1000:
                break
            line = line.strip()
            if not line or line.startswith("#") or "=" not in line:
                continue
            k, v = line.split("=", 1)
            out.setdefault(k.strip(), v.strip())
    return out


def ensure_dir(path):
    os.makedirs(path, exist_ok=True)
