"""The fd2dmpi-compatible command line: parfile and coordinate semantics on the
CPU; the full forward / adjoint file round trip through the GPU engine against
the oracle."""
import os
import types

import numpy as np
import pytest

from swit_gb300 import fd2dmpi, solver, suio, survey


def test_parfile_prefix_semantics(tmp_path):
    p = tmp_path / "par"
    p.write_text("# comment\nDATA_OUT=/w/data/syn/src\nNX=481\nNZ=141\nDX=25.000000\nNXX=7\n")
    assert fd2dmpi.read_par(str(p), "NX") == "481"           # first line starting with NX
    assert fd2dmpi.read_par(str(p), "DATA") == "OUT=/w/data/syn/src"  # plain prefix test, as parser.f90
    assert fd2dmpi.read_par(str(p), "NPML", "40") == "40"   # io.f90 default
    lines = "".join("X%d=1\n" % i for i in range(1000)) + "NPML=12\n"
    p.write_text(lines)
    assert fd2dmpi.read_par(str(p), "NPML", "40") == "40"   # only the first 1000 lines


@pytest.mark.parametrize("line,comp", [("", "p"), ("DATA_COMP=p\n", "p"), ("DATA_COMP=vx\n", "vx"),
                                       ("DATA_COMP=vz\n", "vz"), ("DATA_COMP=pressure\n", "p")])
def test_data_comp_key_of_the_dev_solver(tmp_path, line, comp):
    """DATA_COMP (dev/solver/io.f90:77, default p) picks the recorded component by
    its first letters as dev/solver/fdcore.f90:155-177 does."""
    p = tmp_path / "par"
    p.write_text("NX=20\nNZ=10\nNT_WORK=50\nDX=10.0\nDT_WORK=0.001\n" + line)
    assert fd2dmpi.Job(str(p)).data_comp == comp


def test_unknown_data_comp_is_an_error(tmp_path):
    p = tmp_path / "par"
    p.write_text("NX=20\nNZ=10\nNT_WORK=50\nDX=10.0\nDT_WORK=0.001\nDATA_COMP=vy\n")
    with pytest.raises(ValueError):
        fd2dmpi.Job(str(p))


def test_coord_grouping(tmp_path):
    p = tmp_path / "coord.txt"
    src = np.array([[0.0, 25.0], [100.0, 25.0]])
    rec = np.array([[[0.0, 25.0], [25.0, 25.0], [50.0, 25.0]]] * 2)
    suio.write_coord(str(p), src, rec)
    s, r, ng = fd2dmpi.read_coord(str(p))
    np.testing.assert_array_equal(s, src.astype(np.float32))
    np.testing.assert_array_equal(r, rec.astype(np.float32))
    assert list(ng) == [3, 3]


def test_non_zero_ranks_exit_without_work(tmp_path, monkeypatch):
    monkeypatch.setenv("OMPI_COMM_WORLD_RANK", "3")
    assert fd2dmpi.main(["par=%s" % (tmp_path / "missing")]) == 0
    monkeypatch.setenv("OMPI_COMM_WORLD_RANK", "0")
    assert fd2dmpi.main(["par=%s" % (tmp_path / "missing")]) == 1


def _simu(home, s, vp):
    for d in ("data/obs", "data/syn", "parfile/forward_parfile", "parfile/forward_source",
              "parfile/adjoint_parfile", "parfile/adjoint_source", "parfile/model"):
        os.makedirs(home + d, exist_ok=True)
    wav = np.repeat(survey.ricker(s.nt, s.dt, s.f0)[None], s.ns, axis=0)
    model = types.SimpleNamespace(nx=s.nx, nz=s.nz, dx=s.dx, dt=s.dt, nt=s.nt, pml=s.npml, fs=True,
                                  vp=vp.astype(np.float64), rho=s.rho(vp).astype(np.float64), savestep=1)
    return types.SimpleNamespace(
        model=model, source=types.SimpleNamespace(n=s.ns, xz=s.src_xz.astype(np.float64), wavelet=wav, f0=s.f0),
        receiver=types.SimpleNamespace(n=s.ng, xz=s.rec_xz.astype(np.float64)),
        system=types.SimpleNamespace(homepath=home, mpiproc=1))


@pytest.mark.gpu
def test_forward_and_adjoint_jobs_through_files(tmp_path, monkeypatch):
    from oracle import oracle as O
    s = survey.small(nt=240)
    home = str(tmp_path) + "/"
    simu = _simu(home, s, s.vp_true)
    src = solver._integrate(simu.source.wavelet)
    solver.write_parfile(simu, "syn", src, savesnap=1)          # the toolbox's own files
    for i in range(s.ns):
        os.makedirs(home + "data/syn/src%d_snapshot" % (i + 1), exist_ok=True)
    monkeypatch.chdir(home)
    assert fd2dmpi.main(["par=" + home + "parfile/forward_parfile/parfile"]) == 0
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, suio.parfile_value("%f", s.dx), suio.parfile_value("%f", s.dt),
                   s.src_xz, s.rec_xz)
    src32 = src.astype(np.float32)
    rho = s.rho(s.vp_true)
    ref = O.forward(pb, s.vp_true, rho, src32, store=True)
    for i in range(s.ns):
        np.testing.assert_array_equal(suio.read_su(home + "data/syn/src%d_sg.su" % (i + 1))[1], ref["seis"][i])
        b = np.fromfile(home + "data/syn/src%d_snapshot/boundary.bin" % (i + 1), np.float32)
        np.testing.assert_array_equal(b.reshape(s.nt, -1), ref["boundary"][i])
    adj = np.random.default_rng(1).standard_normal((s.ns, s.ng, s.nt)).astype(np.float32)
    solver.write_parfile(simu, "adj", adj, savesnap=0)
    assert fd2dmpi.main(["par=" + home + "parfile/adjoint_parfile/parfile"]) == 0
    gref = O.adjoint(pb, s.vp_true, rho, src32, adj, ref)
    for name, k in (("kernel_vp", "g"), ("illum_forw", "fw"), ("illum_back", "bk")):
        got = np.fromfile(home + "data/syn/src0_%s.bin" % name, np.float32).reshape(s.nx, s.nz)
        np.testing.assert_array_equal(got, gref[k])
