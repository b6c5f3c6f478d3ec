"""CPU tests of the C-ABI library: it loads, exports every declared symbol,
validates its arguments before touching the GPU, and evaluates the reference's
damping profile in closed form."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from swit_gb300 import _lib, build, damp_profile, survey

HEADER = os.path.join(os.path.dirname(build.HERE), "include", "swit_gb300.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(swit_[a-z0-9_]+)\s*\(", txt)))


def declared_desc_fields():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    body = txt[txt.index("typedef struct swit_desc {"):txt.index("} swit_desc;")]
    out = []
    for decl in body.split("{", 1)[1].split(";"):
        if not decl.strip():
            continue
        head, *rest = decl.strip().split(",")
        out.append(re.findall(r"([a-z_][a-z0-9_]*)\s*$", head.strip())[0])
        out += [r.strip() for r in rest]
    return out


# The descriptor's fields in declaration order, as a caller's own binding lists them.
DESC_FIELDS = ["nx", "nz", "npml", "nt", "dx", "dt", "free_surface", "ns", "ng_max", "ng", "src_x", "src_z", "rec_x",
               "rec_z", "precision", "path", "shots_per_batch", "block_x", "kernel_variant", "checkpoint_every",
               "graph_branches", "adjoint_mode", "receiver_component"]


def test_swit_desc_fields_match_the_ctypes_binding():
    """The header's struct, the library binding and the field list a caller's
    binding uses agree in order (a missing field shifts every later one)."""
    fields = [f[0] for f in _lib.SwitDesc._fields_]
    assert declared_desc_fields() == fields == DESC_FIELDS


def declared_arity():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for name, args in re.findall(r"\b(swit_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", txt, flags=re.S):
        args = args.strip()
        out[name] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_binding_argument_counts_match_the_header():
    lib = _lib.load()
    arity = declared_arity()
    assert set(arity) == set(_lib.EXPORTS)
    for name, n in arity.items():
        argtypes = getattr(lib, name).argtypes
        if argtypes is not None:
            assert len(argtypes) == n, (name, len(argtypes), n)


def test_plain_c_client_compiles_links_and_gets_argument_errors(tmp_path):
    """tests/c_abi_client.c uses only include/swit_gb300.h: it compiles as C99,
    links against the engine library and, given a bad description, gets
    SWIT_E_ARG and a message without touching a GPU."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    libdir = os.path.dirname(_lib.load()._name)
    exe = str(tmp_path / "c_abi_client")
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c_abi_client.c")
    subprocess.run([cc, "-std=c99", "-O2", "-Wall", "-Werror", "-I", os.path.dirname(HEADER), src, "-o", exe,
                    "-L", libdir, "-lswit_gb300", "-Wl,-rpath," + libdir, "-lm"], check=True)
    out = subprocess.run([exe, "invalid"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "nx and nz must be >= 8" in out.stdout


@pytest.mark.gpu
def test_plain_c_client_runs_a_gradient(tmp_path):
    """The same C client, without arguments: create, set model, forward, and a
    Waveform-misfit gradient with host buffers, all through the C ABI."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    libdir = os.path.dirname(_lib.load()._name)
    exe = str(tmp_path / "c_abi_client")
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c_abi_client.c")
    subprocess.run([cc, "-std=c99", "-O2", "-I", os.path.dirname(HEADER), src, "-o", exe, "-L", libdir,
                    "-lswit_gb300", "-Wl,-rpath," + libdir, "-lm"], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("misfit ")


def test_library_builds_and_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_symbols()
    assert set(names) == set(_lib.EXPORTS), names
    for n in names:
        assert hasattr(lib, n), n


def _desc(s, **over):
    ng = np.full(s.ns, s.ng, np.int32)
    xs = np.ascontiguousarray(s.src_xz[:, 0])
    zs = np.ascontiguousarray(s.src_xz[:, 1])
    xg = np.ascontiguousarray(s.rec_xz[:, :, 0]).reshape(-1)
    zg = np.ascontiguousarray(s.rec_xz[:, :, 1]).reshape(-1)
    keep = [ng, xs, zs, xg, zg]
    f = dict(nx=s.nx, nz=s.nz, npml=s.npml, nt=s.nt, dx=s.dx, dt=s.dt, free_surface=1, ns=s.ns, ng_max=s.ng,
             ng=ng.ctypes.data, src_x=xs.ctypes.data, src_z=zs.ctypes.data, rec_x=xg.ctypes.data,
             rec_z=zg.ctypes.data, precision=0, path=0, shots_per_batch=0, block_x=0, kernel_variant=0)
    f.update(over)
    return _lib.SwitDesc(**f), keep


@pytest.mark.parametrize("over,code", [
    (dict(nx=4), _lib.SwitError), (dict(npml=1), _lib.SwitError), (dict(nt=1), _lib.SwitError),
    (dict(dx=0.0), _lib.SwitError), (dict(precision=3), _lib.SwitError),
    (dict(block_x=3, kernel_variant=1), _lib.SwitError), (dict(block_x=300, kernel_variant=2), _lib.SwitError),
    (dict(kernel_variant=7), _lib.SwitError), (dict(checkpoint_every=-1), _lib.SwitError),
    (dict(checkpoint_every=5, kernel_variant=1), _lib.SwitError),
    (dict(graph_branches=-1), _lib.SwitError), (dict(graph_branches=5), _lib.SwitError),
    (dict(adjoint_mode=2), _lib.SwitError), (dict(adjoint_mode=1, kernel_variant=1), _lib.SwitError),
    (dict(adjoint_mode=1, kernel_variant=6), _lib.SwitError),
    (dict(receiver_component=3), _lib.SwitError), (dict(receiver_component=1, kernel_variant=1), _lib.SwitError),
    (dict(receiver_component=2, kernel_variant=6), _lib.SwitError),
])
def test_create_rejects_bad_descriptions_before_any_gpu_work(over, code):
    lib = _lib.load()
    s = survey.small()
    d, keep = _desc(s, **over)
    h = C.c_void_p()
    rc = lib.swit_create(C.byref(d), C.byref(h))
    assert rc == -1
    assert lib.swit_last_error().decode()


@pytest.mark.parametrize("over,code,text", [
    (dict(precision=1), -1, "FP32 vec kernels"), (dict(path=1), -1, "FP32 vec kernels"),
    (dict(kernel_variant=1), -1, "FP32 vec kernels"), (dict(checkpoint_every=10), -1, "boundary saving"),
    (dict(adjoint_mode=1), -1, "FP32 vec kernels"), (dict(receiver_component=1), -1, "FP32 vec kernels"),
    (dict(nx=16400), -8, "16384 PML-grid columns"),
])
def test_multi_create_rejects_unsupported_problems_before_any_gpu_work(over, code, text):
    """A multi-instance engine runs FP32 vec kernels on the batched path with
    boundary saving; any other description, in any position, is refused with
    its index before an engine is created."""
    lib = _lib.load()
    s = survey.small()
    good, keep0 = _desc(s)
    bad, keep1 = _desc(s, **over)
    descs = (_lib.SwitDesc * 2)(good, bad)
    h = C.c_void_p()
    assert lib.swit_multi_create(descs, 2, C.byref(h)) == code
    msg = lib.swit_last_error().decode()
    assert "instance 1" in msg and text in msg, msg
    assert not h.value


def test_multi_create_rejects_an_empty_batch():
    lib = _lib.load()
    h = C.c_void_p()
    s = survey.small()
    d, keep = _desc(s)
    assert lib.swit_multi_create(None, 1, C.byref(h)) == -1
    assert lib.swit_multi_create(C.byref(d), 0, C.byref(h)) == -1
    assert lib.swit_multi_destroy(None) == 0


def test_create_rejects_receivers_outside_the_model():
    lib = _lib.load()
    s = survey.small()
    s.rec_xz = s.rec_xz.copy()
    s.rec_xz[1, 3, 0] = (s.nx + 5) * s.dx
    d, keep = _desc(s)
    h = C.c_void_p()
    assert lib.swit_create(C.byref(d), C.byref(h)) == -2
    assert "receiver 4 of shot 2" in lib.swit_last_error().decode()


def test_null_arguments_are_errors():
    lib = _lib.load()
    h = C.c_void_p()
    assert lib.swit_create(None, C.byref(h)) == -1
    assert lib.swit_set_model(None, None, None, 0, None) == -1
    assert lib.swit_forward(None, None, None, 1, 0, None) == -1
    assert lib.swit_destroy(None) == 0


@pytest.mark.parametrize("nx,nz,npml", [(48, 32, 10), (30, 17, 7), (201, 101, 40)])
def test_closed_form_damping_equals_reference_loops(nx, nz, npml):
    s = survey.small(nx=nx, nz=nz, npml=npml)
    vp = s.vp_true
    pb = O.Problem(nx, nz, npml, 10, s.dx, s.dt, s.src_xz, s.rec_xz)
    ref = O.damp_profile(pb, vp, s.rho(vp))
    # vmin below the free surface: rows 2..nz of the interior (math.f90:342-361)
    vmin = np.float32(vp[:, 1:].min())
    mine = damp_profile(nx, nz, npml, s.dx, vmin)
    np.testing.assert_array_equal(mine, ref)
