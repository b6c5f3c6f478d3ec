"""CPU tests of the host-side file contract (SU header layout and values,
parfile and coord.txt formats) and of the Python engine's argument handling."""
import numpy as np
import pytest

from swit_gb300 import suio


def test_su_header_is_240_bytes_with_the_documented_byte_positions(tmp_path):
    # byte positions documented in fd2dmpi/su.f90 (1-based, SEG-Y/SU convention)
    pos = {"tracl": 1, "cdp": 21, "offset": 37, "sx": 73, "gx": 81, "ns": 115, "dt": 117, "d1": 181, "d2": 189,
           "f2": 193, "mark": 205, "unass": 207}
    for k, p in pos.items():
        assert suio._HDR.fields[k][1] == p - 1, k
    tr = np.arange(3 * 7, dtype=np.float32).reshape(3, 7)
    path = tmp_path / "s.su"
    suio.write_su(str(path), tr, 0.002, 1000.0, np.array([0.0, 25.0, 1012.5], np.float32))
    raw = path.read_bytes()
    assert len(raw) == 3 * (240 + 7 * 4)
    h, d = suio.read_su(str(path))
    np.testing.assert_array_equal(d, tr)
    assert list(h["tracl"]) == [1, 2, 3] and list(h["tracr"]) == [1, 2, 3]
    assert set(h["ns"]) == {7} and set(h["dt"]) == {2000} and set(h["fldr"]) == {1} and set(h["ep"]) == {1}
    assert list(h["gx"]) == [0, 25, 1013]           # NINT rounds half away from zero
    assert list(h["sx"]) == [1000] * 3
    assert list(h["offset"]) == [-1000, -975, 13]
    assert list(h["cdp"]) == [500, 513, 1006]       # nint(0.5 (xs + xg)) in single precision
    assert list(h["cdpt"]) == list(h["cdp"])
    assert np.allclose(h["d1"], 0.002) and set(h["d2"]) == {1.0} and set(h["f1"]) == {0.0}
    assert not np.any(h["unass"]) and not np.any(h["trid"])


def test_su_dt_is_truncated_in_single_precision():
    for dt, us in ((0.002, 2000), (0.001, 1000), (0.0015, 1500), (0.0005, 500)):
        h = suio.su_headers(10, dt, 0.0, np.zeros(1, np.float32))
        assert h["dt"][0] == us


def test_parfile_and_coord_formats(tmp_path):
    p = tmp_path / "parfile"
    suio.write_parfile(str(p), "forward_modeling", "/w/", "syn", 481, 141, 25.0, 40, 4000, 0.002, True, 1, 1)
    kv = suio.read_parfile(str(p))
    assert kv["jobtype"] == "forward_modeling" and kv["DATA_OUT"] == "/w/data/syn/src"
    assert kv["DX"] == "25.000000" and kv["DT_WORK"] == "0.002000" and kv["FREESURFACE"] == "1"
    assert kv["NX"] == "481" and kv["NPML"] == "40" and kv["STORE_SNAP"] == "1"
    c = tmp_path / "coord.txt"
    src = np.array([[0.0, 25.0], [12.34, 25.0]])
    rec = np.array([[[0.0, 25.0], [25.0, 25.0]], [[0.0, 25.0], [25.0, 25.0]]])
    suio.write_coord(str(c), src, rec)
    lines = c.read_text().splitlines()
    assert lines[0] == "     1      1        0.0       25.0        0.0       25.0        1.0"
    assert lines[2].split()[2] == "12.3"
    assert suio.parfile_value("%10.1f", 12.34) == np.float32(12.3)


def test_checkpoint_interval_keeps_boundary_saving_when_it_fits():
    from swit_gb300.engine import checkpoint_interval
    # 481 x 141, 49 shots, nt 4000: 4 GB of strips
    assert checkpoint_interval(481, 141, 40, 4000, 49, 150e9) == 0
    # 2001 x 601 (npml 60), 200 shots, nt 6000: 104 GB of strips + 53 GB of fields and trace staging exceed
    # a 150 GB budget (the engine measured 157 GB on the GPU)
    k = checkpoint_interval(2001, 601, 60, 6000, 200, 150e9)
    assert 1 <= k < 6000
    NX, LD, sl = 2121, 736, 9 * 2001 + 6 * 601
    mem = 200 * (-(-6000 // k) * 3 * NX * LD + k * sl) * 4
    assert mem < 200 * 6000 * sl * 4 / 2  # well under boundary saving


def test_checkpoint_interval_of_the_exact_adjoint():
    """An exact-adjoint engine stores a whole divergence field per step (98.5 GB at
    481 x 141, 49 shots, nt 4000): it fits 150 GB, not 50 GB, where the interval
    that minimises checkpoints + records is about sqrt(3 nt)."""
    from swit_gb300.engine import checkpoint_interval
    assert checkpoint_interval(481, 141, 40, 4000, 49, 150e9, exact=True) == 0
    k = checkpoint_interval(481, 141, 40, 4000, 49, 50e9, exact=True)
    assert 80 <= k <= 140
    assert checkpoint_interval(481, 141, 40, 4000, 49, 50e9) == 0  # fd2dmpi's strips: 4 GB


@pytest.mark.parametrize("kw", [dict(precision="fp16"), dict(path="fast"), dict(adjoint="approx"),
                                dict(receiver_component="vy"), dict(kernel="tensor")])
def test_engine_rejects_unknown_options_before_any_gpu_work(kw):
    from swit_gb300 import Engine, survey
    s = survey.small()
    with pytest.raises(ValueError):
        Engine(**s.engine_args(), **kw)


@pytest.mark.parametrize("kw", [dict(precision="fp64"), dict(path="plain"), dict(checkpoint_every=100)])
def test_multi_engine_refuses_problems_it_cannot_batch_before_any_gpu_work(kw):
    """A MultiEngine runs FP32 problems on the batched path with boundary
    saving; another problem in the list is refused before the C library sees it."""
    from swit_gb300 import MultiEngine, survey
    s = survey.small()
    with pytest.raises(ValueError, match="FP32 problems on the batched path"):
        MultiEngine([s.engine_args(), dict(s.engine_args(), **kw)])


def test_engine_keeps_pinned_float32_host_buffers():
    """Host float32 inputs reach the C ABI without a copy: a pinned buffer stays
    pinned, so the engine's host-to-device copy is one DMA."""
    import torch
    from swit_gb300.engine import Engine
    a = torch.arange(12, dtype=torch.float32)
    assert Engine._f32(a).ctypes.data == a.data_ptr()
    b = np.arange(12, dtype=np.float32)
    assert Engine._f32(b).ctypes.data == b.ctypes.data
    c = Engine._f32(np.arange(12, dtype=np.float64))
    assert c.dtype == np.float32 and c.flags.c_contiguous


@pytest.mark.parametrize("ns", [1, 5, 49, 200])
def test_autotune_candidates_are_vec_launch_shapes_that_cover_every_shot(ns):
    """The tuner times the engine's automatic choice first, then vec batches
    that split ns shots into 1..8 launches on 1..4 branches, never more
    branches than batches; every candidate covers all shots."""
    from swit_gb300.autotune import candidates
    cs = candidates(ns)
    assert cs[0] == dict(kernel="vec", block_x=4, shots_per_batch=0, graph_branches=0)
    assert all(c["kernel"] == "vec" for c in cs)
    assert len({tuple(sorted(c.items())) for c in cs}) == len(cs)
    for c in cs[1:]:
        b, br = c["shots_per_batch"], c["graph_branches"]
        nbatch = -(-ns // b)
        assert 1 <= b <= ns and 1 <= nbatch <= 8
        assert br == 1 or br <= nbatch
