"""The exact discrete adjoint in the oracle (CPU).

``oracle/exact.py`` restates the forward recursion in numpy (bit-identical to
the C++ oracle in FP64), its tangent-linear model and its literal transpose;
the C++ oracle's gather-form exact adjoint (the form the engine's kernels take)
must agree with that transpose.  Dot-product identities hold to 1e-12 in FP64:
<J dvp, r> = <dvp, J^T r> for the vp gradient and <F s, r> = <s, F^T r> for
the source (the identity the reference checks in dev/test/02_adjoint_test.ipynb
cell 9, there for its adjoint solver).
"""
import numpy as np
import pytest

from oracle import exact as X
from oracle import oracle as O
from swit_gb300 import survey


def case(fs, ns=2, nt=160, seed=3):
    s = survey.small(nx=20, nz=14, npml=5, nt=nt, dx=10.0, dt=0.001, ns=ns)
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, free_surface=fs)
    rho = (310 * s.vp_true ** 0.25).astype(np.float32)
    t = np.arange(nt)
    src = np.stack([np.sin(0.07 * (k + 1) * t) * np.exp(-((t - 30) / 12.0) ** 2) for k in range(pb.ns)])
    rng = np.random.default_rng(seed)
    r = rng.standard_normal((pb.ns, pb.ngmax, nt)).astype(np.float32)
    return s, pb, rho, src.astype(np.float32), r, rng


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


@pytest.mark.parametrize("fs", [1, 0])
def test_numpy_forward_is_the_oracle_forward(fs):
    s, pb, rho, src, r, _ = case(fs)
    ref = O.forward(pb, s.vp_true, rho, src, store=False, fp64=True)
    S = X.Setup(pb, s.vp_true, rho)
    seis = np.stack([X.forward(S, k, src[k])[0] for k in range(pb.ns)])
    np.testing.assert_array_equal(seis, ref["seis"])


@pytest.mark.parametrize("fs", [1, 0])
def test_dot_product_identities(fs):
    s, pb, rho, src, r, rng = case(fs)
    g, gsrc = X.gradient(pb, s.vp_true, rho, src, r)
    dvp = rng.standard_normal((s.nx, s.nz))
    seis, dseis = X.tangent(pb, s.vp_true, rho, src, dvp)
    a, b = np.sum(dseis * r), np.sum(dvp * g)
    assert abs(a - b) <= 1e-12 * abs(a)
    a, b = np.sum(seis * r), np.sum(src.astype(np.float64) * gsrc)
    assert abs(a - b) <= 1e-12 * abs(a)


def test_tangent_matches_finite_differences_with_vmin_fixed():
    """The damping profile follows vmin; a perturbation that leaves vmin alone
    is differentiated exactly (central differences, FP32 model rounding)."""
    s, pb, rho, src, r, rng = case(1)
    vp = s.vp_true.astype(np.float64)
    d = rng.standard_normal(vp.shape)
    d[:, 1:][vp[:, 1:] == vp[:, 1:].min()] = 0.0
    _, dseis = X.tangent(pb, vp, rho, src, d)
    h = 0.5
    sp, _ = X.tangent(pb, vp + h * d, rho, src, d)
    sm, _ = X.tangent(pb, vp - h * d, rho, src, d)
    assert rel((sp - sm) / (2 * h), dseis) <= 5e-4


@pytest.mark.parametrize("fs", [1, 0])
def test_gather_form_oracle_is_the_transpose(fs):
    s, pb, rho, src, r, _ = case(fs)
    g, gsrc = X.gradient(pb, s.vp_true, rho, src, r)
    o = O.exact(pb, s.vp_true, rho, src, r, fp64=True)
    assert rel(o["g"], g) <= 1e-12 and rel(o["gsrc"], gsrc) <= 1e-12
    np.testing.assert_array_equal(o["seis"], O.forward(pb, s.vp_true, rho, src, store=False, fp64=True)["seis"])
    o32 = O.exact(pb, s.vp_true, rho, src, r)
    assert o32["g"].dtype == np.float32
    assert rel(o32["g"], g) <= 1e-4 and rel(o32["gsrc"], gsrc) <= 1e-4


def test_gather_form_with_duplicate_receivers_and_ragged_shots():
    s, pb0, rho, src, r, _ = case(1, ns=3)
    rec = np.array(s.rec_xz, np.float32).reshape(-1, 2)[:12]
    rec[5] = rec[4]  # two receivers on one grid point
    recs = np.broadcast_to(rec, (3,) + rec.shape).copy()
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, recs, free_surface=1, ng=[12, 7, 10])
    rr = np.random.default_rng(5).standard_normal((3, 12, s.nt)).astype(np.float32)
    g, gsrc = X.gradient(pb, s.vp_true, rho, src, rr)
    o = O.exact(pb, s.vp_true, rho, src, rr, fp64=True)
    assert rel(o["g"], g) <= 1e-12 and rel(o["gsrc"], gsrc) <= 1e-12


@pytest.mark.parametrize("comp", ["vx", "vz"])
def test_exact_adjoint_of_velocity_receivers(comp):
    """vx / vz receivers record u / w; the transposed record puts the adjoint
    source into the adjoint u / w.  Dot products and the gather form as for p."""
    s, pb0, rho, src, r, rng = case(1)
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, free_surface=1, comp=comp)
    g, gsrc = X.gradient(pb, s.vp_true, rho, src, r)
    dvp = rng.standard_normal((s.nx, s.nz))
    seis, dseis = X.tangent(pb, s.vp_true, rho, src, dvp)
    np.testing.assert_array_equal(seis, O.forward(pb, s.vp_true, rho, src, store=False, fp64=True)["seis"])
    a, b = np.sum(dseis * r), np.sum(dvp * g)
    assert abs(a - b) <= 1e-12 * abs(a)
    a, b = np.sum(seis * r), np.sum(src.astype(np.float64) * gsrc)
    assert abs(a - b) <= 1e-12 * abs(a)
    o = O.exact(pb, s.vp_true, rho, src, r, fp64=True)
    assert rel(o["g"], g) <= 1e-12 and rel(o["gsrc"], gsrc) <= 1e-12


def test_exact_adjoint_properties_on_random_small_problems():
    """Random small grids, PML widths, record lengths, free-surface flags,
    receiver components and geometries (receivers on the surface row, two on one
    node, ragged counts): the numpy forward equals the C++ oracle's in FP64, the
    dot-product identities hold and the gather form equals the literal transpose."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")

    @hyp.settings(max_examples=25, deadline=None, derandomize=True)
    @hyp.given(nx=st.integers(10, 22), nz=st.integers(10, 16), npml=st.integers(2, 6), nt=st.integers(20, 60),
               fs=st.sampled_from([0, 1]), comp=st.sampled_from(["p", "vx", "vz"]), ns=st.integers(1, 3),
               seed=st.integers(0, 10_000))
    def check(nx, nz, npml, nt, fs, comp, ns, seed):
        rng = np.random.default_rng(seed)
        dx = 10.0
        vp = rng.uniform(1500.0, 3000.0, (nx, nz)).astype(np.float32)
        rho = (310 * vp.astype(np.float64) ** 0.25).astype(np.float32)
        ngmax = int(rng.integers(1, 6))
        xs = rng.uniform(0, (nx - 1) * dx, ns)
        zs = rng.choice([0.0, dx, 2 * dx, 3 * dx], ns)
        rec = np.stack([rng.uniform(0, (nx - 1) * dx, (ns, ngmax)), rng.choice([0.0, dx, 2 * dx], (ns, ngmax))], -1)
        if ngmax > 1:
            rec[:, 1] = rec[:, 0]  # two receivers on one node
        ng = rng.integers(1, ngmax + 1, ns).astype(np.int32)
        pb = O.Problem(nx, nz, npml, nt, dx, 0.001, np.stack([xs, zs], 1), rec.astype(np.float32), free_surface=fs,
                       ng=ng, comp=comp)
        t = np.arange(nt)
        src = np.stack([np.sin(0.3 * (k + 1) * t) * np.exp(-((t - 10) / 5.0) ** 2) for k in range(ns)])
        src = src.astype(np.float32)
        r = rng.standard_normal((ns, ngmax, nt)).astype(np.float32)
        for i in range(ns):
            r[i, ng[i]:] = 0.0  # traces beyond a shot's receiver count carry nothing
        S = X.Setup(pb, vp, rho)
        ref = O.forward(pb, vp, rho, src, store=False, fp64=True)["seis"]
        for i in range(ns):
            np.testing.assert_array_equal(X.forward(S, i, src[i])[0], ref[i, :ng[i]])
        g, gsrc = X.gradient(pb, vp, rho, src, r)
        dvp = rng.standard_normal((nx, nz))
        seis, dseis = X.tangent(pb, vp, rho, src, dvp)
        a, b = np.sum(dseis * r), np.sum(dvp * g)
        assert abs(a - b) <= 1e-11 * max(abs(a), 1e-300)
        a, b = np.sum(seis * r), np.sum(src.astype(np.float64) * gsrc)
        assert abs(a - b) <= 1e-11 * max(abs(a), 1e-300)
        o = O.exact(pb, vp, rho, src, r, fp64=True)
        assert np.linalg.norm(o["g"] - g) <= 1e-12 * max(np.linalg.norm(g), 1e-300)
        assert np.linalg.norm(o["gsrc"] - gsrc) <= 1e-12 * max(np.linalg.norm(gsrc), 1e-300)

    check()
