"""CPU tests of the oracle: pinned against the reference's recorded outputs,
then checked for the properties the path must have.

The pin: dev/test/02_adjoint_test.ipynb runs fd2dmpi on a homogeneous 401 x 401
model (dx = 10 m, dt = 1 ms, nt = 1001, npml = 60, vp = 4000 m/s,
rho = 310 vp^0.25, 5 Hz Ricker of amplitude 1e20, source at (2000, 2000) m,
receivers at (2000, 2000) and (3000, 2000) m; cell 3) and prints (cell 9)
    a = 1.25501e+35, b = 1.25501e+35, ratio = 1.00000e+00, rerr = 0.00000
where a = <d, d> for the trace d of the second receiver and b = <s, A^T d>,
the adjoint wavefield recorded at the source.  The oracle must print the same.
"""
import numpy as np
import pytest
from scipy.integrate import cumulative_trapezoid

from oracle import oracle as O
from swit_gb300 import survey


def _dot_test_inputs():
    nx = nz = 401
    npml, dx, dt, nt = 60, 10.0, 0.001, 1001
    vp = np.full((nx, nz), 4000.0, np.float32)
    rho = (np.power(vp.astype(np.float64), 0.25) * 310).astype(np.float32)
    f0, amp0 = 5.0, 1.0e20
    wav = amp0 * survey.ricker(nt, dt, f0)
    src = cumulative_trapezoid(wav, axis=-1, initial=0)
    rec = np.array([[[2000.0, 2000.0], [3000.0, 2000.0]]])
    pb = O.Problem(nx, nz, npml, nt, dx, dt, [[2000.0, 2000.0]], rec)
    return pb, vp, rho, src


def test_dot_product_matches_reference_notebook():
    pb, vp, rho, src = _dot_test_inputs()
    src32 = src[None].astype(np.float32)
    fwd = O.forward(pb, vp, rho, src32, store=True)
    d = fwd["seis"][0]
    adj = np.zeros((1, 2, pb.nt), np.float32)
    adj[0, 1] = d[1]
    r = O.adjoint(pb, vp, rho, src32, adj, fwd, record_adjoint=True)
    a = np.inner(d[1], adj[0, 1].astype(np.float64))
    b = np.inner(src, r["adj_seis"][0, 0])
    line = "a = %2.5e, b = %2.5e, ratio = %2.5e, rerr = %2.5f" % (a, b, a / b, (a - b) / (a + b))
    assert line == "a = 1.25501e+35, b = 1.25501e+35, ratio = 1.00000e+00, rerr = 0.00000", line


def _small_problem(**kw):
    s = survey.small(**kw)
    pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz)
    return s, pb


def test_fp32_against_fp64_oracle():
    s, pb = _small_problem()
    src = s.source()
    rho = s.rho(s.vp_true)
    f32 = O.forward(pb, s.vp_true, rho, src, store=True)
    f64 = O.forward(pb, s.vp_true, rho, src, store=True, fp64=True)
    err = np.linalg.norm(f32["seis"] - f64["seis"]) / np.linalg.norm(f64["seis"])
    assert err < 1e-5, err
    obs = O.forward(pb, s.vp_init, rho, src, store=False)["seis"]
    g32 = O.gradient(pb, s.vp_true, rho, src, obs)
    g64 = O.gradient(pb, s.vp_true, rho, src, obs, fp64=True)
    for k in ("g", "fw", "bk"):
        e = np.linalg.norm(g32[k] - g64[k]) / np.linalg.norm(g64[k])
        assert e < 1e-4, (k, e)


def test_gradient_equals_forward_then_adjoint():
    """gradient() (strips kept per shot in memory) == forward(store) + syn-obs + adjoint()."""
    s, pb = _small_problem()
    src = s.source()
    rho = s.rho(s.vp_true)
    obs = O.forward(pb, s.vp_init, rho, src, store=False)["seis"]
    fwd = O.forward(pb, s.vp_true, rho, src, store=True)
    adj = (fwd["seis"] - obs).astype(np.float32)
    r1 = O.adjoint(pb, s.vp_true, rho, src, adj, fwd)
    r2 = O.gradient(pb, s.vp_true, rho, src, obs)
    for k in ("g", "fw", "bk"):
        np.testing.assert_array_equal(r1[k], r2[k])


def test_thread_count_does_not_change_results():
    s, pb = _small_problem(ns=4)
    src = s.source()
    rho = s.rho(s.vp_true)
    obs = O.forward(pb, s.vp_init, rho, src, store=False)["seis"]
    r1 = O.gradient(pb, s.vp_true, rho, src, obs, nthreads=1)
    r3 = O.gradient(pb, s.vp_true, rho, src, obs, nthreads=3)
    for k in ("g", "fw", "bk"):
        np.testing.assert_array_equal(r1[k], r3[k])


def test_zero_adjoint_source_gives_zero_gradient_and_forward_illumination():
    s, pb = _small_problem()
    src = s.source()
    rho = s.rho(s.vp_true)
    fwd = O.forward(pb, s.vp_true, rho, src, store=True)
    r = O.adjoint(pb, s.vp_true, rho, src, np.zeros_like(fwd["seis"]), fwd)
    assert not np.any(r["g"]) and not np.any(r["bk"])
    assert np.all(r["fw"] >= 0) and r["fw"].max() > 0


def test_reconstruction_recovers_forward_illumination():
    """The reverse loop rebuilds the forward wavefield from the strips: its
    illumination sum_t p_reco(t)^2 must match the forward run's sum_t p(t)^2.
    The forward sum is built here from runs of nt' = 2..nt steps' end states."""
    s, pb = _small_problem(nx=24, nz=20, npml=6, nt=60, ns=1)
    src = s.source()
    rho = s.rho(s.vp_true)
    fwd = O.forward(pb, s.vp_true, rho, src, store=True)
    r = O.adjoint(pb, s.vp_true, rho, src, np.zeros_like(fwd["seis"]), fwd)
    # reverse loop at it = nt..2 accumulates p_end after reconstructing step it-1,
    # i.e. p(1..nt-1) of the forward run (p(1) = 0)
    acc = np.zeros((pb.nx, pb.nz), np.float64)
    for k in range(2, pb.nt):
        pk = O.Problem(pb.nx, pb.nz, pb.npml, k, pb.dx, pb.dt, s.src_xz, s.rec_xz)
        acc += O.forward(pk, s.vp_true, rho, src[:, :k], store=True)["p_end"][0].astype(np.float64) ** 2
    err = np.linalg.norm(r["fw"] - acc) / np.linalg.norm(acc)
    assert err < 1e-4, err


def test_oracle_rejects_sources_outside_the_model():
    s, pb = _small_problem()
    pb.xs[0] = 1e6
    with pytest.raises(ValueError):
        O.forward(pb, s.vp_true, s.rho(s.vp_true), s.source(), store=False)


def test_velocity_receivers_record_u_and_w():
    """vx / vz receivers (dev/solver/fdcore.f90:154-177) record u or w at the
    receiver points; the wavefield itself, and so the strips, do not change.
    Their adjoint source enters u or w (465-485): a zero source gives a zero
    gradient, a non-zero one a gradient different from the pressure one."""
    s = survey.small(nt=200)
    rho = s.rho(s.vp_true)
    src = s.source()
    out = {}
    for comp in ("p", "vx", "vz"):
        pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, comp=comp)
        out[comp] = O.forward(pb, s.vp_true, rho, src, store=True)
    for comp in ("vx", "vz"):
        np.testing.assert_array_equal(out[comp]["boundary"], out["p"]["boundary"])
        assert np.abs(out[comp]["seis"]).max() > 0
        assert not np.array_equal(out[comp]["seis"], out["p"]["seis"])
    assert not np.array_equal(out["vx"]["seis"], out["vz"]["seis"])
    # the last sample of each trace is the field at the receiver point after the last step
    L = s.npml
    for comp, key in (("p", "p_end"), ("vx", "u_end"), ("vz", "w_end")):
        for i in range(s.ns):
            for ig in range(s.ng):
                jx = int(np.float32(s.rec_xz[i, ig, 0]) / np.float32(s.dx)) + 1
                jz = int(np.float32(s.rec_xz[i, ig, 1]) / np.float32(s.dx)) + 1
                jz = jz + 1 if jz + L == L + 1 else jz  # a receiver on the free surface moves one node down
                assert out[comp]["seis"][i, ig, -1] == out["p"][key][i, jx - 1, jz - 1]
    g = {}
    for comp in ("p", "vx"):
        pb = O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, comp=comp)
        zero = np.zeros_like(out[comp]["seis"], dtype=np.float32)
        assert not O.adjoint(pb, s.vp_true, rho, src, zero, out[comp])["g"].any()
        g[comp] = O.adjoint(pb, s.vp_true, rho, src, out[comp]["seis"].astype(np.float32), out[comp])["g"]
        assert np.abs(g[comp]).max() > 0
    assert not np.array_equal(g["p"], g["vx"])
    with pytest.raises(ValueError):
        O.Problem(s.nx, s.nz, s.npml, s.nt, s.dx, s.dt, s.src_xz, s.rec_xz, comp="vy")
