"""Seeded synthetic surveys with the shapes of the benchmark configurations.

No public model or dataset is used: every model here is generated from a seeded
numpy ``default_rng`` and stands in for the layered / Marmousi-like models the
configurations describe.  Density follows Gardner's relation rho = 310 vp^0.25,
as every reference example does (examples/case-01-marmousi2/
SWIT_workflow_LBGFS.py:49-50).  Sources are the reference's Ricker wavelet
(toolbox/solver.py:183-197) integrated with the trapezoidal rule
(toolbox/solver.py:47).
"""
from dataclasses import dataclass, field

import numpy as np
from scipy.integrate import cumulative_trapezoid
from scipy.ndimage import gaussian_filter


def ricker(nt, dt, f0):
    """toolbox/solver.py:183-197: (1 - 2 (pi f0)^2 (t-t0)^2) exp(-(pi f0)^2 (t-t0)^2), t0 = 1.2/f0."""
    t = np.linspace(0, dt * nt, num=nt, endpoint=False)
    t0 = 1.2 / f0
    temp = (np.pi * f0) ** 2
    return (1 - 2 * temp * (t - t0) ** 2) * np.exp(-temp * (t - t0) ** 2)


def integrated_source(wavelet):
    """toolbox/solver.py:47: cumtrapz(wavelet, axis=-1, initial=0) (scipy's cumulative_trapezoid)."""
    return cumulative_trapezoid(wavelet, axis=-1, initial=0).astype(np.float32)


def gardner(vp):
    """Gardner density 310 vp^0.25 (examples/case-01-marmousi2/SWIT_workflow_LBGFS.py:49-50)."""
    return (np.power(np.asarray(vp, np.float64), 0.25) * 310).astype(np.float32)


@dataclass
class Survey:
    name: str
    nx: int
    nz: int
    dx: float
    dt: float
    nt: int
    npml: int
    f0: float
    vp_true: np.ndarray
    vp_init: np.ndarray
    src_xz: np.ndarray          # (ns, 2)
    rec_xz: np.ndarray          # (ns, ng, 2)
    free_surface: int = 1
    meta: dict = field(default_factory=dict)

    @property
    def ns(self):
        return self.src_xz.shape[0]

    @property
    def ng(self):
        return self.rec_xz.shape[1]

    def source(self):
        w = ricker(self.nt, self.dt, self.f0)
        return np.repeat(integrated_source(w)[None, :], self.ns, axis=0)

    def rho(self, vp):
        return gardner(vp)

    def engine_args(self):
        return dict(nx=self.nx, nz=self.nz, npml=self.npml, nt=self.nt, dx=self.dx, dt=self.dt,
                    src_xz=self.src_xz, rec_xz=self.rec_xz, free_surface=self.free_surface)


def _line_geometry(nx, dx, ns, zs, zr, ng=None):
    xmax = (nx - 1) * dx
    sx = np.linspace(0.0, xmax, ns) if ns > 1 else np.array([xmax / 2])
    src = np.stack([sx, np.full(ns, zs)], axis=1)
    ng = nx if ng is None else ng
    rx = np.arange(ng) * dx
    rec = np.stack([rx, np.full(ng, zr)], axis=1)
    return src.astype(np.float32), np.broadcast_to(rec, (ns, ng, 2)).astype(np.float32)


def layered_anomaly(nx=201, nz=101, dx=25.0, seed=1000, n_anom=6, vtop=1500.0, vbot=3500.0):
    """Linear vp gradient from vtop to vbot plus n_anom Gaussian anomalies of +-300 m/s, radius 100-300 m."""
    rng = np.random.default_rng(seed)
    z = np.arange(nz) * dx
    x = np.arange(nx) * dx
    vp = np.broadcast_to(vtop + (vbot - vtop) * z / z[-1], (nx, nz)).astype(np.float64).copy()
    X, Z = np.meshgrid(x, z, indexing="ij")
    for _ in range(n_anom):
        cx, cz = rng.uniform(0.15, 0.85) * x[-1], rng.uniform(0.25, 0.85) * z[-1]
        r = rng.uniform(100.0, 300.0)
        a = rng.choice([-300.0, 300.0])
        vp += a * np.exp(-((X - cx) ** 2 + (Z - cz) ** 2) / (r * r))
    return vp.astype(np.float32)


def faulted_layers(nx=481, nz=141, dx=25.0, seed=1001, nlayers=30, vmin=1500.0, vmax=4700.0, water=12,
                   max_dip_deg=30.0, nfaults=3, throw=(50.0, 300.0), noise=0.05):
    """Marmousi-like model: dipping layers vmin..vmax under a water layer, normal faults, +-noise heterogeneity."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx) * dx
    z = np.arange(nz) * dx
    X, Z = np.meshgrid(x, z, indexing="ij")
    top = water * dx
    depths = np.linspace(top, z[-1] * 1.05, nlayers)[1:]
    # gently varying dips: interface k is z_k + tan(dip_k) (x - xc), with
    # neighbouring interfaces sharing similar dips
    dips = np.cumsum(rng.normal(0, 4.0, nlayers - 1))
    dips = np.clip(dips - dips.mean(), -max_dip_deg, max_dip_deg) * np.pi / 180.0
    xc = x[-1] / 2

    def layer_index(zz):
        idx = np.zeros(zz.shape, np.int32)
        for k, (d0, dp) in enumerate(zip(depths, dips)):
            zk = d0 + np.tan(dp) * (X - xc) * 0.5
            idx += (zz > zk).astype(np.int32)
        return idx

    zeff = Z.copy()
    for _ in range(nfaults):
        xf = rng.uniform(0.15, 0.85) * x[-1]
        ang = rng.uniform(55.0, 70.0) * np.pi / 180.0 * rng.choice([-1.0, 1.0])
        t = rng.uniform(*throw)
        hanging = (X - xf) > (Z - top) / np.tan(ang)
        zeff = np.where(hanging & (Z > top), zeff - t, zeff)
    idx = layer_index(zeff)
    vel = np.linspace(vmin + 200.0, vmax, nlayers)
    vp = vel[np.clip(idx, 0, nlayers - 1)]
    vp *= 1.0 + noise * rng.uniform(-1.0, 1.0, vp.shape)
    vp[:, :water] = vmin
    return np.clip(vp, vmin, vmax * (1 + noise)).astype(np.float32)


def thrust_fold(nx=501, nz=171, dx=20.0, seed=1002, nlayers=25, vmin=2000.0, vmax=6000.0, amp=(300.0, 800.0),
                nthrust=2, offset=(200.0, 500.0)):
    """Thrust-fold model: nlayers layers vmin..vmax (increasing with depth) folded by
    one Gaussian anticline of amplitude amp and cut by nthrust thrust faults (dip
    25-40 degrees) whose hanging walls are raised by offset."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx) * dx
    z = np.arange(nz) * dx
    X, Z = np.meshgrid(x, z, indexing="ij")
    a = rng.uniform(*amp)
    xc = rng.uniform(0.3, 0.7) * x[-1]
    width = rng.uniform(0.15, 0.3) * x[-1]
    zeff = Z + a * np.exp(-((X - xc) / width) ** 2)  # layers pushed up over the anticline
    for _ in range(nthrust):
        xf = rng.uniform(0.2, 0.8) * x[-1]
        ang = rng.uniform(25.0, 40.0) * np.pi / 180.0
        side = rng.choice([-1.0, 1.0])
        hanging = Z < side * (X - xf) * np.tan(ang)  # above the fault plane
        zeff = np.where(hanging, zeff + rng.uniform(*offset), zeff)
    depths = np.linspace(zeff.min(), zeff.max(), nlayers + 1)[1:-1]  # every layer appears in the section
    depths = depths + rng.uniform(-0.2, 0.2, depths.shape) * (depths[1] - depths[0])
    idx = np.searchsorted(np.sort(depths), zeff)
    vel = np.linspace(vmin, vmax, nlayers)
    return vel[np.clip(idx, 0, nlayers - 1)].astype(np.float32)


def smooth_layered_random(nx=2001, nz=601, dx=10.0, seed=1003, vmin=1500.0, vmax=5000.0, nlayers=12,
                          corr_m=200.0, std=0.04):
    """Smooth-plus-layered model vmin..vmax with a 2-D Gaussian-correlated random field (relative std, correlation
    length corr_m), clipped to [vmin, 1.1 vmax]."""
    rng = np.random.default_rng(seed)
    z = np.arange(nz) * dx
    trend = vmin + (vmax - vmin) * (z / z[-1]) ** 0.8
    steps = np.sort(rng.uniform(0.1, 0.95, nlayers)) * z[-1]
    jumps = rng.uniform(-150.0, 250.0, nlayers)
    layered = trend + sum(j * (z > s0) for j, s0 in zip(jumps, steps))
    vp = np.broadcast_to(layered, (nx, nz)).astype(np.float64)
    field = gaussian_filter(rng.standard_normal((nx, nz)), sigma=corr_m / dx / np.sqrt(2.0), mode="wrap")
    field /= field.std()
    vp = vp * (1.0 + std * field)
    return np.clip(vp, vmin, 1.1 * vmax).astype(np.float32)


def smooth(vp, sigma_m, dx, keep_top=0):
    out = gaussian_filter(np.asarray(vp, np.float64), sigma=sigma_m / dx, mode="nearest")
    if keep_top:
        out[:, :keep_top] = vp[:, :keep_top]
    return out.astype(np.float32)


def config(idx, ns=None, nt=None):
    """The seeded survey of benchmark configuration idx (0: plain small, 1: batched Marmousi-like,
    2: correlation misfits on a thrust-fold model, 3: large memory-bound case)."""
    if idx == 0:
        nx, nz, dx, dt, nt_, npml, f0 = 201, 101, 25.0, 0.002, 2000, 40, 5.0
        vp = layered_anomaly(nx, nz, dx, seed=1000)
        init = smooth(vp, 250.0, dx)
        src, rec = _line_geometry(nx, dx, 5 if ns is None else ns, 50.0, 50.0)
        name = "plain-small 201x101 dx25 nt2000 5 shots"
    elif idx == 1:
        nx, nz, dx, dt, nt_, npml, f0 = 481, 141, 25.0, 0.002, 4000, 40, 5.0
        vp = faulted_layers(nx, nz, dx, seed=1001)
        init = smooth(vp, 250.0, dx, keep_top=12)
        src, rec = _line_geometry(nx, dx, 49 if ns is None else ns, 25.0, 25.0)
        name = "marmousi-like 481x141 dx25 nt4000 49 shots"
    elif idx == 2:
        nx, nz, dx, dt, nt_, npml, f0 = 501, 171, 20.0, 0.0015, 5000, 40, 5.0
        vp = thrust_fold(nx, nz, dx, seed=1002)
        init = smooth(vp, 250.0, dx)
        src, rec = _line_geometry(nx, dx, 51 if ns is None else ns, 20.0, 20.0)
        name = "thrust-fold 501x171 dx20 nt5000 51 shots"
    elif idx == 3:
        nx, nz, dx, dt, nt_, npml, f0 = 2001, 601, 10.0, 0.001, 6000, 60, 10.0
        vp = smooth_layered_random(nx, nz, dx, seed=1003)
        init = smooth(vp, 200.0, dx)
        src, rec = _line_geometry(nx, dx, 200 if ns is None else ns, 20.0, 20.0)
        name = "large 2001x601 dx10 nt6000 200 shots"
    else:
        raise ValueError("configuration %d is not generated here" % idx)
    return Survey(name=name, nx=nx, nz=nz, dx=dx, dt=dt, nt=nt_ if nt is None else nt, npml=npml, f0=f0,
                  vp_true=vp, vp_init=init, src_xz=src, rec_xz=rec)


def config4_instances(n=64, shot_scale=1.0, nt_scale=1.0, npml=40):
    """The uneven multi-instance batch: instance i (seed 2000 + i) has nx, nz drawn
    from [201, 801] x [101, 301], dx from {10, 20, 25} m, a Ricker of 3-12 Hz, nt
    from [1500, 5000], 8-64 shots and one receiver per surface cell, vp from the
    layered + anomaly generator, dt = 0.5 dx / vmax (CFL 0.5).  shot_scale and
    nt_scale shrink the shot counts and record lengths of a bounded sample."""
    out = []
    for i in range(n):
        rng = np.random.default_rng(2000 + i)
        nx, nz = int(rng.integers(201, 802)), int(rng.integers(101, 302))
        dx = float(rng.choice([10.0, 20.0, 25.0]))
        f0 = float(rng.uniform(3.0, 12.0))
        nt = max(50, int(round(int(rng.integers(1500, 5001)) * nt_scale)))
        ns = max(1, int(round(int(rng.integers(8, 65)) * shot_scale)))
        vp = layered_anomaly(nx, nz, dx, seed=2000 + i)
        dt = float(np.float32(0.5 * dx / float(vp.max())))
        src, rec = _line_geometry(nx, dx, ns, 2 * dx, 2 * dx, ng=nx)
        out.append(Survey(name="instance %d %dx%d dx%g nt%d %d shots" % (i, nx, nz, dx, nt, ns), nx=nx, nz=nz,
                          dx=dx, dt=dt, nt=nt, npml=npml, f0=f0, vp_true=vp, vp_init=smooth(vp, 250.0, dx),
                          src_xz=src, rec_xz=rec))
    return out


def small(nx=48, nz=32, npml=10, nt=300, dx=10.0, dt=0.001, ns=3, ng=None, seed=7, zs=20.0, zr=10.0):
    """A small seeded problem for parity tests (layered + anomalies, a few shots)."""
    vp = layered_anomaly(nx, nz, dx, seed=seed, n_anom=3, vtop=1800.0, vbot=3200.0)
    src, rec = _line_geometry(nx, dx, ns, zs, zr, ng=ng)
    return Survey(name="small", nx=nx, nz=nz, dx=dx, dt=dt, nt=nt, npml=npml, f0=25.0, vp_true=vp,
                  vp_init=smooth(vp, 3 * dx, dx), src_xz=src, rec_xz=rec)
