"""Literal forward recursion, tangent-linear model and exact discrete adjoint
in numpy FP64 (test infrastructure only).

Only tests/ import this module.  It pins the C++ oracle's gather-form exact
adjoint (``oracle_exact_f64``) and, through it, the engine's exact-adjoint
kernels:

* ``forward`` restates fd2dmpi's forward step (fd2dmpi/fdcore.f90:75-128) with
  whole-array slices, in the same evaluation order as the C++ oracle, so in
  FP64 its seismograms equal ``oracle.forward(..., fp64=True)`` bit for bit.
  It can also carry a tangent-linear state for a perturbation of the padded
  velocity, dA = 2 den c dc dt / dx (the damping profile held fixed).
* ``adjoint`` is the transpose of that recursion written statement by
  statement in reverse (scatter form): record, w mirror, velocity updates,
  p mirror, source, pressure update.

So <J dvp, r> = <dvp, J^T r> and <F s, r> = <s, F^T r> hold to rounding.  The
damping profile depends on vp only through vmin (pml.f90:80); like the
absorbing layer it is held fixed, so J is the derivative for perturbations that
leave vmin unchanged.
Model setup follows fd2dmpi/io.f90:243-292 (edge padding), math.f90:342-361
(vmin) and pml.f90:74-101 (damping profile); C1, C2 from global.f90:34-35.
Small grids only (a few thousand points, a few hundred steps).
"""
import math

import numpy as np

C1 = 9.0 / 8.0
C2 = -1.0 / 24.0


class Setup:
    """Padded model, damping and geometry of an ``oracle.Problem`` in FP64, on
    1-based (NZ + 1, NX + 1) arrays (row/column 0 unused)."""

    def __init__(self, pb, vp, rho):
        self.pb = pb
        nx, nz, L = pb.nx, pb.nz, pb.npml
        self.nx, self.nz, self.L = nx, nz, L
        self.NX, self.NZ = nx + 2 * L, nz + 2 * L
        self.nt = pb.nt
        self.dx = float(np.float32(pb.dx))
        self.dt = float(np.float32(pb.dt))
        self.fs = L + 1
        self.fold = pb.free_surface == 1
        self.comp = getattr(pb, "comp", 0)  # recorded component: 0 = p, 1 = vx (u), 2 = vz (w)
        self.c = self.pad(np.asarray(vp, np.float32))
        self.den = self.pad(np.asarray(rho, np.float32))
        NX, NZ, dx, dt = self.NX, self.NZ, self.dx, self.dt
        vmin = float(self.c[L + 2:L + nz + 1, L + 1:L + nx + 1].min())  # rows i > fs - npml = 1
        a = (L - 1) * dx
        kappa = 3.0 * vmin * math.log(1000.0) / (2.0 * a)
        damp = [0.0] * (L + 1)
        for ix in range(1, L + 1):
            xa = (ix - 1) * dx / a
            damp[ix] = kappa * xa * xa
        dg = np.zeros((NZ + 1, NX + 1))
        for ix in range(1, L + 1):
            dg[1:, L - ix + 1] = damp[ix]
            dg[1:, NX + ix - L] = damp[ix]
        for iz in range(1, L + 1):
            lo, hi = 1 + (L - (iz - 1)), NX - (L - (iz - 1))
            dg[L - iz + 1, lo:hi + 1] = damp[iz]
            dg[NZ + iz - L, lo:hi + 1] = damp[iz]
        self.damp_g = dg
        c, den = self.c, self.den
        self.A = den * c * c * dt / dx
        self.B = np.zeros_like(den)
        self.B[1:, 1:] = dt / (den[1:, 1:] * dx)
        self.dAdc = 2.0 * den * c * dt / dx
        self.kp = dg * dt
        self.ku = np.zeros_like(dg)
        self.ku[:, 1:NX] = 0.5 * (dg[:, 1:NX] + dg[:, 2:NX + 1]) * dt
        self.kw = np.zeros_like(dg)
        self.kw[1:NZ, :] = 0.5 * (dg[1:NZ, :] + dg[2:NZ + 1, :]) * dt
        gi = lambda x: L + int(np.float32(x) / np.float32(pb.dx)) + 1  # fdcore.f90:70-71, single precision
        self.src = []
        self.rec = []
        for s in range(pb.ns):
            sx, sz = gi(pb.xs[s]), gi(pb.zs[s])
            if sz == self.fs:
                sz += 1
            self.src.append((sz, sx))
            r = []
            for g in range(int(pb.ng[s])):
                gx, gz = gi(pb.xg[s * pb.ngmax + g]), gi(pb.zg[s * pb.ngmax + g])
                if gz == self.fs:
                    gz += 1
                r.append((gz, gx))
            self.rec.append(r)

    def pad(self, m):
        """(nx, nz) interior -> (NZ+1, NX+1) padded copy, io.f90:243-292 order."""
        L, nx, nz, NX, NZ = self.L, self.nx, self.nz, self.NX, self.NZ
        a = np.zeros((NZ + 1, NX + 1))
        a[L + 1:L + nz + 1, L + 1:L + nx + 1] = np.asarray(m, np.float64).T
        a[L + 1:L + nz + 1, 1:L + 1] = a[L + 1:L + nz + 1, L + 1:L + 2]
        a[L + 1:L + nz + 1, NX - L + 1:NX + 1] = a[L + 1:L + nz + 1, NX - L:NX - L + 1]
        a[1:L + 1, 1:] = a[L + 1:L + 2, 1:]
        a[NZ - L + 1:NZ + 1, 1:] = a[NZ - L:NZ - L + 1, 1:]
        return a

    def fold_pad(self, a):
        """Transpose of pad: (NZ+1, NX+1) -> (nx, nz), summing each padded copy
        into the interior point it was copied from."""
        L, nx, nz, NX, NZ = self.L, self.nx, self.nz, self.NX, self.NZ
        z = np.clip(np.arange(1, NZ + 1) - L, 1, nz) - 1
        x = np.clip(np.arange(1, NX + 1) - L, 1, nx) - 1
        out = np.zeros((nz, nx))
        np.add.at(out, (z[:, None], x[None, :]), a[1:, 1:])
        return out.T

    # ranges (1-based, inclusive) of the three updates
    def rp(self):
        return slice(self.fs + 1, self.NZ - 1), slice(3, self.NX - 1)

    def ru(self):
        return slice(self.fs, self.NZ), slice(2, self.NX - 1)

    def rw(self):
        return slice(self.fs, self.NZ - 1), slice(2, self.NX)


def _sh(sl, d):
    return slice(sl.start + d, sl.stop + d)


def forward(S, s_idx, src, dc=None, save_d=False):
    """One shot: seismograms (ng, nt); with dc (padded velocity perturbation,
    (NZ+1, NX+1)) also the tangent-linear seismograms; with save_d the
    divergence term D of every step (nt, NZ+1, NX+1)."""
    NZ, NX, nt, dt = S.NZ, S.NX, S.nt, S.dt
    p, u, w = (np.zeros((NZ + 1, NX + 1)) for _ in range(3))
    tl = dc is not None
    if tl:
        dA = S.dAdc * dc
        dp, du, dw = (np.zeros((NZ + 1, NX + 1)) for _ in range(3))
    rec = S.rec[s_idx]
    sz, sx = S.src[s_idx]
    seis = np.zeros((len(rec), nt))
    dseis = np.zeros((len(rec), nt)) if tl else None
    Ds = np.zeros((nt + 1, NZ + 1, NX + 1)) if save_d else None
    s = np.zeros(nt + 2)
    s[1:nt + 1] = np.asarray(src, np.float32).astype(np.float64)
    Z, X = S.rp()
    Zu, Xu = S.ru()
    Zw, Xw = S.rw()
    F = S.fs

    def div(u, w):
        return (C1 * (u[Z, X] - u[Z, _sh(X, -1)] + w[Z, X] - w[_sh(Z, -1), X]) +
                C2 * (u[Z, _sh(X, 1)] - u[Z, _sh(X, -2)] + w[_sh(Z, 1), X] - w[_sh(Z, -2), X]))

    def gx(p):
        return C1 * (p[Zu, _sh(Xu, 1)] - p[Zu, Xu]) + C2 * (p[Zu, _sh(Xu, 2)] - p[Zu, _sh(Xu, -1)])

    def gz(p):
        return C1 * (p[_sh(Zw, 1), Xw] - p[Zw, Xw]) + C2 * (p[_sh(Zw, 2), Xw] - p[_sh(Zw, -1), Xw])

    for it in range(2, nt + 1):
        D = div(u, w)
        if tl:
            dD = div(du, dw)
            dp[Z, X] = (1.0 - S.kp[Z, X]) * dp[Z, X] - S.A[Z, X] * dD - dA[Z, X] * D
        p[Z, X] = (1.0 - S.kp[Z, X]) * p[Z, X] - S.A[Z, X] * D
        if save_d:
            Ds[it][Z, X] = D
        p[sz, sx] = p[sz, sx] + dt * s[it]
        if S.fold:
            p[F - 1, 1:] = -p[F + 1, 1:]
            if tl:
                dp[F - 1, 1:] = -dp[F + 1, 1:]
        gu, gw = gx(p), gz(p)
        u[Zu, Xu] = (1.0 - S.ku[Zu, Xu]) * u[Zu, Xu] - S.B[Zu, Xu] * gu
        w[Zw, Xw] = (1.0 - S.kw[Zw, Xw]) * w[Zw, Xw] - S.B[Zw, Xw] * gw
        if tl:
            du[Zu, Xu] = (1.0 - S.ku[Zu, Xu]) * du[Zu, Xu] - S.B[Zu, Xu] * gx(dp)
            dw[Zw, Xw] = (1.0 - S.kw[Zw, Xw]) * dw[Zw, Xw] - S.B[Zw, Xw] * gz(dp)
        if S.fold:
            w[F - 1, 1:] = w[F, 1:]
            if tl:
                dw[F - 1, 1:] = dw[F, 1:]
        rf = (p, u, w)[S.comp]
        for g, (rz, rx) in enumerate(rec):
            seis[g, it - 1] = rf[rz, rx]
            if tl:
                dseis[g, it - 1] = (dp, du, dw)[S.comp][rz, rx]
    return seis, dseis, Ds


def adjoint(S, s_idx, adj, Ds):
    """Transpose of ``forward`` for one shot, statement by statement in reverse.
    adj (ng, nt) = dJ/dseis.  Returns (gA (NZ+1, NX+1): dJ/dA per PML point,
    gsrc (nt,): dJ/dsrc)."""
    NZ, NX, nt, dt = S.NZ, S.NX, S.nt, S.dt
    lp, lu, lw = (np.zeros((NZ + 1, NX + 1)) for _ in range(3))
    gA = np.zeros((NZ + 1, NX + 1))
    gsrc = np.zeros(nt)
    rec = S.rec[s_idx]
    sz, sx = S.src[s_idx]
    Z, X = S.rp()
    Zu, Xu = S.ru()
    Zw, Xw = S.rw()
    F = S.fs
    for it in range(nt, 1, -1):
        # S6 record (p, u or w at the receivers)
        lr = (lp, lu, lw)[S.comp]
        for g, (rz, rx) in enumerate(rec):
            lr[rz, rx] += adj[g, it - 1]
        # S5 w mirror
        if S.fold:
            lw[F, 1:] += lw[F - 1, 1:]
            lw[F - 1, 1:] = 0.0
        # S4 velocity updates (both read p only)
        t = S.B[Zw, Xw] * lw[Zw, Xw]
        lp[_sh(Zw, 1), Xw] += -C1 * t
        lp[Zw, Xw] += C1 * t
        lp[_sh(Zw, 2), Xw] += -C2 * t
        lp[_sh(Zw, -1), Xw] += C2 * t
        lw[Zw, Xw] = (1.0 - S.kw[Zw, Xw]) * lw[Zw, Xw]
        t = S.B[Zu, Xu] * lu[Zu, Xu]
        lp[Zu, _sh(Xu, 1)] += -C1 * t
        lp[Zu, Xu] += C1 * t
        lp[Zu, _sh(Xu, 2)] += -C2 * t
        lp[Zu, _sh(Xu, -1)] += C2 * t
        lu[Zu, Xu] = (1.0 - S.ku[Zu, Xu]) * lu[Zu, Xu]
        # S3 p mirror
        if S.fold:
            lp[F + 1, 1:] += -lp[F - 1, 1:]
            lp[F - 1, 1:] = 0.0
        # S2 source
        gsrc[it - 1] = dt * lp[sz, sx]
        # S1 pressure update
        t = lp[Z, X].copy()
        gA[Z, X] += -t * Ds[it][Z, X]
        a = S.A[Z, X] * t
        lu[Z, X] += -C1 * a
        lu[Z, _sh(X, -1)] += C1 * a
        lw[Z, X] += -C1 * a
        lw[_sh(Z, -1), X] += C1 * a
        lu[Z, _sh(X, 1)] += -C2 * a
        lu[Z, _sh(X, -2)] += C2 * a
        lw[_sh(Z, 1), X] += -C2 * a
        lw[_sh(Z, -2), X] += C2 * a
        lp[Z, X] = (1.0 - S.kp[Z, X]) * t
    return gA, gsrc


def gradient(pb, vp, rho, src, adj):
    """dJ/dvp (nx, nz) and dJ/dsrc (ns, nt) for adjoint sources adj (ns, ngmax, nt)."""
    S = Setup(pb, vp, rho)
    gA = np.zeros((S.NZ + 1, S.NX + 1))
    gsrc = np.zeros((pb.ns, pb.nt))
    for s in range(pb.ns):
        _, _, Ds = forward(S, s, src[s], save_d=True)
        a, gsrc[s] = adjoint(S, s, np.asarray(adj[s], np.float64)[:len(S.rec[s])], Ds)
        gA += a
    return S.fold_pad(gA * S.dAdc), gsrc


def tangent(pb, vp, rho, src, dvp):
    """Seismograms and their tangent-linear response to dvp, (ns, ngmax, nt) each."""
    S = Setup(pb, vp, rho)
    dc = S.pad(np.asarray(dvp, np.float64))
    seis = np.zeros((pb.ns, pb.ngmax, pb.nt))
    dseis = np.zeros_like(seis)
    for s in range(pb.ns):
        a, b, _ = forward(S, s, src[s], dc=dc)
        seis[s, :a.shape[0]] = a
        dseis[s, :b.shape[0]] = b
    return seis, dseis
