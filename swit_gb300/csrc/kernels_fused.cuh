// kernels_fused.cuh -- one kernel per time step (forward, and reverse) for grids
// whose padded column fits one CTA (LD <= 1024).
//
// A CTA owns TX consecutive columns [x0, x0+TX) of one shot and all LD rows:
// thread iz holds row iz and walks the columns left to right.  Neighbours along
// x come from per-thread register windows; neighbours along z come from a
// shared-memory copy of the current column.  Because a step reads the old
// state and writes the new one, state is double-buffered (ping-pong) and every
// array is read once and written once per step; the few halo columns a CTA
// recomputes come from L2.
//
// Arithmetic is identical to kernels.cuh (same expressions, same order, no FMA):
// results are bit-identical to the split kernels and to the CPU oracle.
#pragma once
#include "kernels.cuh"

namespace swit {

// Damping of one fixed row along the columns (pml.f90:88-99): the side profile,
// overwritten on the row's trapezoid span when the row lies in the top or
// bottom PML.
template <class R>
struct RowDamp {
  int lo, hi;  // trapezoid span of this row (lo > hi: none)
  R v;         // damping on the span
  __device__ void init(const R* damp, int iz, int L, int NX, int NZ) {
    lo = 1;
    hi = 0;
    v = R(0);
    if (iz >= 1 && iz <= L) {
      lo = iz + 1;
      hi = NX - iz;
      v = damp[L - iz + 1];
    } else if (iz >= NZ - L + 1 && iz <= NZ) {
      const int k = iz - NZ + L;
      lo = L - k + 2;
      hi = NX - L + k - 1;
      v = damp[k];
    }
  }
  __device__ R at(const R* damp, int ix, int L, int NX) const {
    if (ix >= lo && ix <= hi) return v;
    if (ix <= L) return damp[L - ix + 1];
    if (ix >= NX - L + 1) return damp[ix - (NX - L)];
    return R(0);
  }
};

template <class R>
__device__ inline R ld_col(const R* f, int col, int ncol, int LD, int iz, bool ok) {
  return (ok && col >= 1 && col <= ncol) ? f[(size_t)(col - 1) * LD + (iz - 1)] : R(0);
}

// ---------------------------------------------------------------------------
// Forward step `it` (fdcore.f90:77-159) from (P0,U0,W0) into (P1,U1,W1).
// Shared memory: two columns of LD+4 values (w_old, p_new), index iz+1.
template <class R, int TX>
__global__ void __launch_bounds__(1024) k_fwd_step(Grid<R> g, Sources src, Receivers rec,
                                                   const R* __restrict__ s_fwd, const R* __restrict__ P0,
                                                   const R* __restrict__ U0, const R* __restrict__ W0, R* __restrict__ P1,
                                                   R* __restrict__ U1, R* __restrict__ W1, R* __restrict__ seis_t,
                                                   R* __restrict__ strips, int it, int shot0) {
  extern __shared__ unsigned char smem_raw[];
  R* colw = reinterpret_cast<R*>(smem_raw);
  R* colp = colw + (g.LD + 4);
  const int iz = threadIdx.x + 1;
  const int s = shot0 + blockIdx.y;
  const int NX = g.NX, NZ = g.NZ, L = g.L, LD = g.LD, fs = g.fs;
  const int x0 = blockIdx.x * TX + 1;
  const int x1 = min(x0 + TX, NX + 1);
  const bool row = iz <= NZ;
  const size_t off = (size_t)s * g.FSZ;
  const R* p0 = P0 + off;
  const R* u0 = U0 + off;
  const R* w0 = W0 + off;
  R* p1 = P1 + off;
  R* u1 = U1 + off;
  R* w1 = W1 + off;
  const R dt = g.dt, c1 = g.c1, c2 = g.c2;
  RowDamp<R> rd0, rd1;
  rd0.init(g.damp, iz, L, NX, NZ);
  rd1.init(g.damp, iz + 1, L, NX, NZ);
  const bool p_row = iz >= fs + 1 && iz <= NZ - 2;
  const bool u_row = iz >= fs && iz <= NZ - 1;
  const bool w_row = iz >= fs && iz <= NZ - 2;
  const int isx = src.isx[s], isz = src.isz[s];
  const R sval = dt * s_fwd[(size_t)s * (g.nt + 1) + (it - 1)];
  R* b = strips ? strips + ((size_t)s * g.snt + (it - g.sit0)) * g.SL : nullptr;
  const StripOff so = strip_offsets(g.nx, g.nz);
  const int* cp = rec.colptr + (size_t)s * (NX + 2);
  R* trace = seis_t + ((size_t)s * g.nt + (it - 1)) * g.ngmax;

  // windows: u_old(c-2..c+1), p_new(c-3..c), B(c-2..c)
  R um2 = ld_col(u0, x0 - 3, NX - 1, LD, iz, row);
  R um1 = ld_col(u0, x0 - 2, NX - 1, LD, iz, row);
  R uc = ld_col(u0, x0 - 1, NX - 1, LD, iz, row);
  R up1;
  R pm3 = R(0), pm2 = R(0), pm1 = R(0), pc = R(0);
  R bm2 = R(0), bm1 = R(0), bc = R(0);
  R wold = R(0);

  for (int c = x0 - 1; c <= x1 + 1; ++c) {
    // phase 1: column c of w_old to shared memory; this column's loads
    up1 = ld_col(u0, c + 1, NX - 1, LD, iz, row);
    const bool colok = row && c >= 1 && c <= NX;
    const size_t k = (size_t)(c - 1) * LD + (iz - 1);
    wold = colok ? w0[k] : R(0);
    const R pold = colok ? p0[k] : R(0);
    const R a = colok ? g.A[k] : R(0);
    bm2 = bm1;
    bm1 = bc;
    bc = colok ? g.B[k] : R(0);
    colw[iz + 1] = wold;
    __syncthreads();
    // phase 2: p_new(c) (fdcore.f90:77-89)
    R pv = pold;
    if (p_row && c >= 3 && c <= NX - 2) {
      const R kappa = rd0.at(g.damp, c, L, NX) * dt;
      pv = (R(1.0) - kappa) * pold - a * (c1 * (uc - um1 + colw[iz + 1] - colw[iz]) +
                                          c2 * (up1 - um2 + colw[iz + 2] - colw[iz - 1]));
    }
    if (c == isx && iz == isz) pv = pv + sval;
    colp[iz + 1] = pv;
    pm3 = pm2;
    pm2 = pm1;
    pm1 = pc;
    pc = pv;
    __syncthreads();
    // phase 3: w_new(c), stores of column c; u_new(c-2)
    if (c >= x0 && c < x1 && row) {
      // p_new(fs-1) = -p_new(fs+1) (fdcore.f90:92-94) as seen by the w stencil
      auto pz = [&](int r) -> R { return (g.fs_flag == 1 && r == fs - 1) ? -colp[fs + 2] : colp[r + 1]; };
      R wv = wold;
      if (w_row && c >= 2 && c <= NX - 1) {
        const R kappa = R(0.5) * (rd0.at(g.damp, c, L, NX) + rd1.at(g.damp, c, L, NX)) * dt;
        wv = (R(1.0) - kappa) * wold - bc * (c1 * (pz(iz + 1) - pz(iz)) + c2 * (pz(iz + 2) - pz(iz - 1)));
      }
      if (iz != fs - 1 || g.fs_flag != 1) {
        p1[k] = pv;
        w1[k] = wv;
      }
      if (g.fs_flag == 1 && iz == fs + 1) p1[k - 2] = -pv;  // p(fs-1) = -p(fs+1)
      if (g.fs_flag == 1 && iz == fs) w1[k - 1] = wv;      // w(fs-1) = w(fs), fdcore.f90:116-120
      // receiver gather (fdcore.f90:123-128)
      for (int e = cp[c]; e < cp[c + 1]; ++e)
        if (rec.zrow[e] == iz) trace[rec.ig[e]] = pv;
      if (b) {
        const int jx = c - L, jz = iz - L;
        if (jx >= 1 && jx <= g.nx) {
          if (iz == NZ - L) b[so.B0 + jx - 1] = pv;
          if (iz == NZ - L - 1) {
            b[so.B1 + jx - 1] = pv;
            b[so.B2 + jx - 1] = wv;
          }
          if (iz == fs) {
            b[so.T0 + jx - 1] = pv;
            b[so.T5 + jx - 1] = wv;
          }
          if (iz == fs + 1) b[so.T1 + jx - 1] = pv;
          if (iz == fs + 2) b[so.T2 + jx - 1] = pv;
        }
        if (jz >= 1 && jz <= g.nz) {
          if (c == L + 1) b[so.S0 + jz - 1] = pv;
          if (c == L + 2) b[so.S1 + jz - 1] = pv;
          if (c == NX - L) b[so.S3 + jz - 1] = pv;
          if (c == NX - L - 1) b[so.S4 + jz - 1] = pv;
        }
      }
    }
    const int cu = c - 2;  // u_new(cu) needs p_new(cu-1 .. cu+2) = (pm3, pm2, pm1, pc)
    if (cu >= x0 && cu < x1 && row) {
      R uv = um2;  // u_old(cu)
      if (u_row && cu >= 2 && cu <= NX - 2) {
        const R kappa = R(0.5) * (rd0.at(g.damp, cu, L, NX) + rd0.at(g.damp, cu + 1, L, NX)) * dt;
        uv = (R(1.0) - kappa) * um2 - bm2 * (c1 * (pm1 - pm2) + c2 * (pc - pm3));
      }
      const size_t ku = (size_t)(cu - 1) * LD + (iz - 1);
      u1[ku] = uv;
      if (b) {
        const int jx = cu - L, jz = iz - L;
        if (jx >= 1 && jx <= g.nx) {
          if (iz == fs) b[so.T3 + jx - 1] = uv;
          if (iz == fs + 1) b[so.T4 + jx - 1] = uv;
        }
        if (jz >= 1 && jz <= g.nz) {
          if (cu == L + 1) b[so.S2 + jz - 1] = uv;
          if (cu == NX - L - 1) b[so.S5 + jz - 1] = uv;
        }
      }
    }
    um2 = um1;
    um1 = uc;
    uc = up1;
  }
}

// ---------------------------------------------------------------------------
// Reverse step `it`: adjoint (fdcore.f90:309-373) from (PB0,UB0,WB0) into
// (PB1,UB1,WB1); reconstruction (fdcore.f90:220-287) from (PE0,UE0,WE0) into
// (PE1,UE1,WE1); imaging sums updated in place (solver.f90:237-239).
// Shared memory: four columns of LD+4 values (pb_old, wb_new, pe_old, we_new).
template <class R, int TX>
__global__ void __launch_bounds__(1024) k_bwd_step(
    Grid<R> g, Sources src, Receivers rec, const R* __restrict__ s_fwd, const R* __restrict__ adj_t,
    const R* __restrict__ PB0, const R* __restrict__ UB0, const R* __restrict__ WB0, R* __restrict__ PB1,
    R* __restrict__ UB1, R* __restrict__ WB1, const R* __restrict__ PE0, const R* __restrict__ UE0,
    const R* __restrict__ WE0, R* __restrict__ PE1, R* __restrict__ UE1, R* __restrict__ WE1, R* __restrict__ DG,
    R* __restrict__ DFW, R* __restrict__ DBK, const R* __restrict__ strips, int it, int shot0) {
  extern __shared__ unsigned char smem_raw[];
  R* cpb = reinterpret_cast<R*>(smem_raw);
  R* cwb = cpb + (g.LD + 4);
  R* cpe = cwb + (g.LD + 4);
  R* cwe = cpe + (g.LD + 4);
  const int iz = threadIdx.x + 1;
  const int s = shot0 + blockIdx.y;
  const int NX = g.NX, NZ = g.NZ, L = g.L, LD = g.LD, fs = g.fs, nx = g.nx, nz = g.nz, LDI = g.LDI;
  const int x0 = blockIdx.x * TX + 1;
  const int x1 = min(x0 + TX, NX + 1);
  const bool row = iz <= NZ;
  const size_t off = (size_t)s * g.FSZ, offi = (size_t)s * g.FSI;
  const R *pb0 = PB0 + off, *ub0 = UB0 + off, *wb0 = WB0 + off;
  R *pb1 = PB1 + off, *ub1 = UB1 + off, *wb1 = WB1 + off;
  const R *pe0 = PE0 + offi, *ue0 = UE0 + offi, *we0 = WE0 + offi;
  R *pe1 = PE1 + offi, *ue1 = UE1 + offi, *we1 = WE1 + offi;
  R *dg = DG + offi, *dfw = DFW + offi, *dbk = DBK + offi;
  const R dt = g.dt, c1 = g.c1, c2 = g.c2;
  RowDamp<R> rd0, rd1;
  rd0.init(g.damp, iz, L, NX, NZ);
  rd1.init(g.damp, iz + 1, L, NX, NZ);
  const bool fsf = g.fs_flag == 1;
  // adjoint ranges (fdcore.f90:310-311, 319-320, 336-337)
  const bool ub_row = iz >= 2 && iz <= NZ - 1;
  const bool wb_row = iz >= 2 && iz <= NZ - 2;
  const bool pb_row = iz >= 3 && iz <= NZ - 2;
  // reconstruction rows (interior indices), fs' = fs - L
  const int jz = iz - L, fsi = fs - L;
  const bool irow = row && jz >= 1 && jz <= nz;
  const bool ue_row = jz >= fsi + 1 && jz <= nz - 1;
  const bool we_row = jz >= fsi + 1 && jz <= nz - 2;
  const bool pe_row = jz >= fsi + 2 && jz <= nz - 2;
  const R* b = strips + ((size_t)s * g.snt + (it - 1 - g.sit0)) * g.SL;  // boundary(:, it-1)
  const StripOff so = strip_offsets(nx, nz);
  const int* cp = rec.colptr + (size_t)s * (NX + 2);
  const R* adj = adj_t + ((size_t)s * g.nt + (it - 1)) * g.ngmax;
  const int risx = src.risx[s], risz = src.risz[s];
  const R ssub = g.dt * s_fwd[(size_t)s * (g.nt + 1) + it];  // dt s(it+1)

  auto ldi = [&](const R* f, int jx) -> R {  // interior field at (jz, jx)
    return (irow && jx >= 1 && jx <= nx) ? f[(size_t)(jx - 1) * LDI + (jz - 1)] : R(0);
  };
  // windows at step c: pb_old(c..c+3), ub_new(c-2..c+1), pe_old(c..c+3), ue_new(c-2..c+1)
  R pb_0 = ld_col(pb0, x0 - 3, NX, LD, iz, row), pb_1 = ld_col(pb0, x0 - 2, NX, LD, iz, row);
  R pb_2 = ld_col(pb0, x0 - 1, NX, LD, iz, row), pb_3;
  R pe_0 = ldi(pe0, x0 - 3 - L), pe_1 = ldi(pe0, x0 - 2 - L), pe_2 = ldi(pe0, x0 - 1 - L), pe_3;
  R ubm2 = R(0), ubm1 = R(0), ubc = R(0), ubp1;
  R uem2 = R(0), uem1 = R(0), uec = R(0), uep1;

  for (int c = x0 - 3; c < x1; ++c) {
    // ---- phase 1: loads; u updates of column c+1; pb_old(c), pe_old(c) to smem
    pb_3 = ld_col(pb0, c + 3, NX, LD, iz, row);
    pe_3 = ldi(pe0, c + 3 - L);
    {
      const int cu = c + 1;
      const bool ok = row && cu >= 1 && cu <= NX;
      const size_t ku = (size_t)(cu - 1) * LD + (iz - 1);
      R uv = ok ? ub0[ku] : R(0);
      if (ok && ub_row && cu >= 2 && cu <= NX - 2) {
        const R alpha = g.A[ku];
        const R kappa = R(0.5) * (rd0.at(g.damp, cu, L, NX) + rd0.at(g.damp, cu + 1, L, NX)) * dt;
        uv = (R(1.0) - kappa) * uv - alpha * (c1 * (pb_2 - pb_1) + c2 * (pb_3 - pb_0));
      }
      ubp1 = uv;
      if (ok && cu >= x0 && cu < x1) ub1[ku] = uv;
      const int jx = cu - L;
      R ue = ldi(ue0, jx);
      if (irow && jx >= 2 && jx <= nx - 2 && ue_row) {
        const R alpha = g.B[ku];
        ue = ue + alpha * (c1 * (pe_2 - pe_1) + c2 * (pe_3 - pe_0));
      }
      if (irow && jx == 1) ue = b[so.S2 + jz - 1];
      if (irow && jx == nx - 1) ue = b[so.S5 + jz - 1];
      uep1 = ue;
      if (irow && jx >= 1 && jx <= nx && cu >= x0 && cu < x1) ue1[(size_t)(jx - 1) * LDI + (jz - 1)] = ue;
    }
    cpb[iz + 1] = pb_0;  // pb_old(c)
    cpe[iz + 1] = pe_0;  // pe_old(c) (zero outside the interior)
    const bool own = c >= x0 && row;
    const size_t k = (size_t)(c - 1) * LD + (iz - 1);
    const int jx = c - L;
    const bool icol = irow && jx >= 1 && jx <= nx;
    const size_t ki = (size_t)(jx - 1) * LDI + (jz - 1);
    __syncthreads();
    // ---- phase 2: w updates of column c
    R wbv = R(0), wev = R(0);
    if (own) {
      wbv = wb0[k];
      if (wb_row && c >= 2 && c <= NX - 1) {
        const R alpha = g.A[k];
        const R kappa = R(0.5) * (rd0.at(g.damp, c, L, NX) + rd1.at(g.damp, c, L, NX)) * dt;
        wbv = (R(1.0) - kappa) * wbv - alpha * (c1 * (cpb[iz + 2] - cpb[iz + 1]) + c2 * (cpb[iz + 3] - cpb[iz]));
      }
      if (icol) {
        wev = we0[ki];
        if (jx >= 2 && jx <= nx - 1 && we_row) {
          const R alpha = g.B[k];
          wev = wev + alpha * (c1 * (cpe[iz + 2] - cpe[iz + 1]) + c2 * (cpe[iz + 3] - cpe[iz]));
        }
        if (jz == nz - 1) wev = b[so.B2 + jx - 1];
      }
    }
    cwb[iz + 1] = wbv;
    cwe[iz + 1] = wev;
    __syncthreads();
    // ---- phase 3: p updates of column c, stores, imaging
    if (own) {
      // w_b(fs-1, c) = w_b(fs, c) for c in [2, NX-1] (fdcore.f90:329-333)
      const bool wmir = fsf && c >= 2 && c <= NX - 1;
      auto wz = [&](int r) -> R { return (wmir && r == fs - 1) ? cwb[fs + 1] : cwb[r + 1]; };
      if (!(wmir && iz == fs - 1)) wb1[k] = wbv;
      if (wmir && iz == fs) wb1[k - 1] = wbv;
      const R pold = pb_0;
      R pv = pold;
      if (pb_row && c >= 3 && c <= NX - 2) {
        const R alpha = g.B[k];
        const R kappa = rd0.at(g.damp, c, L, NX) * dt;
        pv = (R(1.0) - kappa) * pold - alpha * (c1 * (ubc - ubm1 + wz(iz) - wz(iz - 1)) +
                                                c2 * (ubp1 - ubm2 + wz(iz + 1) - wz(iz - 2)));
      }
      for (int e = cp[c]; e < cp[c + 1]; ++e)
        if (rec.zrow[e] == iz) pv = pv + dt * adj[rec.ig[e]];
      if (iz != fs - 1) pb1[k] = pv;
      if (iz == fs + 1) pb1[k - 2] = -pv;  // p(fs-1) = -p(fs+1), all columns (fdcore.f90:370-373)
      if (icol) {
        we1[ki] = wev;
        R pf = pe_0;
        if (jx == risx && jz == risz) pf = pf - ssub;
        if (jx >= 3 && jx <= nx - 2 && pe_row) {
          const R alpha = g.A[k];
          pf = pf + alpha * (c1 * (uec - uem1 + cwe[iz + 1] - cwe[iz]) + c2 * (uep1 - uem2 + cwe[iz + 2] - cwe[iz - 1]));
        }
        if (jz == nz) pf = b[so.B0 + jx - 1];
        if (jz == nz - 1) pf = b[so.B1 + jx - 1];
        if (jx == 1) pf = b[so.S0 + jz - 1];
        if (jx == 2) pf = b[so.S1 + jz - 1];
        if (jx == nx) pf = b[so.S3 + jz - 1];
        if (jx == nx - 1) pf = b[so.S4 + jz - 1];
        if (jz == fsi) pf = b[so.T0 + jx - 1];
        if (jz == fsi + 1) pf = b[so.T1 + jx - 1];
        if (jz == fsi + 2) pf = b[so.T2 + jx - 1];
        pe1[ki] = pf;
        dg[ki] = dg[ki] + pf * (pold - pv);
        dfw[ki] = dfw[ki] + pf * pf;
        dbk[ki] = dbk[ki] + pv * pv;
      }
    }
    // slide windows
    pb_0 = pb_1;
    pb_1 = pb_2;
    pb_2 = pb_3;
    pe_0 = pe_1;
    pe_1 = pe_2;
    pe_2 = pe_3;
    ubm2 = ubm1;
    ubm1 = ubc;
    ubc = ubp1;
    uem2 = uem1;
    uem1 = uec;
    uec = uep1;
  }
}

}  // namespace swit
