// kernels_walk.cuh -- one launch per time step, each warp walking a tile of
// columns along x.
//
// Geometry.  A warp holds 32 consecutive 4-row vectors of one column: lane l of
// warp wz holds vector q = 28 wz + l - 2 (rows 4q+1 .. 4q+4).  Lanes 2..29 own
// their vector (they store it); lanes 0, 1, 30, 31 are halo lanes that compute
// the same updates so that the owners get their z-neighbours by warp shuffle:
// a step's second phase needs the first phase's values one vector up and
// down, and those need the old values one vector further out.  ceil(nvec/28)
// warps cover a column (nvec = LD/4).  A CTA is the warps of one column range;
// it walks the columns of its tile [x0, x0+TX) left to right (plus the halo
// columns the x-stencils need), keeping the x-neighbours of every field in
// register windows, so each vector of each field is loaded once per step.
//
// State is double-buffered: a step reads the old arrays and writes the new
// ones, so tiles never race on each other's halo columns.  Every owned vector
// is stored every step (points the reference does not update are copied
// through); the new arrays therefore hold the full state after the step.
//
// Arithmetic is that of kernels_vec.cuh: the same expressions in the same order
// (fdcore.f90), no FMA.  The damping factors are evaluated from the damping
// table in the order k_kappa uses, so results are bit-identical to the other
// variants and to the oracle.
#pragma once
#include "kernels_vec.cuh"

namespace swit {

constexpr int kWalkOwn = 28;   // owned vectors per warp (lanes 2..29)
constexpr int kWalkWarps = 2;  // warps per CTA (blockDim.y); blockIdx.z selects the warp group

// Resident 64-thread CTAs per SM the FP32 walk kernels are compiled for (caps
// their registers at 65536 / (64 * SWIT_WALK_MINB)); the FP64 builds are not capped.
#ifndef SWIT_WALK_MINB
#define SWIT_WALK_MINB 10
#endif
#define SWIT_WALK_MINB_R(R) (sizeof(R) == 4 ? SWIT_WALK_MINB : 1)
// Unrolling of the column walks.  Measured at 481x141 (49 shots, 8-column
// tiles, 25-shot batches): 1 (no unrolling) 70.8, 2: 58.8, 4: 56.3
// shot-gradients/s -- larger bodies stall on instruction fetch.
#ifndef SWIT_WALK_UNROLL
#define SWIT_WALK_UNROLL 1
#endif
#define SWIT_PRAGMA(x) _Pragma(#x)
#define SWIT_UNROLL(n) SWIT_PRAGMA(unroll n)

template <class R>
__device__ __forceinline__ R shup(R v) {
  return __shfl_up_sync(0xffffffffu, v, 1);
}
template <class R>
__device__ __forceinline__ R shdn(R v) {
  return __shfl_down_sync(0xffffffffu, v, 1);
}

// Element j (0..3, a run-time value) of a vector without indexing the register
// array at run time (which would place it in local memory).
template <class R>
__device__ __forceinline__ R vget(const V4<R>& v, int j) {
  R r = v.x[0];
#pragma unroll
  for (int i = 1; i < 4; ++i)
    if (j == i) r = v.x[i];
  return r;
}

// Damping of the rows iz0 .. iz0+4 of one lane along the columns
// (pml.f90:88-99, damp_at in kernels.cuh): a row in the top or bottom PML has
// the value v on its trapezoid span [lo, hi]; everywhere else the value is the
// side profile of the column.
template <class R>
struct LaneDamp {
  int lo[5], hi[5];
  R v[5];
  __device__ void init(const R* damp, int iz0, int L, int NX, int NZ) {
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      const int iz = iz0 + r;
      lo[r] = 1;
      hi[r] = 0;
      v[r] = R(0);
      if (iz >= 1 && iz <= L) {
        lo[r] = iz + 1;
        hi[r] = NX - iz;
        v[r] = damp[L - iz + 1];
      } else if (iz >= NZ - L + 1 && iz <= NZ) {
        const int k = iz - NZ + L;
        lo[r] = L - k + 2;
        hi[r] = NX - L + k - 1;
        v[r] = damp[k];
      }
    }
  }
  // damp(iz0 + r, c) given the column's side value
  __device__ __forceinline__ R at(int r, int c, R side) const { return (c >= lo[r] && c <= hi[r]) ? v[r] : side; }
};

template <class R>
__device__ __forceinline__ R side_damp(const R* damp, int c, int L, int NX) {
  if (c <= L) return c >= 1 ? damp[L - c + 1] : R(0);
  if (c >= NX - L + 1) return c <= NX ? damp[c - (NX - L)] : R(0);
  return R(0);
}

// Lane and tile of the calling thread.
struct WalkIdx {
  int lane, wz, q, iz0, s, x0, xe;
  bool qok, own;
};
template <class R>
__device__ __forceinline__ WalkIdx walk_index(const Grid<R>& g, int TX, int shot0) {
  WalkIdx w;
  w.lane = threadIdx.x;
  w.wz = (int)(blockIdx.z * blockDim.y + threadIdx.y);
  w.q = kWalkOwn * w.wz + w.lane - 2;
  w.iz0 = 4 * w.q + 1;
  const int nvec = g.LD >> 2;
  w.qok = w.q >= 0 && w.q < nvec;
  w.own = w.qok && w.lane >= 2 && w.lane <= 29;
  w.s = shot0 + blockIdx.y;
  w.x0 = blockIdx.x * TX + 1;
  w.xe = min(w.x0 + TX, g.NX + 1);
  return w;
}

// Boundary-strip entries of one vector (fdcore.f90:130-159) at column c: the
// pressure and w entries (PW) or the u entries (!PW).
template <class R, bool PW>
__device__ __forceinline__ void walk_strips(const Grid<R>& g, R* __restrict__ bs, int c, int iz0, const V4<R>& pv,
                                            const V4<R>& wv) {
  const StripOff o = strip_offsets(g.nx, g.nz);
  const int L = g.L, NX = g.NX, NZ = g.NZ, fs = g.fs, jx = c - L;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int iz = iz0 + r, jz = iz - L;
    if (jx >= 1 && jx <= g.nx) {
      if constexpr (PW) {
        if (iz == NZ - L) bs[o.B0 + jx - 1] = pv.x[r];
        if (iz == NZ - L - 1) {
          bs[o.B1 + jx - 1] = pv.x[r];
          bs[o.B2 + jx - 1] = wv.x[r];
        }
        if (iz == fs) {
          bs[o.T0 + jx - 1] = pv.x[r];
          bs[o.T5 + jx - 1] = wv.x[r];
        }
        if (iz == fs + 1) bs[o.T1 + jx - 1] = pv.x[r];
        if (iz == fs + 2) bs[o.T2 + jx - 1] = pv.x[r];
      } else {
        if (iz == fs) bs[o.T3 + jx - 1] = pv.x[r];
        if (iz == fs + 1) bs[o.T4 + jx - 1] = pv.x[r];
      }
    }
    if (jz >= 1 && jz <= g.nz) {
      if constexpr (PW) {
        if (c == L + 1) bs[o.S0 + jz - 1] = pv.x[r];
        if (c == L + 2) bs[o.S1 + jz - 1] = pv.x[r];
        if (c == NX - L) bs[o.S3 + jz - 1] = pv.x[r];
        if (c == NX - L - 1) bs[o.S4 + jz - 1] = pv.x[r];
      } else {
        if (c == L + 1) bs[o.S2 + jz - 1] = pv.x[r];
        if (c == NX - L - 1) bs[o.S5 + jz - 1] = pv.x[r];
      }
    }
  }
}

// Records of the receivers in a column whose row lies in this lane's vector
// (fdcore.f90:123-128; vx / vz after dev/solver/fdcore.f90:162-175), in
// receiver order, from the column's table entry rc = rcol[c] (loaded with the
// iteration's other loads, so the common one-receiver column adds no
// dependent load).
template <class R>
__device__ __forceinline__ void walk_record1(const Grid<R>& g, const Receivers& rec, R* __restrict__ seis_t, int s,
                                             int it, int iz0, int4 rc, const V4<R>& v) {
  if (rc.z == 1) {
    const int j = rc.y - iz0;
    if (j >= 0 && j < 4) seis_t[((size_t)s * g.nt + (it - 1)) * g.ngmax + rc.x] = vget(v, j);
  } else {
    for (int e = rc.w; e < rc.w + rc.z; ++e) {
      const int j = rec.zrow[e] - iz0;
      if (j >= 0 && j < 4) seis_t[((size_t)s * g.nt + (it - 1)) * g.ngmax + rec.ig[e]] = vget(v, j);
    }
  }
}

// Vector of column c of a field whose column-1 vector of this lane is at f
// (c-1 columns of LD values further on), or zeros when ok is false.
template <class R>
__device__ __forceinline__ V4<R> ldc(const R* __restrict__ f, int c, int LD, bool ok) {
  V4<R> v;
  if (ok) {
    const R* a = f + (ptrdiff_t)(c - 1) * LD;
    if constexpr (sizeof(R) == 4) {
      const float4 t = __ldg(reinterpret_cast<const float4*>(a));
      v.x[0] = t.x;
      v.x[1] = t.y;
      v.x[2] = t.z;
      v.x[3] = t.w;
    } else {
      const double2 t0 = __ldg(reinterpret_cast<const double2*>(a));
      const double2 t1 = __ldg(reinterpret_cast<const double2*>(a) + 1);
      v.x[0] = t0.x;
      v.x[1] = t0.y;
      v.x[2] = t1.x;
      v.x[3] = t1.y;
    }
  } else {
#pragma unroll
    for (int r = 0; r < 4; ++r) v.x[r] = R(0);
  }
  return v;
}
template <class R>
__device__ __forceinline__ void stc(R* __restrict__ f, int c, int LD, const V4<R>& v) {
  R* a = f + (ptrdiff_t)(c - 1) * LD;
  if constexpr (sizeof(R) == 4) {
    *reinterpret_cast<float4*>(a) = make_float4(v.x[0], v.x[1], v.x[2], v.x[3]);
  } else {
    reinterpret_cast<double2*>(a)[0] = make_double2(v.x[0], v.x[1]);
    reinterpret_cast<double2*>(a)[1] = make_double2(v.x[2], v.x[3]);
  }
}

// Bit r set when row iz0 + r lies in [lo, hi].
__device__ __forceinline__ int row_mask(int iz0, int lo, int hi) {
  int m = 0;
#pragma unroll
  for (int r = 0; r < 4; ++r)
    if (iz0 + r >= lo && iz0 + r <= hi) m |= 1 << r;
  return m;
}

// ---------------------------------------------------------------------------
// Forward step `it` (fdcore.f90:77-159) of one tile: pressure update, source,
// p(fs-1) mirror, u and w updates, w(fs-1) mirror, receiver records and strips,
// from (P0, U0, W0) into (P1, U1, W1).  Walk position j: p and w of column j,
// u of column j-2 (its stencil needs the new p of columns j-3 .. j).
//
// Per lane the rows each update covers are bit masks, and the damping factors
// of the columns without side damping ([L+1, NX-L], where only the row's own
// profile acts) are computed once; the update is evaluated for all four rows
// and selected by the mask, so a warp never branches on its lane's rows.
template <class R>
__global__ void __launch_bounds__(64, SWIT_WALK_MINB_R(R)) k_fwd_walk(Grid<R> g, Sources src, Receivers rec, const R* __restrict__ s_fwd,
                                                 const R* __restrict__ P0, const R* __restrict__ U0,
                                                 const R* __restrict__ W0, R* __restrict__ P1, R* __restrict__ U1,
                                                 R* __restrict__ W1, R* __restrict__ seis_t, R* __restrict__ strips,
                                                 int it, int shot0, int TX) {
  const WalkIdx w = walk_index(g, TX, shot0);
  pdl_enter();
  if (kWalkOwn * w.wz >= (g.LD >> 2)) return;  // a whole warp past the column (odd warp count)
  const int LD = g.LD, NX = g.NX, NZ = g.NZ, L = g.L, fs = g.fs, iz0 = w.iz0;
  const bool qok = w.qok;
  const size_t off = (size_t)w.s * g.FSZ + 4 * (size_t)(qok ? w.q : 0);
  const R *p0 = P0 + off, *u0 = U0 + off, *w0 = W0 + off, *ca = g.A + (off - (size_t)w.s * g.FSZ),
          *cb = g.B + (off - (size_t)w.s * g.FSZ);
  R *p1 = P1 + off, *u1 = U1 + off, *w1 = W1 + off;
  LaneDamp<R> ld;
  ld.init(g.damp, iz0, L, NX, NZ);
  const R dt = g.dt, c1 = g.c1, c2 = g.c2;
  R kpi[4], kui[4], kwi[4];  // damping of columns [L+1, NX-L] (u: [L+1, NX-L-1])
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    kpi[r] = ld.v[r] * dt;
    kui[r] = R(0.5) * (ld.v[r] + ld.v[r]) * dt;
    kwi[r] = R(0.5) * (ld.v[r] + ld.v[r + 1]) * dt;
  }
  const int pm = row_mask(iz0, fs + 1, NZ - 2), um = row_mask(iz0, fs, NZ - 1), wm = row_mask(iz0, fs, NZ - 2);
  const int isx = src.isx[w.s], js = src.isz[w.s] - iz0;
  const R sval = (js >= 0 && js < 4) ? dt * s_fwd[(size_t)w.s * (g.nt + 1) + (it - 1)] : R(0);
  const int jm = fs - 1 - iz0;  // row fs-1 in this vector (rows fs, fs+1 follow it)
  const bool mir = g.fs_flag == 1 && jm >= 0 && jm < 4;
  const bool rec_rows = w.own && iz0 + 3 >= rec.zlo[w.s] && iz0 <= rec.zhi[w.s];
  R* bs = strips ? strips + ((size_t)w.s * g.snt + (it - g.sit0)) * g.SL : nullptr;
  const bool strip_rows = (iz0 <= fs + 2 && iz0 + 3 >= fs) || (iz0 <= NZ - L && iz0 + 3 >= NZ - L - 1);
  const int4 none = make_int4(-1, -1, 0, 0);
  const int4* rcol = rec.rcol + (size_t)w.s * (NX + 2);

  const int x0 = w.x0, xe = w.xe;
  V4<R> um2 = ldc(u0, x0 - 3, LD, qok && x0 - 3 >= 1), um1 = ldc(u0, x0 - 2, LD, qok && x0 - 2 >= 1),
        u00 = ldc(u0, x0 - 1, LD, qok && x0 - 1 >= 1);
  V4<R> pm3, pm2, pm1;  // new p of columns j-3, j-2, j-1
#pragma unroll
  for (int r = 0; r < 4; ++r) pm3.x[r] = pm2.x[r] = pm1.x[r] = R(0);
  SWIT_UNROLL(SWIT_WALK_UNROLL)
  for (int j = x0 - 1; j <= xe + 1; ++j) {
    const bool cok = qok && j >= 1 && j <= NX;
    const int4 rc = rec_rows && rec.comp != 1 && j >= x0 && j < xe ? rcol[j] : none;
    const int4 ru = rec_rows && rec.comp == 1 && j - 2 >= x0 && j - 2 < xe ? rcol[j - 2] : none;
    const V4<R> up1 = ldc(u0, j + 1, LD, qok && j + 1 <= NX);
    const V4<R> po = ldc(p0, j, LD, cok), wo = ldc(w0, j, LD, cok);
    const V4<R> a = ldc(ca, j, LD, cok), b = ldc(cb, j, LD, cok);
    const bool dint = j >= L + 1 && j <= NX - L;  // no side damping in column j
    // ---- pressure (fdcore.f90:77-84); w rows iz0-2 .. iz0+4
    R wz[7];
    wz[0] = shup(wo.x[2]);
    wz[1] = shup(wo.x[3]);
    wz[2] = wo.x[0];
    wz[3] = wo.x[1];
    wz[4] = wo.x[2];
    wz[5] = wo.x[3];
    wz[6] = shdn(wo.x[0]);
    V4<R> pn = po;
    if (j >= 3 && j <= NX - 2) {
      R kp[4];
      if (dint) {
#pragma unroll
        for (int r = 0; r < 4; ++r) kp[r] = kpi[r];
      } else {
        const R sj = side_damp(g.damp, j, L, NX);
#pragma unroll
        for (int r = 0; r < 4; ++r) kp[r] = ld.at(r, j, sj) * dt;
      }
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const R D = c1 * (u00.x[r] - um1.x[r] + wz[r + 2] - wz[r + 1]) + c2 * (up1.x[r] - um2.x[r] + wz[r + 3] - wz[r]);
        const R t = (R(1.0) - kp[r]) * po.x[r] - a.x[r] * D;
        if ((pm >> r) & 1) pn.x[r] = t;
      }
    }
    // source (fdcore.f90:87-88) and p(fs-1,:) = -p(fs+1,:) (fdcore.f90:91-93)
    if (j == isx) {
#pragma unroll
      for (int r = 0; r < 4; ++r)
        if (r == js) pn.x[r] = pn.x[r] + sval;
    }
    {
      const R n0 = shdn(pn.x[0]), n1 = shdn(pn.x[1]);
      if (mir) {
#pragma unroll
        for (int r = 0; r < 4; ++r)
          if (r == jm) pn.x[r] = -(r + 2 < 4 ? pn.x[(r + 2) & 3] : (r + 2 == 4 ? n0 : n1));
      }
    }
    const bool cown = w.own && j >= x0 && j < xe;
    if (cown) stc(p1, j, LD, pn);
    // ---- w (fdcore.f90:105-113); new p rows iz0-1 .. iz0+5
    R pz[7];
    pz[0] = shup(pn.x[3]);
    pz[1] = pn.x[0];
    pz[2] = pn.x[1];
    pz[3] = pn.x[2];
    pz[4] = pn.x[3];
    pz[5] = shdn(pn.x[0]);
    pz[6] = shdn(pn.x[1]);
    V4<R> wn = wo;
    if (j >= 2 && j <= NX - 1) {
      R kw[4];
      if (dint) {
#pragma unroll
        for (int r = 0; r < 4; ++r) kw[r] = kwi[r];
      } else {
        const R sj = side_damp(g.damp, j, L, NX);
#pragma unroll
        for (int r = 0; r < 4; ++r) kw[r] = R(0.5) * (ld.at(r, j, sj) + ld.at(r + 1, j, sj)) * dt;
      }
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const R t = (R(1.0) - kw[r]) * wo.x[r] - b.x[r] * (c1 * (pz[r + 2] - pz[r + 1]) + c2 * (pz[r + 3] - pz[r]));
        if ((wm >> r) & 1) wn.x[r] = t;
      }
    }
    // w(fs-1, ix) = w(fs, ix) for every column (fdcore.f90:116-120)
    {
      const R n0 = shdn(wn.x[0]);
      if (mir) {
#pragma unroll
        for (int r = 0; r < 4; ++r)
          if (r == jm) wn.x[r] = r + 1 < 4 ? wn.x[(r + 1) & 3] : n0;
      }
    }
    if (cown) {
      stc(w1, j, LD, wn);
      if (rc.z) walk_record1(g, rec, seis_t, w.s, it, iz0, rc, rec.comp == 2 ? wn : pn);
      if (bs && (strip_rows || j == L + 1 || j == L + 2 || j == NX - L || j == NX - L - 1))
        walk_strips<R, true>(g, bs, j, iz0, pn, wn);
    }
    // ---- u of column jj = j - 2 (fdcore.f90:96-104)
    const int jj = j - 2;
    if (jj >= x0 && jj < xe) {
      V4<R> un = um2;
      if (jj >= 2 && jj <= NX - 2) {
        const V4<R> bu = ldc(cb, jj, LD, qok);
        R ku[4];
        if (jj >= L + 1 && jj <= NX - L - 1) {
#pragma unroll
          for (int r = 0; r < 4; ++r) ku[r] = kui[r];
        } else {
          const R s0 = side_damp(g.damp, jj, L, NX), s1 = side_damp(g.damp, jj + 1, L, NX);
#pragma unroll
          for (int r = 0; r < 4; ++r) ku[r] = R(0.5) * (ld.at(r, jj, s0) + ld.at(r, jj + 1, s1)) * dt;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const R t = (R(1.0) - ku[r]) * um2.x[r] - bu.x[r] * (c1 * (pm1.x[r] - pm2.x[r]) + c2 * (pn.x[r] - pm3.x[r]));
          if ((um >> r) & 1) un.x[r] = t;
        }
      }
      if (w.own) {
        stc(u1, jj, LD, un);
        if (ru.z) walk_record1(g, rec, seis_t, w.s, it, iz0, ru, un);
        if (bs && (strip_rows || jj == L + 1 || jj == NX - L - 1)) walk_strips<R, false>(g, bs, jj, iz0, un, un);
      }
    }
    um2 = um1;
    um1 = u00;
    u00 = up1;
    pm3 = pm2;
    pm2 = pm1;
    pm1 = pn;
  }
}

// Adjoint sources of the receivers in column c whose injection row lies in
// this lane's vector, added in receiver order (sign +1: pressure,
// fdcore.f90:345-362; -1: vx / vz, dev/solver/fdcore.f90:472-485).
template <class R>
__device__ __forceinline__ void walk_inject(const Grid<R>& g, const Receivers& rec, const R* __restrict__ adj_t,
                                            int s, int it, int c, int iz0, V4<R>& v, bool minus) {
  const int* cp = rec.colptr + (size_t)s * (g.NX + 2);
  const int e1 = cp[c + 1];
  for (int e = cp[c]; e < e1; ++e) {
    const int j = rec.zrow[e] - iz0;
    if (j >= 0 && j < 4) {
      const R a = g.dt * adj_t[((size_t)s * g.nt + (it - 1)) * g.ngmax + rec.ig[e]];
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (i == j) v.x[i] = minus ? v.x[i] - a : v.x[i] + a;
    }
  }
}

// ---------------------------------------------------------------------------
// Reverse step `it` of one tile (solver.f90:230-239): the reconstruction step
// (fdcore.f90:202-287) on the interior fields (PML-grid layout, interior point
// (jz, jx) at row jz+L, column jx+L) from (PE0, UE0, WE0) into (PE1, UE1, WE1),
// then the adjoint step (fdcore.f90:293-373) from (PB0, UB0, WB0) into
// (PB1, UB1, WB1) with the imaging sums (solver.f90:237-239) updated in place.
// Each walk at position j updates the velocities of column j and the pressure
// of column j-1 (its stencil needs the new velocities of columns j-3 .. j).
// Rows are selected by per-lane masks as in k_fwd_walk.
template <class R>
__global__ void __launch_bounds__(64, SWIT_WALK_MINB_R(R)) k_bwd_walk(Grid<R> g, Sources src, Receivers rec,
                                                 const R* __restrict__ s_fwd, const R* __restrict__ adj_t,
                                                 const R* __restrict__ PB0, const R* __restrict__ UB0,
                                                 const R* __restrict__ WB0, R* __restrict__ PB1, R* __restrict__ UB1,
                                                 R* __restrict__ WB1, const R* __restrict__ PE0,
                                                 const R* __restrict__ UE0, const R* __restrict__ WE0, R* PE1,
                                                 R* __restrict__ UE1, R* __restrict__ WE1, R* __restrict__ DG,
                                                 R* __restrict__ DFW, R* __restrict__ DBK,
                                                 const R* __restrict__ strips, int it, int shot0, int TX) {
  const WalkIdx w = walk_index(g, TX, shot0);
  pdl_enter();
  if (kWalkOwn * w.wz >= (g.LD >> 2)) return;  // a whole warp past the column (odd warp count)
  const int LD = g.LD, NX = g.NX, NZ = g.NZ, L = g.L, fs = g.fs, iz0 = w.iz0;
  const int nx = g.nx, nz = g.nz, fsi = fs - L, jz0 = iz0 - L;
  const bool qok = w.qok;
  const size_t lane_off = 4 * (size_t)(qok ? w.q : 0), off = (size_t)w.s * g.FSZ + lane_off;
  const R *ca = g.A + lane_off, *cb = g.B + lane_off;
  const R dt = g.dt, c1 = g.c1, c2 = g.c2;
  const int x0 = w.x0, xe = w.xe;
  const StripOff o = strip_offsets(nx, nz);
  const R* bs = strips + ((size_t)w.s * g.snt + (it - 1 - g.sit0)) * g.SL;  // boundary(:, it-1)
  const int irow = row_mask(jz0, 1, nz);  // interior rows of this vector

  // ================= reconstruction (interior, undamped)
  // columns whose new pressure this tile owns on the interior: [cx0, cx1)
  const int cx0 = max(x0, L + 1), cx1 = min(xe, L + nx + 1);
  const bool rows_in = iz0 + 3 + 8 >= L + 1 && iz0 - 8 <= L + nz;  // this lane or a neighbour it feeds
  if (cx0 < cx1 && __any_sync(0xffffffffu, rows_in)) {
    const R* pe0 = PE0 + off;
    const R* ue0 = UE0 + off;
    const R* we0 = WE0 + off;
    R* pe1 = PE1 + off;
    R* ue1 = UE1 + off;
    R* we1 = WE1 + off;
    const int um = row_mask(jz0, fsi + 1, nz - 1), wm = row_mask(jz0, fsi + 1, nz - 2),
              pm = row_mask(jz0, fsi + 2, nz - 2);
    const bool wins = irow & row_mask(jz0, nz - 1, nz - 1);               // w(nz-1, :) re-insert
    const bool pins = irow & (row_mask(jz0, nz - 1, nz) | row_mask(jz0, fsi, fsi + 2));  // p row re-inserts
    const int rsx = src.risx[w.s], rj = src.risz[w.s] - jz0;
    const R rsv = (rj >= 0 && rj < 4) ? dt * s_fwd[(size_t)w.s * (g.nt + 1) + it] : R(0);
    // interior column range [L+1, L+nx]; the walk covers [cx0-2, cx1] of it
    const int ja = max(cx0 - 2, L + 1), jb = cx1, jl = L + nx;
    V4<R> pem1 = ldc(pe0, ja - 1, LD, qok && ja - 1 >= L + 1), pe00 = ldc(pe0, ja, LD, qok),
          pep1 = ldc(pe0, ja + 1, LD, qok && ja + 1 <= jl);
    V4<R> um3, um2, um1, wprev;
#pragma unroll
    for (int r = 0; r < 4; ++r) um3.x[r] = um2.x[r] = um1.x[r] = wprev.x[r] = R(0);
    SWIT_UNROLL(SWIT_WALK_UNROLL)
    for (int j = ja; j <= jb; ++j) {
      const int jx = j - L;
      const bool cok = qok && j <= jl;
      const V4<R> pep2 = ldc(pe0, j + 2, LD, qok && j + 2 <= jl);
      V4<R> un = ldc(ue0, j, LD, cok);
      V4<R> wn = ldc(we0, j, LD, cok);
      const V4<R> b = ldc(cb, j, LD, qok);
      // u (fdcore.f90:219-225)
      if (jx >= 2 && jx <= nx - 2) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const R t = un.x[r] + b.x[r] * (c1 * (pep1.x[r] - pe00.x[r]) + c2 * (pep2.x[r] - pem1.x[r]));
          if ((um >> r) & 1) un.x[r] = t;
        }
      }
      // w (fdcore.f90:227-233); old p rows iz0-1 .. iz0+5
      R pz[7];
      pz[0] = shup(pe00.x[3]);
      pz[1] = pe00.x[0];
      pz[2] = pe00.x[1];
      pz[3] = pe00.x[2];
      pz[4] = pe00.x[3];
      pz[5] = shdn(pe00.x[0]);
      pz[6] = shdn(pe00.x[1]);
      if (jx >= 2 && jx <= nx - 1) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const R t = wn.x[r] + b.x[r] * (c1 * (pz[r + 2] - pz[r + 1]) + c2 * (pz[r + 3] - pz[r]));
          if ((wm >> r) & 1) wn.x[r] = t;
        }
      }
      // re-insert w(nz-1, :), u(:, 1), u(:, nx-1) from boundary(:, it-1) (fdcore.f90:236-245)
      if (jx >= 1 && jx <= nx) {
        if (wins) {
#pragma unroll
          for (int r = 0; r < 4; ++r)
            if (jz0 + r == nz - 1) wn.x[r] = bs[o.B2 + jx - 1];
        }
        if (jx == 1 || jx == nx - 1) {
          const R* sc = bs + (jx == 1 ? o.S2 : o.S5) - 1;
#pragma unroll
          for (int r = 0; r < 4; ++r)
            if ((irow >> r) & 1) un.x[r] = sc[jz0 + r];
        }
      }
      if (w.own && j >= cx0 && j < cx1) {
        stc(ue1, j, LD, un);
        stc(we1, j, LD, wn);
      }
      // ---- pressure of column jc = j - 1 (fdcore.f90:247-287); new w rows iz0-2 .. iz0+4
      R wz[7];
      wz[0] = shup(wprev.x[2]);
      wz[1] = shup(wprev.x[3]);
      wz[2] = wprev.x[0];
      wz[3] = wprev.x[1];
      wz[4] = wprev.x[2];
      wz[5] = wprev.x[3];
      wz[6] = shdn(wprev.x[0]);
      const int jc = j - 1, jxc = jc - L;
      if (jc >= cx0 && jc < cx1) {
        V4<R> ev = pem1;
        // subtract the source s(it+1) (fdcore.f90:247-255)
        if (jxc == rsx) {
#pragma unroll
          for (int r = 0; r < 4; ++r)
            if (r == rj) ev.x[r] = ev.x[r] - rsv;
        }
        if (jxc >= 3 && jxc <= nx - 2) {
          const V4<R> a = ldc(ca, jc, LD, qok);
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const R t = ev.x[r] + a.x[r] * (c1 * (um1.x[r] - um2.x[r] + wz[r + 2] - wz[r + 1]) +
                                             c2 * (un.x[r] - um3.x[r] + wz[r + 3] - wz[r]));
            if ((pm >> r) & 1) ev.x[r] = t;
          }
        }
        // re-insert p (fdcore.f90:266-285): bottom rows, side columns, top rows
        const bool pcol = jxc == 1 || jxc == 2 || jxc == nx - 1 || jxc == nx;
        if (pins || (pcol && irow)) {
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const int jz = jz0 + r;
            if (jz < 1 || jz > nz) continue;
            if (jz == nz) ev.x[r] = bs[o.B0 + jxc - 1];
            if (jz == nz - 1) ev.x[r] = bs[o.B1 + jxc - 1];
            if (jxc == 1) ev.x[r] = bs[o.S0 + jz - 1];
            if (jxc == 2) ev.x[r] = bs[o.S1 + jz - 1];
            if (jxc == nx) ev.x[r] = bs[o.S3 + jz - 1];
            if (jxc == nx - 1) ev.x[r] = bs[o.S4 + jz - 1];
            if (jz == fsi) ev.x[r] = bs[o.T0 + jxc - 1];
            if (jz == fsi + 1) ev.x[r] = bs[o.T1 + jxc - 1];
            if (jz == fsi + 2) ev.x[r] = bs[o.T2 + jxc - 1];
          }
        }
        if (w.own) stc(pe1, jc, LD, ev);
      }
      um3 = um2;
      um2 = um1;
      um1 = un;
      wprev = wn;
      pem1 = pe00;
      pe00 = pep1;
      pep1 = pep2;
    }
  }

  // ================= adjoint (PML grid, damped) and imaging
  {
    const R* pb0 = PB0 + off;
    const R* ub0 = UB0 + off;
    const R* wb0 = WB0 + off;
    R* pb1 = PB1 + off;
    R* ub1 = UB1 + off;
    R* wb1 = WB1 + off;
    const R* pe1 = PE1 + off;
    R* dg = DG + off;
    R* dfw = DFW + off;
    R* dbk = DBK + off;
    LaneDamp<R> ld;
    ld.init(g.damp, iz0, L, NX, NZ);
    R kpi[4], kui[4], kwi[4];  // damping of columns [L+1, NX-L] (u: [L+1, NX-L-1])
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      kpi[r] = ld.v[r] * dt;
      kui[r] = R(0.5) * (ld.v[r] + ld.v[r]) * dt;
      kwi[r] = R(0.5) * (ld.v[r] + ld.v[r + 1]) * dt;
    }
    const int um = row_mask(iz0, 2, NZ - 1), wm = row_mask(iz0, 2, NZ - 2), pm = row_mask(iz0, 3, NZ - 2);
    const int jm = fs - 1 - iz0;  // row fs-1 in this vector (rows fs, fs+1 follow it)
    const bool rec_rows = w.own && iz0 + 3 >= rec.zlo[w.s] && iz0 <= rec.zhi[w.s];
    const bool wmir = g.fs_flag == 1 && jm >= 0 && jm < 4;
    const bool pmir = jm >= 0 && jm < 4;
    const bool img_rows = w.own && irow != 0;
    V4<R> pm1 = ldc(pb0, x0 - 3, LD, qok && x0 - 3 >= 1), p00 = ldc(pb0, x0 - 2, LD, qok && x0 - 2 >= 1),
          pp1 = ldc(pb0, x0 - 1, LD, qok && x0 - 1 >= 1);
    V4<R> um3, um2, um1, wprev;
#pragma unroll
    for (int r = 0; r < 4; ++r) um3.x[r] = um2.x[r] = um1.x[r] = wprev.x[r] = R(0);
    // pressure receivers: the table entry of column j is loaded at position j
    // and its adjoint source at position j+1, where column j's pressure is updated
    const int4 none = make_int4(-1, -1, 0, 0);
    const int4* rcol = rec.rcol + (size_t)w.s * (NX + 2);
    const R* adj_it = adj_t + ((size_t)w.s * g.nt + (it - 1)) * g.ngmax;
    int4 rcur = none;
    SWIT_UNROLL(SWIT_WALK_UNROLL)
    for (int j = x0 - 2; j <= xe; ++j) {
      const bool cok = qok && j >= 1 && j <= NX;
      const int4 rn = rec_rows && rec.comp == 0 && j >= x0 && j < xe ? rcol[j] : none;
      const int jrc = rcur.z == 1 ? rcur.y - iz0 : -1;
      const R av = (jrc >= 0 && jrc < 4) ? dt * adj_it[rcur.x] : R(0);
      const V4<R> pp2 = ldc(pb0, j + 2, LD, qok && j + 2 >= 1 && j + 2 <= NX);
      const V4<R> uo = ldc(ub0, j, LD, cok), wo = ldc(wb0, j, LD, cok);
      const V4<R> a = ldc(ca, j, LD, cok);
      const bool dint = j >= L + 1 && j <= NX - L;
      // u (fdcore.f90:309-316)
      V4<R> un = uo;
      if (j >= 2 && j <= NX - 2) {
        R ku[4];
        if (j <= NX - L - 1 && dint) {
#pragma unroll
          for (int r = 0; r < 4; ++r) ku[r] = kui[r];
        } else {
          const R sj = side_damp(g.damp, j, L, NX), sj1 = side_damp(g.damp, j + 1, L, NX);
#pragma unroll
          for (int r = 0; r < 4; ++r) ku[r] = R(0.5) * (ld.at(r, j, sj) + ld.at(r, j + 1, sj1)) * dt;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const R t = (R(1.0) - ku[r]) * uo.x[r] - a.x[r] * (c1 * (pp1.x[r] - p00.x[r]) + c2 * (pp2.x[r] - pm1.x[r]));
          if ((um >> r) & 1) un.x[r] = t;
        }
      }
      // w (fdcore.f90:318-325); old p rows iz0-1 .. iz0+5
      R pz[7];
      pz[0] = shup(p00.x[3]);
      pz[1] = p00.x[0];
      pz[2] = p00.x[1];
      pz[3] = p00.x[2];
      pz[4] = p00.x[3];
      pz[5] = shdn(p00.x[0]);
      pz[6] = shdn(p00.x[1]);
      V4<R> wn = wo;
      if (j >= 2 && j <= NX - 1) {
        R kw[4];
        if (dint) {
#pragma unroll
          for (int r = 0; r < 4; ++r) kw[r] = kwi[r];
        } else {
          const R sj = side_damp(g.damp, j, L, NX);
#pragma unroll
          for (int r = 0; r < 4; ++r) kw[r] = R(0.5) * (ld.at(r, j, sj) + ld.at(r + 1, j, sj)) * dt;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const R t = (R(1.0) - kw[r]) * wo.x[r] - a.x[r] * (c1 * (pz[r + 2] - pz[r + 1]) + c2 * (pz[r + 3] - pz[r]));
          if ((wm >> r) & 1) wn.x[r] = t;
        }
      }
      // w(fs-1, ix) = w(fs, ix) for ix in [2, NX-1] (fdcore.f90:328-332)
      {
        const R n0 = shdn(wn.x[0]);
        if (wmir && j >= 2 && j <= NX - 1) {
#pragma unroll
          for (int r = 0; r < 4; ++r)
            if (r == jm) wn.x[r] = r + 1 < 4 ? wn.x[(r + 1) & 3] : n0;
        }
      }
      if (w.own && j >= x0 && j < xe) {
        V4<R> us = un, ws = wn;
        // vx / vz receivers: adjoint source into u / w after the pressure phase
        if (rec_rows && rec.comp == 1) walk_inject(g, rec, adj_t, w.s, it, j, iz0, us, true);
        if (rec_rows && rec.comp == 2) walk_inject(g, rec, adj_t, w.s, it, j, iz0, ws, true);
        stc(ub1, j, LD, us);
        stc(wb1, j, LD, ws);
      }
      // ---- pressure of column jc = j - 1 (fdcore.f90:335-373); new w rows iz0-2 .. iz0+4
      R wz[7];
      wz[0] = shup(wprev.x[2]);
      wz[1] = shup(wprev.x[3]);
      wz[2] = wprev.x[0];
      wz[3] = wprev.x[1];
      wz[4] = wprev.x[2];
      wz[5] = wprev.x[3];
      wz[6] = shdn(wprev.x[0]);
      const int jc = j - 1;
      V4<R> pv = pm1;  // old p of column jc
      if (jc >= 3 && jc <= NX - 2) {
        const V4<R> bc = ldc(cb, jc, LD, qok);
        R kp[4];
        if (jc >= L + 1 && jc <= NX - L) {
#pragma unroll
          for (int r = 0; r < 4; ++r) kp[r] = kpi[r];
        } else {
          const R sc = side_damp(g.damp, jc, L, NX);
#pragma unroll
          for (int r = 0; r < 4; ++r) kp[r] = ld.at(r, jc, sc) * dt;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const R t = (R(1.0) - kp[r]) * pv.x[r] - bc.x[r] * (c1 * (um1.x[r] - um2.x[r] + wz[r + 2] - wz[r + 1]) +
                                                            c2 * (un.x[r] - um3.x[r] + wz[r + 3] - wz[r]));
          if ((pm >> r) & 1) pv.x[r] = t;
        }
      }
      if (rcur.z == 1) {  // fdcore.f90:345-362, one receiver in the column
#pragma unroll
        for (int r = 0; r < 4; ++r)
          if (r == jrc) pv.x[r] = pv.x[r] + av;
      } else if (rcur.z > 1) {
        walk_inject(g, rec, adj_t, w.s, it, jc, iz0, pv, false);
      }
      // p(fs-1, ix) = -p(fs+1, ix) for every column (fdcore.f90:369-372)
      {
        const R n0 = shdn(pv.x[0]), n1 = shdn(pv.x[1]);
        if (pmir) {
#pragma unroll
          for (int r = 0; r < 4; ++r)
            if (r == jm) pv.x[r] = -(r + 2 < 4 ? pv.x[(r + 2) & 3] : (r + 2 == 4 ? n0 : n1));
        }
      }
      if (w.own && jc >= x0 && jc < xe) {
        stc(pb1, jc, LD, pv);
        // imaging on the interior (solver.f90:237-239)
        const int jxc = jc - L;
        if (img_rows && jxc >= 1 && jxc <= nx) {
          const size_t k = (size_t)(jc - 1) * LD;
          // pe1 was written by this thread in the reconstruction walk above: a coherent (L2) load
          V4<R> pf;
          if constexpr (sizeof(R) == 4) {
            const float4 t = __ldcg(reinterpret_cast<const float4*>(pe1 + k));
            pf.x[0] = t.x;
            pf.x[1] = t.y;
            pf.x[2] = t.z;
            pf.x[3] = t.w;
          } else {
            const double2 t0 = __ldcg(reinterpret_cast<const double2*>(pe1 + k));
            const double2 t1 = __ldcg(reinterpret_cast<const double2*>(pe1 + k) + 1);
            pf.x[0] = t0.x;
            pf.x[1] = t0.y;
            pf.x[2] = t1.x;
            pf.x[3] = t1.y;
          }
          V4<R> g0 = ldc(dg, jc, LD, true), f0 = ldc(dfw, jc, LD, true), k0 = ldc(dbk, jc, LD, true);
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            if (!((irow >> r) & 1)) continue;
            g0.x[r] = g0.x[r] + pf.x[r] * (pm1.x[r] - pv.x[r]);
            f0.x[r] = f0.x[r] + pf.x[r] * pf.x[r];
            k0.x[r] = k0.x[r] + pv.x[r] * pv.x[r];
          }
          stc(dg, jc, LD, g0);
          stc(dfw, jc, LD, f0);
          stc(dbk, jc, LD, k0);
        }
      }
      um3 = um2;
      um2 = um1;
      um1 = un;
      wprev = wn;
      pm1 = p00;
      p00 = pp1;
      pp1 = pp2;
      rcur = rn;
    }
  }
}

}  // namespace swit
