// kernels.cuh -- sm_103a kernels of the staggered-grid forward / reconstruction /
// adjoint / imaging path.  Included by engine.cu only.
//
// Grid conventions.  Indices are the reference's 1-based Fortran indices
// (iz, ix) on the PML grid of NZ x NX points (NZ = nz + 2 npml), z fastest.
// Every field of a shot occupies NX columns of LD >= NZ floats (LD a multiple
// of 32, so columns start 128-byte aligned); the reconstruction fields and the
// imaging sums live on the interior nz x nx grid with leading dimension LDI.
// Shots are the slowest dimension: one launch updates a whole batch of shots.
//
// Arithmetic is kept in the reference's order and compiled with --fmad=false,
// so FP32 results match the CPU oracle bit for bit:
//   p  := (1-kappa) p - alpha [c1 (du0 + dw0) + c2 (du1 + dw1)]   fdcore.f90:79-83
//   u  := (1-kappa) u - alpha [c1 dp0 + c2 dp1]                  fdcore.f90:99-102
//   ...
// The two kernels of a step split it where the reference has a data
// dependence: the pressure phase reads only velocities and its own point, the
// velocity phase reads only pressures and its own point, so each can update in
// place.  Mirror rows (free surface) are written by the thread that owns the
// mirrored point, never by two threads.
#pragma once
#include <cstdint>

namespace swit {

// Per-launch constant description of the grid and the coefficient arrays.
template <class R>
struct Grid {
  int nx, nz, L, NX, NZ, LD, LDI, fs, fs_flag, nt, ngmax, SL;
  int snt, sit0;  // strip steps held per shot and the step of slot 0: step it at (s * snt + it - sit0) * SL
  size_t FSZ;  // floats per PML field of one shot (NX * LD)
  size_t FSI;  // floats per interior field of one shot (nx * LDI)
  int IL;      // interior layout offset: interior (jz, jx) at ((jx-1+IL)*LDI + jz-1+IL); npml or 0
  R dt, c1, c2;
  const R* __restrict__ A;     // den c^2 dt / dx   (fdcore.f90:79)
  const R* __restrict__ B;     // dt / (den dx)     (fdcore.f90:99)
  const R* __restrict__ damp;  // damp(1..L) at [1..L]  (pml.f90:84-87)
  // damping factors per point of the PML-grid layout (k_kappa; vectorised kernels)
  const R* __restrict__ kp;    // damp(iz,ix) dt
  const R* __restrict__ ku;    // (damp(iz,ix) + damp(iz,ix+1)) dt / 2
  const R* __restrict__ kw;    // (damp(iz,ix) + damp(iz+1,ix)) dt / 2
};

// Receiver tables: per shot a CSR over grid columns 1..NX.  Entries of column ix
// are [colptr[s*(NX+2)+ix], colptr[s*(NX+2)+ix+1]) in receiver order; each entry
// holds the receiver number ig and its recording / injection row.
struct Receivers {
  const int* __restrict__ colptr;
  const int* __restrict__ ig;
  const int* __restrict__ zrow;
  const int* __restrict__ zlo;  // per shot: lowest and highest receiver row (vectorised kernels;
  const int* __restrict__ zhi;  // may be null elsewhere)
  int comp;                     // recorded component: 0 = p, 1 = vx (u), 2 = vz (w); vec kernels only
  // per shot and column 0 .. NX+1: {ig, row} of the column's first entry, the
  // column's entry count and its first entry (walk kernels; may be null elsewhere)
  const int4* __restrict__ rcol;
};

struct Sources {
  const int* __restrict__ isx;   // forward source column (PML grid)
  const int* __restrict__ isz;   // forward source row
  const int* __restrict__ risx;  // reconstruction source column (interior grid), 0 = none
  const int* __restrict__ risz;
};

// Strip segments of one time step, structure-of-arrays; together the same
// 9 nx + 6 nz values that fdcore.f90:130-159 stores interleaved.
//   bottom  B0 p(NZ-L,j)  B1 p(NZ-L-1,j)  B2 w(NZ-L-1,j)            j = interior columns
//   sides   S0 p(r,L+1)   S1 p(r,L+2)     S2 u(r,L+1)
//           S3 p(r,NX-L)  S4 p(r,NX-L-1)  S5 u(r,NX-L-1)            r = interior rows
//   top     T0 p(fs,j) T1 p(fs+1,j) T2 p(fs+2,j) T3 u(fs,j) T4 u(fs+1,j) T5 w(fs,j)
struct StripOff {
  int B0, B1, B2, S0, S1, S2, S3, S4, S5, T0, T1, T2, T3, T4, T5;
};
__host__ __device__ inline StripOff strip_offsets(int nx, int nz) {
  StripOff o;
  o.B0 = 0;
  o.B1 = nx;
  o.B2 = 2 * nx;
  o.S0 = 3 * nx;
  o.S1 = o.S0 + nz;
  o.S2 = o.S1 + nz;
  o.S3 = o.S2 + nz;
  o.S4 = o.S3 + nz;
  o.S5 = o.S4 + nz;
  o.T0 = o.S5 + nz;
  o.T1 = o.T0 + nx;
  o.T2 = o.T1 + nx;
  o.T3 = o.T2 + nx;
  o.T4 = o.T3 + nx;
  o.T5 = o.T4 + nx;
  return o;
}

// damp_global(iz, ix) of pml.f90:88-99 in closed form.  Columns 1..L and
// NX-L+1..NX carry the side profile; rows 1..L and NZ-L+1..NZ overwrite it on
// the trapezoid the reference's loops cover, which splits the corners along
// their diagonals.  damp[k] is the reference's damp(k), damp(1) = 0.
template <class R>
__host__ __device__ inline R damp_at(const R* damp, int iz, int ix, int L, int NX, int NZ) {
  R v = R(0);
  if (ix <= L)
    v = damp[L - ix + 1];
  else if (ix >= NX - L + 1)
    v = damp[ix - (NX - L)];
  if (iz <= L) {
    if (ix >= iz + 1 && ix <= NX - iz) v = damp[L - iz + 1];
  } else if (iz >= NZ - L + 1) {
    const int k = iz - NZ + L;
    if (ix >= L - k + 2 && ix <= NX - L + k - 1) v = damp[k];
  }
  return v;
}

// Damping factors of the pressure and the two velocity updates at every point
// of the PML grid (LD rows per column), each in the expression and order its
// update uses (fdcore.f90:80, 100, 109; adjoint 313, 322, 340), so a kernel that
// loads them computes the same values as one that evaluates damp_at.
template <class R>
__global__ void k_kappa(Grid<R> g, R* kp, R* ku, R* kw) {
  const size_t n = (size_t)g.NX * g.LD;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int ix = (int)(t / g.LD) + 1, iz = (int)(t % g.LD) + 1;
    R a = R(0), b = R(0), c = R(0);
    if (iz <= g.NZ) {
      const R d = damp_at(g.damp, iz, ix, g.L, g.NX, g.NZ);
      a = d * g.dt;
      if (ix + 1 <= g.NX) b = R(0.5) * (d + damp_at(g.damp, iz, ix + 1, g.L, g.NX, g.NZ)) * g.dt;
      if (iz + 1 <= g.NZ) c = R(0.5) * (d + damp_at(g.damp, iz + 1, ix, g.L, g.NX, g.NZ)) * g.dt;
    }
    kp[t] = a;
    ku[t] = b;
    kw[t] = c;
  }
}

// ---------------------------------------------------------------------------
// Forward, pressure phase of step `it` (fdcore.f90:77-94): p update on
// ix in [3, NX-2], iz in [fs+1, NZ-2]; source injection; p(fs-1,:) = -p(fs+1,:).
template <class R>
__global__ void __launch_bounds__(256) k_fwd_p(Grid<R> g, Sources src, const R* __restrict__ s_fwd, R* P,
                                               const R* __restrict__ U, const R* __restrict__ W, int it, int shot0) {
  const int iz = blockIdx.x * 32 + threadIdx.x + 1;
  const int ix = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int s = shot0 + blockIdx.z;
  if (iz > g.NZ || ix > g.NX) return;
  const size_t off = (size_t)s * g.FSZ;
  R* p = P + off;
  const R* u = U + off;
  const R* w = W + off;
  const int LD = g.LD;
  const size_t k = (size_t)(ix - 1) * LD + (iz - 1);
  R pv = p[k];
  bool write = false;
  if (ix >= 3 && ix <= g.NX - 2 && iz >= g.fs + 1 && iz <= g.NZ - 2) {
    const R alpha = g.A[k];
    const R kappa = damp_at(g.damp, iz, ix, g.L, g.NX, g.NZ) * g.dt;
    pv = (R(1.0) - kappa) * pv - alpha * (g.c1 * (u[k] - u[k - LD] + w[k] - w[k - 1]) +
                                          g.c2 * (u[k + LD] - u[k - 2 * LD] + w[k + 1] - w[k - 2]));
    write = true;
  }
  if (iz == src.isz[s] && ix == src.isx[s]) {
    pv = pv + g.dt * s_fwd[(size_t)s * (g.nt + 1) + (it - 1)];
    write = true;
  }
  if (write) p[k] = pv;
  if (g.fs_flag == 1 && iz == g.fs + 1) p[k - 2] = -pv;
}

// Forward, velocity phase of step `it` (fdcore.f90:97-159): u on ix in
// [2, NX-2], iz in [fs, NZ-1]; w on ix in [2, NX-1], iz in [fs, NZ-2];
// w(fs-1,:) = w(fs,:); receiver gather; boundary-strip save.
template <class R>
__global__ void __launch_bounds__(256) k_fwd_uw(Grid<R> g, Receivers rec, const R* __restrict__ P, R* U, R* W,
                                                R* __restrict__ seis_t, R* __restrict__ strips, int it, int shot0) {
  const int iz = blockIdx.x * 32 + threadIdx.x + 1;
  const int ix = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int s = shot0 + blockIdx.z;
  if (iz > g.NZ || ix > g.NX) return;
  const size_t off = (size_t)s * g.FSZ;
  const R* p = P + off;
  R* u = U + off;
  R* w = W + off;
  const int LD = g.LD;
  const size_t k = (size_t)(ix - 1) * LD + (iz - 1);
  const int L = g.L, NX = g.NX, NZ = g.NZ, fs = g.fs;
  R uv = u[k], wv = w[k];
  if (ix >= 2 && ix <= NX - 2 && iz >= fs && iz <= NZ - 1) {
    const R alpha = g.B[k];
    const R kappa = R(0.5) * (damp_at(g.damp, iz, ix, L, NX, NZ) + damp_at(g.damp, iz, ix + 1, L, NX, NZ)) * g.dt;
    uv = (R(1.0) - kappa) * uv - alpha * (g.c1 * (p[k + LD] - p[k]) + g.c2 * (p[k + 2 * LD] - p[k - LD]));
    u[k] = uv;
  }
  if (ix >= 2 && ix <= NX - 1 && iz >= fs && iz <= NZ - 2) {
    const R alpha = g.B[k];
    const R kappa = R(0.5) * (damp_at(g.damp, iz, ix, L, NX, NZ) + damp_at(g.damp, iz + 1, ix, L, NX, NZ)) * g.dt;
    wv = (R(1.0) - kappa) * wv - alpha * (g.c1 * (p[k + 1] - p[k]) + g.c2 * (p[k + 2] - p[k - 1]));
    w[k] = wv;
  }
  if (g.fs_flag == 1 && iz == fs) w[k - 1] = wv;
  // receiver gather, fdcore.f90:123-128
  {
    const int* cp = rec.colptr + (size_t)s * (NX + 2);
    const int e0 = cp[ix], e1 = cp[ix + 1];
    for (int e = e0; e < e1; ++e)
      if (rec.zrow[e] == iz) seis_t[((size_t)s * g.nt + (it - 1)) * g.ngmax + rec.ig[e]] = p[k];
  }
  // boundary strips of step it, fdcore.f90:130-159
  if (strips) {
    R* b = strips + ((size_t)s * g.snt + (it - g.sit0)) * g.SL;
    const StripOff o = strip_offsets(g.nx, g.nz);
    const int jx = ix - L, jz = iz - L;
    if (jx >= 1 && jx <= g.nx) {
      if (iz == NZ - L) b[o.B0 + jx - 1] = p[k];
      if (iz == NZ - L - 1) {
        b[o.B1 + jx - 1] = p[k];
        b[o.B2 + jx - 1] = wv;
      }
      if (iz == fs) {
        b[o.T0 + jx - 1] = p[k];
        b[o.T3 + jx - 1] = uv;
        b[o.T5 + jx - 1] = wv;
      }
      if (iz == fs + 1) {
        b[o.T1 + jx - 1] = p[k];
        b[o.T4 + jx - 1] = uv;
      }
      if (iz == fs + 2) b[o.T2 + jx - 1] = p[k];
    }
    if (jz >= 1 && jz <= g.nz) {
      if (ix == L + 1) {
        b[o.S0 + jz - 1] = p[k];
        b[o.S2 + jz - 1] = uv;
      }
      if (ix == L + 2) b[o.S1 + jz - 1] = p[k];
      if (ix == NX - L) b[o.S3 + jz - 1] = p[k];
      if (ix == NX - L - 1) {
        b[o.S4 + jz - 1] = p[k];
        b[o.S5 + jz - 1] = uv;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Backward, velocity phase of step `it`:
//   adjoint u, w on the PML grid (fdcore.f90:309-333), w(fs-1,ix) = w(fs,ix);
//   reconstruction u, w on the interior (fdcore.f90:220-235) and the re-insert
//   of u(:,1), u(:,nx-1), w(nz-1,:) from the strips of step it-1 (:237-247).
template <class R>
__global__ void __launch_bounds__(256) k_bwd_uw(Grid<R> g, const R* __restrict__ PB, R* UB, R* WB,
                                                const R* __restrict__ PE, R* UE, R* WE,
                                                const R* __restrict__ strips, int it, int shot0) {
  const int iz = blockIdx.x * 32 + threadIdx.x + 1;
  const int ix = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int s = shot0 + blockIdx.z;
  if (iz > g.NZ || ix > g.NX) return;
  const int LD = g.LD, L = g.L, NX = g.NX, NZ = g.NZ, fs = g.fs;
  const size_t k = (size_t)(ix - 1) * LD + (iz - 1);
  {
    const size_t off = (size_t)s * g.FSZ;
    const R* pb = PB + off;
    R* ub = UB + off;
    R* wb = WB + off;
    if (ix >= 2 && ix <= NX - 2 && iz >= 2 && iz <= NZ - 1) {
      const R alpha = g.A[k];
      const R kappa = R(0.5) * (damp_at(g.damp, iz, ix, L, NX, NZ) + damp_at(g.damp, iz, ix + 1, L, NX, NZ)) * g.dt;
      ub[k] = (R(1.0) - kappa) * ub[k] - alpha * (g.c1 * (pb[k + LD] - pb[k]) + g.c2 * (pb[k + 2 * LD] - pb[k - LD]));
    }
    if (ix >= 2 && ix <= NX - 1 && iz >= 2 && iz <= NZ - 2) {
      const R alpha = g.A[k];
      const R kappa = R(0.5) * (damp_at(g.damp, iz, ix, L, NX, NZ) + damp_at(g.damp, iz + 1, ix, L, NX, NZ)) * g.dt;
      const R wv = (R(1.0) - kappa) * wb[k] - alpha * (g.c1 * (pb[k + 1] - pb[k]) + g.c2 * (pb[k + 2] - pb[k - 1]));
      // the mirror row fs-1 belongs to the thread of row fs (fdcore.f90:329-333)
      if (!(g.fs_flag == 1 && iz == fs - 1)) wb[k] = wv;
      if (g.fs_flag == 1 && iz == fs) wb[k - 1] = wv;
    }
  }
  const int jx = ix - L, jz = iz - L;
  if (jx < 1 || jx > g.nx || jz < 1 || jz > g.nz) return;
  const int nx = g.nx, nz = g.nz, LDI = g.LDI;
  const size_t ki = (size_t)(jx - 1) * LDI + (jz - 1);
  const size_t offi = (size_t)s * g.FSI;
  const R* pe = PE + offi;
  R* ue = UE + offi;
  R* we = WE + offi;
  const int fsi = fs - L;  // fs(ix+npml) - npml
  if (jx >= 2 && jx <= nx - 2 && jz >= fsi + 1 && jz <= nz - 1) {
    const R alpha = g.B[k];
    ue[ki] = ue[ki] + alpha * (g.c1 * (pe[ki + LDI] - pe[ki]) + g.c2 * (pe[ki + 2 * LDI] - pe[ki - LDI]));
  }
  if (jx >= 2 && jx <= nx - 1 && jz >= fsi + 1 && jz <= nz - 2) {
    const R alpha = g.B[k];
    we[ki] = we[ki] + alpha * (g.c1 * (pe[ki + 1] - pe[ki]) + g.c2 * (pe[ki + 2] - pe[ki - 1]));
  }
  const R* b = strips + ((size_t)s * g.snt + (it - 1 - g.sit0)) * g.SL;  // boundary(:, it-1)
  const StripOff o = strip_offsets(nx, nz);
  if (jz == nz - 1) we[ki] = b[o.B2 + jx - 1];
  if (jx == 1) ue[ki] = b[o.S2 + jz - 1];
  if (jx == nx - 1) ue[ki] = b[o.S5 + jz - 1];
}

// Backward, pressure phase of step `it`:
//   adjoint p (fdcore.f90:336-345), adjoint-source injection (:348-367) and
//   p(fs-1,:) = -p(fs+1,:) (:370-373); reconstruction source subtraction,
//   p update and strip re-insert (:249-287); imaging and illumination
//   (solver.f90:237-239) accumulated per shot.
template <class R>
__global__ void __launch_bounds__(256) k_bwd_p(Grid<R> g, Receivers rec, Sources src, const R* __restrict__ s_fwd,
                                               const R* __restrict__ adj_t, R* PB, const R* __restrict__ UB,
                                               const R* __restrict__ WB, R* PE, const R* __restrict__ UE,
                                               const R* __restrict__ WE, R* DG, R* DFW, R* DBK,
                                               const R* __restrict__ strips, int it, int shot0) {
  const int iz = blockIdx.x * 32 + threadIdx.x + 1;
  const int ix = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int s = shot0 + blockIdx.z;
  if (iz > g.NZ || ix > g.NX) return;
  const int LD = g.LD, L = g.L, NX = g.NX, NZ = g.NZ, fs = g.fs;
  const size_t k = (size_t)(ix - 1) * LD + (iz - 1);
  const size_t off = (size_t)s * g.FSZ;
  R* pb = PB + off;
  const R* ub = UB + off;
  const R* wb = WB + off;
  const R pold = pb[k];
  R pv = pold;
  bool write = false;
  if (ix >= 3 && ix <= NX - 2 && iz >= 3 && iz <= NZ - 2) {
    const R alpha = g.B[k];
    const R kappa = damp_at(g.damp, iz, ix, L, NX, NZ) * g.dt;
    pv = (R(1.0) - kappa) * pold - alpha * (g.c1 * (ub[k] - ub[k - LD] + wb[k] - wb[k - 1]) +
                                            g.c2 * (ub[k + LD] - ub[k - 2 * LD] + wb[k + 1] - wb[k - 2]));
    write = true;
  }
  {
    const int* cp = rec.colptr + (size_t)s * (NX + 2);
    const int e0 = cp[ix], e1 = cp[ix + 1];
    for (int e = e0; e < e1; ++e)
      if (rec.zrow[e] == iz) {
        pv = pv + g.dt * adj_t[((size_t)s * g.nt + (it - 1)) * g.ngmax + rec.ig[e]];
        write = true;
      }
  }
  // row fs-1 is overwritten by the mirror written by the thread of row fs+1
  if (write && iz != fs - 1) pb[k] = pv;
  if (iz == fs + 1) pb[k - 2] = -pv;

  const int jx = ix - L, jz = iz - L;
  if (jx < 1 || jx > g.nx || jz < 1 || jz > g.nz) return;
  const int nx = g.nx, nz = g.nz, LDI = g.LDI;
  const size_t ki = (size_t)(jx - 1) * LDI + (jz - 1);
  const size_t offi = (size_t)s * g.FSI;
  R* pe = PE + offi;
  const R* ue = UE + offi;
  const R* we = WE + offi;
  const int fsi = fs - L;
  R pf = pe[ki];
  if (jx == src.risx[s] && jz == src.risz[s]) pf = pf - g.dt * s_fwd[(size_t)s * (g.nt + 1) + it];  // s(it+1)
  if (jx >= 3 && jx <= nx - 2 && jz >= fsi + 2 && jz <= nz - 2) {
    const R alpha = g.A[k];
    pf = pf + alpha * (g.c1 * (ue[ki] - ue[ki - LDI] + we[ki] - we[ki - 1]) +
                       g.c2 * (ue[ki + LDI] - ue[ki - 2 * LDI] + we[ki + 1] - we[ki - 2]));
  }
  const R* b = strips + ((size_t)s * g.snt + (it - 1 - g.sit0)) * g.SL;
  const StripOff o = strip_offsets(nx, nz);
  // re-insert in the reference's order: bottom, sides, top (last write wins)
  if (jz == nz) pf = b[o.B0 + jx - 1];
  if (jz == nz - 1) pf = b[o.B1 + jx - 1];
  if (jx == 1) pf = b[o.S0 + jz - 1];
  if (jx == 2) pf = b[o.S1 + jz - 1];
  if (jx == nx) pf = b[o.S3 + jz - 1];
  if (jx == nx - 1) pf = b[o.S4 + jz - 1];
  if (jz == fsi) pf = b[o.T0 + jx - 1];
  if (jz == fsi + 1) pf = b[o.T1 + jx - 1];
  if (jz == fsi + 2) pf = b[o.T2 + jx - 1];
  pe[ki] = pf;
  R* dg = DG + offi;
  R* dfw = DFW + offi;
  R* dbk = DBK + offi;
  dg[ki] = dg[ki] + pf * (pold - pv);
  dfw[ki] = dfw[ki] + pf * pf;
  dbk[ki] = dbk[ki] + pv * pv;
}

// ---------------------------------------------------------------------------
// Shot sum in shot order and g = -2 g / c (solver.f90:263-270), written to the
// caller's (nx, nz) layout in type O.
template <class R, class O>
__global__ void k_reduce(Grid<R> g, const R* __restrict__ DG, const R* __restrict__ DFW, const R* __restrict__ DBK,
                         const R* __restrict__ cint, int ns, O* grad, O* fw, O* bk) {
  const int n = g.nx * g.nz;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int jx = t / g.nz, jz = t - jx * g.nz;
    const size_t ki = (size_t)(jx + g.IL) * g.LDI + (jz + g.IL);
    R a = DG[ki], b = DFW[ki], c = DBK[ki];
    for (int s = 1; s < ns; ++s) {
      a = a + DG[(size_t)s * g.FSI + ki];
      b = b + DFW[(size_t)s * g.FSI + ki];
      c = c + DBK[(size_t)s * g.FSI + ki];
    }
    if (grad) grad[t] = (O)(R(-2.0) * a / cint[ki]);
    if (fw) fw[t] = (O)b;
    if (bk) bk[t] = (O)c;
  }
}

// seis_t [s][it][ig] (time-major staging) -> out [s][ig][it].
template <class R, class O>
__global__ void k_seis_out(const R* __restrict__ seis_t, O* out, int ns, int nt, int ngmax) {
  __shared__ R tile[32][33];
  const int s = blockIdx.z;
  const int t0 = blockIdx.x * 32, g0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int t = t0 + j, gi = g0 + threadIdx.x;
    tile[j][threadIdx.x] = (t < nt && gi < ngmax) ? seis_t[((size_t)s * nt + t) * ngmax + gi] : R(0);
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int gi = g0 + j, t = t0 + threadIdx.x;
    if (t < nt && gi < ngmax) out[((size_t)s * ngmax + gi) * nt + t] = (O)tile[threadIdx.x][j];
  }
}

// in [s][ig][it] (float, the caller's layout) -> adj_t [s][it][ig].
template <class R>
__global__ void k_adj_in(const float* __restrict__ in, R* adj_t, int ns, int nt, int ngmax) {
  __shared__ float tile[32][33];
  const int s = blockIdx.z;
  const int t0 = blockIdx.x * 32, g0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int gi = g0 + j, t = t0 + threadIdx.x;
    tile[j][threadIdx.x] = (t < nt && gi < ngmax) ? in[((size_t)s * ngmax + gi) * nt + t] : 0.f;
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int t = t0 + j, gi = g0 + threadIdx.x;
    if (t < nt && gi < ngmax) adj_t[((size_t)s * nt + t) * ngmax + gi] = (R)tile[threadIdx.x][j];
  }
}

// Per-trace live flags and misfit of the Waveform misfit (misfit.py:128-148,
// 263-282): one block per trace (s, ig) over the time-major synthetics and the
// caller's obs [s][ig][it].
template <class R>
__global__ void k_trace_stats(const R* __restrict__ seis_t, const float* __restrict__ obs, const int* __restrict__ ng,
                              int nt, int ngmax, float dt, int* live, double* misfit_trace) {
  const int ig = blockIdx.x, s = blockIdx.y;
  __shared__ double red[3][256];
  double so = 0, ss = 0, rr = 0;
  if (ig < ng[s]) {
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
      const float o = obs[((size_t)s * ngmax + ig) * nt + t];
      const float y = (float)seis_t[((size_t)s * nt + t) * ngmax + ig];
      const float r = y - o;
      so += (double)o * o;
      ss += (double)y * y;
      rr += (double)r * r;
    }
  }
  red[0][threadIdx.x] = so;
  red[1][threadIdx.x] = ss;
  red[2][threadIdx.x] = rr;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int ok = (ig < ng[s] && red[0][0] > 0.0 && red[1][0] > 0.0) ? 1 : 0;
    live[(size_t)s * ngmax + ig] = ok;
    misfit_trace[(size_t)s * ngmax + ig] = ok ? sqrt(red[2][0] * (double)dt) : 0.0;
  }
}

// Adjoint source syn - obs of live traces, written time-major.
template <class R>
__global__ void k_residual(const R* __restrict__ seis_t, const float* __restrict__ obs, const int* __restrict__ live,
                           R* adj_t, int nt, int ngmax) {
  __shared__ float tile[32][33];
  const int s = blockIdx.z;
  const int t0 = blockIdx.x * 32, g0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int gi = g0 + j, t = t0 + threadIdx.x;
    tile[j][threadIdx.x] = (t < nt && gi < ngmax) ? obs[((size_t)s * ngmax + gi) * nt + t] : 0.f;
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int t = t0 + j, gi = g0 + threadIdx.x;
    if (t < nt && gi < ngmax) {
      const size_t q = ((size_t)s * nt + t) * ngmax + gi;
      const float y = (float)seis_t[q];
      adj_t[q] = live[(size_t)s * ngmax + gi] ? (R)(y - tile[threadIdx.x][j]) : R(0);
    }
  }
}

// Interior copy of the final forward wavefields into the reconstruction fields
// (fdcore.f90:164-166).
template <class R>
__global__ void k_copy_end(Grid<R> g, const R* __restrict__ P, const R* __restrict__ U, const R* __restrict__ W,
                           R* PE, R* UE, R* WE, int ns) {
  const size_t n = (size_t)ns * g.nx * g.nz;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(t / ((size_t)g.nx * g.nz));
    const int r = (int)(t - (size_t)s * g.nx * g.nz);
    const int jx = r / g.nz, jz = r - jx * g.nz;
    const size_t k = (size_t)s * g.FSZ + (size_t)(jx + g.L) * g.LD + (jz + g.L);
    const size_t ki = (size_t)s * g.FSI + (size_t)(jx + g.IL) * g.LDI + (jz + g.IL);
    PE[ki] = P[k];
    UE[ki] = U[k];
    WE[ki] = W[k];
  }
}

// Interior (nx, nz) of a padded interior field -> caller layout, all shots.
template <class R, class O>
__global__ void k_interior_out(Grid<R> g, const R* __restrict__ F, O* out, int ns) {
  const size_t n = (size_t)ns * g.nx * g.nz;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(t / ((size_t)g.nx * g.nz));
    const int r = (int)(t - (size_t)s * g.nx * g.nz);
    const int jx = r / g.nz, jz = r - jx * g.nz;
    out[t] = (O)F[(size_t)s * g.FSI + (size_t)(jx + g.IL) * g.LDI + (jz + g.IL)];
  }
}

// Strips (SoA per step) -> the reference's interleaved boundary(S, nt) layout.
template <class R, class O>
__global__ void k_strips_out(Grid<R> g, const R* __restrict__ strips, O* out, int ns) {
  const int nx = g.nx, nz = g.nz, SL = g.SL;
  const size_t n = (size_t)ns * g.nt * SL;
  const StripOff o = strip_offsets(nx, nz);
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t rec = t / SL;
    const int q = (int)(t - rec * SL);
    const R* b = strips + rec * SL;
    R v;
    if (q < 3 * nx) {
      const int j = q / 3, e = q - 3 * j;
      v = b[(e == 0 ? o.B0 : e == 1 ? o.B1 : o.B2) + j];
    } else if (q < 3 * nx + 6 * nz) {
      const int r = (q - 3 * nx) / 6, e = (q - 3 * nx) - 6 * r;
      const int seg[6] = {o.S0, o.S1, o.S2, o.S3, o.S4, o.S5};
      v = b[seg[e] + r];
    } else {
      const int j = (q - 3 * nx - 6 * nz) / 6, e = (q - 3 * nx - 6 * nz) - 6 * j;
      const int seg[6] = {o.T0, o.T1, o.T2, o.T3, o.T4, o.T5};
      v = b[seg[e] + j];
    }
    out[t] = (O)v;
  }
}

// The reference's interleaved boundary(S, nt) layout (float) -> strips (SoA per step).
template <class R>
__global__ void k_strips_in(Grid<R> g, const float* __restrict__ in, R* strips, int ns) {
  const int nx = g.nx, nz = g.nz, SL = g.SL;
  const size_t n = (size_t)ns * g.nt * SL;
  const StripOff o = strip_offsets(nx, nz);
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t rec = t / SL;
    const int q = (int)(t - rec * SL);
    R* b = strips + rec * SL;
    const R v = (R)in[t];
    if (q < 3 * nx) {
      const int j = q / 3, e = q - 3 * j;
      b[(e == 0 ? o.B0 : e == 1 ? o.B1 : o.B2) + j] = v;
    } else if (q < 3 * nx + 6 * nz) {
      const int r = (q - 3 * nx) / 6, e = (q - 3 * nx) - 6 * r;
      const int seg[6] = {o.S0, o.S1, o.S2, o.S3, o.S4, o.S5};
      b[seg[e] + r] = v;
    } else {
      const int j = (q - 3 * nx - 6 * nz) / 6, e = (q - 3 * nx - 6 * nz) - 6 * j;
      const int seg[6] = {o.T0, o.T1, o.T2, o.T3, o.T4, o.T5};
      b[seg[e] + j] = v;
    }
  }
}

// (ns, nx, nz) float -> interior points of a PML-grid field (the final forward state).
template <class R>
__global__ void k_end_in(Grid<R> g, const float* __restrict__ in, R* F, int ns) {
  const size_t n = (size_t)ns * g.nx * g.nz;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(t / ((size_t)g.nx * g.nz));
    const int r = (int)(t - (size_t)s * g.nx * g.nz);
    const int jx = r / g.nz, jz = r - jx * g.nz;
    F[(size_t)s * g.FSZ + (size_t)(jx + g.L) * g.LD + (jz + g.L)] = (R)in[t];
  }
}

}  // namespace swit
