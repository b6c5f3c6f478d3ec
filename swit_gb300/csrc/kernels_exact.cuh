// kernels_exact.cuh -- exact discrete adjoint of the forward recursion.
//
// The forward step it (fdcore.f90:75-128) is linear in the wavefields:
//   S1  p := (1-kp) p - A D(u, w)       ix in [3, NX-2], iz in [fs+1, NZ-2]
//   S2  p(isz, isx) += dt s(it)
//   S3  p(fs-1, :) := -p(fs+1, :)        (free surface)
//   S4  u := (1-ku) u - B Gx(p)          ix in [2, NX-2], iz in [fs, NZ-1]
//       w := (1-kw) w - B Gz(p)          ix in [2, NX-1], iz in [fs, NZ-2]
//   S5  w(fs-1, :) := w(fs, :)           (free surface)
//   S6  seis(ig, it) = p(gz, gx)        (u or w for vx / vz receivers)
// with A = den c^2 dt/dx and B = dt/(den dx).  Its transpose, run for it = nt
// .. 2 on the adjoint fields (lp, lu, lw) in the engine's backward buffers, is
// two gathers per step, each thread owning one 4-row vector as in
// kernels_vec.cuh:
//   k_xadj_p   pressure points of S1's range: lp = (1-kp) lp (S1's scaling,
//              deferred from step it+1) + adjoint sources (S6) + the S4
//              transposes from lu and lw~ (lw~(fs) = lw(fs) + m: the S5 fold)
//              - c2 B(fs) lw~(fs) on row fs+1 (the S3 fold); then the source
//              gradient dt lp (S2), gA -= lp D_it (S1), and lp is stored
//              unscaled.
//   k_xadj_uw  velocity points: lu = (1-ku) lu + the S1 transposes from lp;
//              lw likewise from lw~; the row that S1 at fs+1 reads through the
//              mirror goes to m_new(ix) = c2 A(fs+1, ix) lp(fs+1, ix).
// m alternates between two rows per shot by step parity, so no element is
// read and written by different threads in one launch.  D_it is stored by
// the forward (fwd_p_body with SAVE).  The damping profile is held fixed (it
// depends on vp only through vmin).  gA is dJ/dA per PML point and shot; the
// reduction multiplies by dA/dc = 2 den c dt/dx and sums the padded copies of
// each interior point (io.f90:243-292).  The expressions and their order are
// those of the oracle (oracle_exact_*), compiled without FMA.
#pragma once
#include "kernels_vec.cuh"

namespace swit {

// Forward pressure phase that also stores D of step it for the exact adjoint:
// shot s, step it at dsave + (s * snt + it - sit0) * FSZ.
template <class R>
__global__ void __launch_bounds__(SWIT_VEC_BLOCK, SWIT_VEC_MINB_BLK(R)) k_fwd_p_vx(Grid<R> g, VecList L, Sources src, const R* __restrict__ s_fwd, R* P,
                                                  const R* __restrict__ U, const R* __restrict__ W, int it, int shot0,
                                                  R* __restrict__ dsave) {
  VecIdx v;
  int t;
  const bool ok = list_index(g, L, shot0, v, t);
  pdl_enter();
  if (!ok) return;
  const size_t off = (size_t)v.s * g.FSZ;
  R* ds = dsave + ((size_t)v.s * g.snt + (it - g.sit0)) * g.FSZ;
  if (t == 0)
    fwd_p_body<R, 0, true>(g, src, s_fwd, P + off, U + off, W + off, it, v, ds);
  else if (t == 1)
    fwd_p_body<R, 1, true>(g, src, s_fwd, P + off, U + off, W + off, it, v, ds);
  else
    fwd_p_body<R, 2, true>(g, src, s_fwd, P + off, U + off, W + off, it, v, ds);
}

// Per-launch pointers of the exact adjoint (all shots; per-shot offsets inside).
template <class R>
struct XAdj {
  R* lp;               // adjoint pressure, PML-grid layout
  R* lu;
  R* lw;
  R* gA;               // dJ/dA sums per shot
  R* m;                // mirror rows: [shot][parity][NX]
  R* gsrc;             // dJ/dsrc [shot][nt]
  const R* dsave;      // D records (strip buffer)
  const R* adj_t;      // adjoint sources [shot][it-1][ig]
};

template <class R>
__global__ void __launch_bounds__(SWIT_VEC_BLOCK) k_xadj_p(Grid<R> g, VecList L, Receivers rec, Sources src, XAdj<R> x, int it,
                                                int shot0) {
  VecIdx v;
  int t;
  const bool ok = list_index(g, L, shot0, v, t);
  pdl_enter();
  if (!ok) return;
  const int ix = v.ix, iz0 = v.iz0, F = g.fs, NZ = g.NZ, NX = g.NX, LD4 = g.LD >> 2, s = v.s;
  if (ix < 3 || ix > NX - 2 || iz0 + 3 < F + 1 || iz0 > NZ - 2) return;
  const size_t off = (size_t)s * g.FSZ, k4 = v.k4;
  const R* lu = x.lu + off;
  const R* lw = x.lw + off;
  V4<R> lp = ld4(x.lp + off, k4);
  const V4<R> kp = ld4(g.kp, k4);
  const V4<R> D = ld4(x.dsave + ((size_t)s * g.snt + (it - g.sit0)) * g.FSZ, k4);
  V4<R> gA = ld4(x.gA + off, k4);
  const V4<R> um2 = ld4(lu, k4 - 2 * LD4), um1 = ld4(lu, k4 - LD4), u0 = ld4(lu, k4), up1 = ld4(lu, k4 + LD4);
  const V4<R> bm2 = ld4(g.B, k4 - 2 * LD4), bm1 = ld4(g.B, k4 - LD4), b0 = ld4(g.B, k4), bp1 = ld4(g.B, k4 + LD4);
  R wt[7], bz[7];  // rows iz0-2 .. iz0+4 of column ix
  col_window(lw, v, LD4, ld4(lw, k4), wt, -2, 1);
  col_window(g.B, v, LD4, b0, bz, -2, 1);
  const bool fold = g.fs_flag == 1;
  if (fold && F >= iz0 - 2 && F <= iz0 + 4)
    wt[F - (iz0 - 2)] = wt[F - (iz0 - 2)] + x.m[((size_t)s * 2 + (it & 1)) * NX + (ix - 1)];
  R l[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) l[j] = (R(1.0) - kp.x[j]) * lp.x[j];
  // adjoint sources of this column, in receiver order (pressure receivers)
  if (rec.comp == 0 && iz0 + 3 >= rec.zlo[s] && iz0 <= rec.zhi[s]) {
    const int c0 = rec.colptr[(size_t)s * (NX + 2) + ix], c1 = rec.colptr[(size_t)s * (NX + 2) + ix + 1];
    for (int e = c0; e < c1; ++e) {
      const int j = rec.zrow[e] - iz0;
      if (j >= 0 && j < 4) l[j] = l[j] + x.adj_t[((size_t)s * g.nt + (it - 1)) * g.ngmax + rec.ig[e]];
    }
  }
  const bool sx = src.isx[s] == ix;
  const int isz = src.isz[s];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int iz = iz0 + j;
    if (iz < F + 1 || iz > NZ - 2) continue;
    R a = l[j];
    a = a - g.c1 * (bm1.x[j] * um1.x[j]);
    a = a + g.c1 * (b0.x[j] * u0.x[j]);
    if (ix - 2 >= 2) a = a - g.c2 * (bm2.x[j] * um2.x[j]);
    if (ix + 1 <= NX - 2) a = a + g.c2 * (bp1.x[j] * up1.x[j]);
    const int zi = j + 2;
    a = a - g.c1 * (bz[zi - 1] * wt[zi - 1]);
    a = a + g.c1 * (bz[zi] * wt[zi]);
    if (iz - 2 >= F) a = a - g.c2 * (bz[zi - 2] * wt[zi - 2]);
    if (iz + 1 <= NZ - 2) a = a + g.c2 * (bz[zi + 1] * wt[zi + 1]);
    if (fold && iz == F + 1) a = a - g.c2 * (bz[zi - 1] * wt[zi - 1]);
    if (sx && iz == isz) x.gsrc[(size_t)s * g.nt + (it - 1)] = g.dt * a;
    gA.x[j] = gA.x[j] - a * D.x[j];
    lp.x[j] = a;
  }
  st4(x.lp + off, k4, lp);
  st4(x.gA + off, k4, gA);
}

template <class R>
__global__ void __launch_bounds__(SWIT_VEC_BLOCK, SWIT_VEC_MINB_BLK(R)) k_xadj_uw(Grid<R> g, VecList L, XAdj<R> x, int it, int shot0) {
  VecIdx v;
  int t;
  const bool ok = list_index(g, L, shot0, v, t);
  pdl_enter();
  if (!ok) return;
  const int ix = v.ix, iz0 = v.iz0, F = g.fs, NZ = g.NZ, NX = g.NX, LD4 = g.LD >> 2, s = v.s;
  if (ix < 2 || ix > NX - 1 || iz0 + 3 < F || iz0 > NZ - 1) return;
  const size_t off = (size_t)s * g.FSZ, k4 = v.k4;
  const R* lp = x.lp + off;
  const bool fold = g.fs_flag == 1;
  auto inRp = [&](int z, int c) { return c >= 3 && c <= NX - 2 && z >= F + 1 && z <= NZ - 2; };
  // u on ix in [2, NX-2], rows [F, NZ-1]
  if (ix <= NX - 2) {
    V4<R> lu = ld4(x.lu + off, k4);
    const V4<R> ku = ld4(g.ku, k4);
    const V4<R> pm1 = ld4(lp, k4 - LD4), p0 = ld4(lp, k4), pp1 = ld4(lp, k4 + LD4), pp2 = ld4(lp, k4 + 2 * LD4);
    const V4<R> am1 = ld4(g.A, k4 - LD4), a0 = ld4(g.A, k4), ap1 = ld4(g.A, k4 + LD4), ap2 = ld4(g.A, k4 + 2 * LD4);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int iz = iz0 + j;
      if (iz < F || iz > NZ - 1) continue;
      R a = (R(1.0) - ku.x[j]) * lu.x[j];
      if (inRp(iz, ix)) a = a - g.c1 * (a0.x[j] * p0.x[j]);
      if (inRp(iz, ix + 1)) a = a + g.c1 * (ap1.x[j] * pp1.x[j]);
      if (inRp(iz, ix - 1)) a = a - g.c2 * (am1.x[j] * pm1.x[j]);
      if (inRp(iz, ix + 2)) a = a + g.c2 * (ap2.x[j] * pp2.x[j]);
      lu.x[j] = a;
    }
    st4(x.lu + off, k4, lu);
  }
  // w on ix in [2, NX-1], rows [F, NZ-2]
  V4<R> lw = ld4(x.lw + off, k4);
  const V4<R> kw = ld4(g.kw, k4);
  R pz[7], az[7];  // rows iz0-1 .. iz0+5 of column ix
  col_window(lp, v, LD4, ld4(lp, k4), pz, -1, 2);
  col_window(g.A, v, LD4, ld4(g.A, k4), az, -1, 2);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int iz = iz0 + j;
    if (iz < F || iz > NZ - 2) continue;
    R wt = lw.x[j];
    if (fold && iz == F) wt = wt + x.m[((size_t)s * 2 + (it & 1)) * NX + (ix - 1)];
    const int zi = j + 1;
    R a = (R(1.0) - kw.x[j]) * wt;
    if (inRp(iz, ix)) a = a - g.c1 * (az[zi] * pz[zi]);
    if (inRp(iz + 1, ix)) a = a + g.c1 * (az[zi + 1] * pz[zi + 1]);
    if (inRp(iz - 1, ix)) a = a - g.c2 * (az[zi - 1] * pz[zi - 1]);
    if (inRp(iz + 2, ix)) a = a + g.c2 * (az[zi + 2] * pz[zi + 2]);
    if (fold && iz == F && inRp(F + 1, ix))
      x.m[((size_t)s * 2 + ((it - 1) & 1)) * NX + (ix - 1)] = g.c2 * (az[zi + 1] * pz[zi + 1]);
    lw.x[j] = a;
  }
  st4(x.lw + off, k4, lw);
}

// vx / vz receivers record u / w (S6), so the transposed record adds the
// adjoint sources of step it to lu / lw before the step's two gathers; one
// thread per column and shot, in receiver order.
template <class R>
__global__ void k_xinject_vel(Grid<R> g, Receivers rec, XAdj<R> x, int it, int shot0) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int s = shot0 + blockIdx.y;
  pdl_enter();
  if (ix > g.NX) return;
  const int* cp = rec.colptr + (size_t)s * (g.NX + 2);
  const int e1 = cp[ix + 1];
  if (cp[ix] == e1) return;
  R* f = (rec.comp == 1 ? x.lu : x.lw) + (size_t)s * g.FSZ + (size_t)(ix - 1) * g.LD;
  for (int e = cp[ix]; e < e1; ++e) {
    const int z = rec.zrow[e];
    f[z - 1] = f[z - 1] + x.adj_t[((size_t)s * g.nt + (it - 1)) * g.ngmax + rec.ig[e]];
  }
}

// dJ/dvp on the interior, (nx, nz) z-fastest: per PML point the shots' gA in
// shot order times dA/dc, summed over the PML points padded from the interior
// point (columns, then rows, ascending).
template <class R, class O>
__global__ void k_xgrad(Grid<R> g, const R* __restrict__ gA, const R* __restrict__ dadc, int ns, O* __restrict__ out) {
  const size_t n = (size_t)g.nx * g.nz;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(k / g.nz) + 1, i = (int)(k % g.nz) + 1, L = g.L;
    const int x0 = j == 1 ? 1 : L + j, x1 = j == g.nx ? g.NX : L + j;
    const int z0 = i == 1 ? 1 : L + i, z1 = i == g.nz ? g.NZ : L + i;
    R acc = R(0);
    for (int ix = x0; ix <= x1; ++ix)
      for (int iz = z0; iz <= z1; ++iz) {
        const size_t q = (size_t)(ix - 1) * g.LD + (iz - 1);
        R t = gA[q];
        for (int s = 1; s < ns; ++s) t = t + gA[(size_t)s * g.FSZ + q];
        acc = acc + t * dadc[q];
      }
    out[k] = (O)acc;
  }
}

}  // namespace swit
