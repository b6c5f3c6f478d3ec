// kernels_vec.cuh -- the split step kernels, vectorised along z.
//
// Each thread owns one 16-byte vector of 4 consecutive z-points of one column
// (LD is a multiple of 32, so vectors never straddle columns).  Neighbours
// along x are +-LD/4 vectors away, neighbours along z come from the adjacent
// vectors of the same column.  A thread writes its own vector; the only other
// element it may write is a free-surface mirror row (fs-1) lying in the vector
// above its own, and the owner of that vector then leaves that one element
// untouched -- so the in-place updates stay race-free.
//
// The reconstruction fields and imaging sums use the PML-grid layout of the
// wavefields (interior point (jz, jx) at PML row jz+npml, column jx+npml), so
// one vector covers the same rows in every array.
//
// Every scalar expression is the one of kernels.cuh (fdcore.f90 order, no
// FMA): results stay bit-identical to the oracle.
#pragma once
#include "kernels.cuh"

namespace swit {

template <class R>
struct V4 {
  R x[4];
};

template <class R>
__device__ __forceinline__ V4<R> ld4(const R* p, size_t k4) {
  V4<R> v;
  if constexpr (sizeof(R) == 4) {
    const float4 t = reinterpret_cast<const float4*>(p)[k4];
    v.x[0] = t.x;
    v.x[1] = t.y;
    v.x[2] = t.z;
    v.x[3] = t.w;
  } else {
    const double2 a = reinterpret_cast<const double2*>(p)[2 * k4];
    const double2 b = reinterpret_cast<const double2*>(p)[2 * k4 + 1];
    v.x[0] = a.x;
    v.x[1] = a.y;
    v.x[2] = b.x;
    v.x[3] = b.y;
  }
  return v;
}

template <class R>
__device__ __forceinline__ void st4(R* p, size_t k4, const V4<R>& v) {
  if constexpr (sizeof(R) == 4) {
    reinterpret_cast<float4*>(p)[k4] = make_float4(v.x[0], v.x[1], v.x[2], v.x[3]);
  } else {
    reinterpret_cast<double2*>(p)[2 * k4] = make_double2(v.x[0], v.x[1]);
    reinterpret_cast<double2*>(p)[2 * k4 + 1] = make_double2(v.x[2], v.x[3]);
  }
}

// Stores the vector except element `skip` (the mirror row another thread writes).
template <class R>
__device__ __forceinline__ void st4_except(R* p, size_t k4, const V4<R>& v, int skip) {
#pragma unroll
  for (int j = 0; j < 4; ++j)
    if (j != skip) p[4 * k4 + j] = v.x[j];
}

// Index set of one vector task: shot, column, first row, and the vector's
// position in the wavefield, coefficient and imaging-sum arrays.
struct VecIdx {
  int s, ix, iz0, q;
  size_t k4;  // vector index of the wavefield arrays (column stride LD/4)
  size_t kc;  // vector index of the coefficient arrays A, B
  size_t kg;  // vector index of the per-shot imaging sums dg, dfw, dbk and the kappa arrays
  bool ok;
  bool dint;  // columns ix, ix+1 and rows iz0..iz0+4 all interior: every damping term is 0
  bool deep;  // columns [L+3, NX-L-3], rows [L+4, NZ-L-3]: every update range holds, no
              // strip, mirror or re-insert row or column, no damping
};
template <class R>
__device__ __forceinline__ void vec_flags(const Grid<R>& g, VecIdx& v) {
  v.dint = v.ix > g.L && v.ix + 1 <= g.NX - g.L && v.iz0 > g.L && v.iz0 + 4 <= g.NZ - g.L;
  v.deep = v.ix >= g.L + 3 && v.ix <= g.NX - g.L - 3 && v.iz0 >= g.L + 4 && v.iz0 + 3 <= g.NZ - g.L - 3;
}

// Resident 256-thread blocks per SM the FP32 vec step kernels are compiled for
// (caps their registers at 65536 / (256 * SWIT_VEC_MINB)); the FP64 builds are
// not capped.  4 (64 registers, no spill) measured 2-5 % faster than the
// uncapped build (70-72 registers in k_bwd_p_v and k_fwd_uw_v, 3 blocks per SM);
// 5 and 6 spill and are slower.
#ifndef SWIT_VEC_MINB
#define SWIT_VEC_MINB 4
#endif
#define SWIT_VEC_MINB_R(R) (sizeof(R) == 4 ? SWIT_VEC_MINB : 1)
// Threads per block of the vec step kernels.  Measured at 481x141, 49 shots
// (64 registers): 128 threads 133.6, 256: 127.3, 512: 118.9, 64: 119.0
// shot-gradients/s -- 8 resident blocks per SM schedule and drain more finely.
#ifndef SWIT_VEC_BLOCK
#define SWIT_VEC_BLOCK 128
#endif
// Launch bounds of the vec step kernels: SWIT_VEC_BLOCK threads, registers
// capped as for SWIT_VEC_MINB blocks of 256 threads per SM (FP32 builds)
#define SWIT_VEC_MINB_BLK(R) (SWIT_VEC_MINB_R(R) * 256 / SWIT_VEC_BLOCK > 0 ? SWIT_VEC_MINB_R(R) * 256 / SWIT_VEC_BLOCK : 1)
// Own caps of the reverse velocity kernel, which fits 48 registers without
// spilling (5: 134.7 vs 133.4 shot-gradients/s at 4), and of the forward
// pressure kernel.
#ifndef SWIT_VEC_MINB_BUW
#define SWIT_VEC_MINB_BUW 5
#endif
#define SWIT_VEC_MINB_BUW_BLK(R) (sizeof(R) == 4 ? SWIT_VEC_MINB_BUW * 256 / SWIT_VEC_BLOCK : 1)
#ifndef SWIT_VEC_MINB_FP
#define SWIT_VEC_MINB_FP SWIT_VEC_MINB
#endif
#define SWIT_VEC_MINB_FP_BLK(R) (sizeof(R) == 4 ? SWIT_VEC_MINB_FP * 256 / SWIT_VEC_BLOCK : 1)

// Programmatic dependent launch: wait until the previous kernel in the stream
// has completed and its writes are visible, then let the next kernel's blocks
// be scheduled (they wait in the same way).  Without the launch attribute both
// instructions return at once.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}


#ifndef SWIT_VEC_REVERSE
#define SWIT_VEC_REVERSE 1
#endif

// Task list of a vectorised kernel: entries (ix - 1) << 16 | q, the vectors
// grouped by the body tier the kernel needs there (the highest over all
// shots), each group ordered by 2-D tiles for cache locality; entries [0, n0)
// run tier 0, [n0, n1) tier 1, [n1, len) tier 2.  Vectors on which the phase
// does no work are left out.  A warp therefore runs one body.
struct VecList {
  const uint32_t* __restrict__ e;
  int n0, n1, len;
  // A rectangle of tier-0 vectors kept out of the list: columns [rx0+1, ...),
  // rnq vectors from rq0 in each, rn vectors in all, covered by the first rnb
  // blocks, whose threads find their vector arithmetically (no list load).
  int rx0, rq0, rnq, rn, rnb;
};

// Thread -> (shot, vector, tier) from the list; false past its end.
template <class R>
__device__ __forceinline__ bool list_index(const Grid<R>& g, const VecList& L, int shot0, VecIdx& v, int& t) {
  // blocks are dispatched about in index order: the last list blocks (tier 2,
  // the most work) take the lowest block indices, the rectangle the highest
  const int bx = SWIT_VEC_REVERSE ? (int)(gridDim.x - 1 - blockIdx.x) : (int)blockIdx.x;
  const int i = bx * blockDim.x + threadIdx.x;
  v.s = shot0 + blockIdx.y;
  if (bx < L.rnb) {  // the tier-0 rectangle, column by column (uniform over the block)
    const int r = bx * blockDim.x + threadIdx.x;
    if (r >= L.rn) return false;
    const int c = r / L.rnq;
    v.ix = L.rx0 + c + 1;
    v.q = L.rq0 + (r - c * L.rnq);
    v.iz0 = 4 * v.q + 1;
    v.ok = true;
    v.k4 = (size_t)(v.ix - 1) * (g.LD >> 2) + v.q;
    v.kc = v.k4;
    v.kg = v.k4;
    t = 0;
    return true;
  }
  const int il = i - L.rnb * (int)blockDim.x;
  if (il >= L.len) return false;
  const uint32_t e = L.e[il];
  v.ix = (int)(e >> 16) + 1;
  v.q = (int)(e & 0xffffu);
  v.iz0 = 4 * v.q + 1;
  v.ok = true;
  v.k4 = (size_t)(v.ix - 1) * (g.LD >> 2) + v.q;
  v.kc = v.k4;
  v.kg = v.k4;
  t = il < L.n0 ? 0 : (il < L.n1 ? 1 : 2);
  return true;
}

// Damping loads of a body of tier T from the global kappa arrays (indexed like
// the imaging sums): none on the fast path, where every factor is 0.
template <class R, int T>
__device__ __forceinline__ V4<R> kappa4(const R* k, const VecIdx& v) {
  V4<R> z;
  if constexpr (T == 0) {
#pragma unroll
    for (int j = 0; j < 4; ++j) z.x[j] = R(0);
  } else {
    z = ld4(k, v.kg);
  }
  return z;
}

// z-neighbours: the rows iz0+lo .. iz0+4+hi-1 of column ix around vector k4, as an
// array r[0 .. 4-lo+hi-1] (r[-lo] is row iz0); rows outside the column read 0.
template <class R>
__device__ __forceinline__ void col_window(const R* f, const VecIdx& v, int LD4, const V4<R>& own, R* r, int lo,
                                           int hi) {
  // lo in {-2, -1}, hi in {1, 2}
  if (v.q > 0) {
    const V4<R> m = ld4(f, v.k4 - 1);
    if (lo == -2) {
      r[0] = m.x[2];
      r[1] = m.x[3];
    } else {
      r[0] = m.x[3];
    }
  } else {
    r[0] = R(0);
    if (lo == -2) r[1] = R(0);
  }
  const int o = -lo;
  r[o] = own.x[0];
  r[o + 1] = own.x[1];
  r[o + 2] = own.x[2];
  r[o + 3] = own.x[3];
  if (v.q + 1 < LD4) {
    const V4<R> n = ld4(f, v.k4 + 1);
    r[o + 4] = n.x[0];
    if (hi == 2) r[o + 5] = n.x[1];
  } else {
    r[o + 4] = R(0);
    if (hi == 2) r[o + 5] = R(0);
  }
}

// ---------------------------------------------------------------------------
// Forward pressure phase (fdcore.f90:77-94).  SAVE: also store the divergence
// term D of every updated row into dsave (the step's record; 0 elsewhere), for
// the exact adjoint (kernels_exact.cuh).
template <class R, int T, bool SAVE = false>
__device__ __forceinline__ void fwd_p_body(const Grid<R>& g, const Sources& src, const R* __restrict__ s_fwd, R* __restrict__ p,
                                           const R* __restrict__ u, const R* __restrict__ w, int it,
                                           const VecIdx& v, R* __restrict__ dsave = nullptr) {
  constexpr bool CHK = T == 2;
  const int LD4 = g.LD >> 2, ix = v.ix, iz0 = v.iz0, fs = g.fs, NZ = g.NZ;
  V4<R> pv = ld4(p, v.k4);
  V4<R> dv;
  if constexpr (SAVE) {
#pragma unroll
    for (int j = 0; j < 4; ++j) dv.x[j] = R(0);
  }
  bool dirty = false;
  if (!CHK || (ix >= 3 && ix <= g.NX - 2 && iz0 + 3 >= fs + 1 && iz0 <= NZ - 2)) {
    const V4<R> a = ld4(g.A, v.kc);
    const V4<R> kk = kappa4<R, T>(g.kp, v);
    const V4<R> u0 = ld4(u, v.k4), um1 = ld4(u, v.k4 - LD4), up1 = ld4(u, v.k4 + LD4), um2 = ld4(u, v.k4 - 2 * LD4);
    R wz[7];  // w at rows iz0-2 .. iz0+4
    col_window(w, v, LD4, ld4(w, v.k4), wz, -2, 1);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int iz = iz0 + j;
      if (!CHK || (iz >= fs + 1 && iz <= NZ - 2)) {
        const R kappa = T == 0 ? R(0) : kk.x[j];
        const R D = g.c1 * (u0.x[j] - um1.x[j] + wz[j + 2] - wz[j + 1]) +
                    g.c2 * (up1.x[j] - um2.x[j] + wz[j + 3] - wz[j]);
        pv.x[j] = (R(1.0) - kappa) * pv.x[j] - a.x[j] * D;
        if constexpr (SAVE) dv.x[j] = D;
      }
    }
    dirty = true;
  }
  if (CHK) {
    const int js = src.isz[v.s] - iz0;
    if (ix == src.isx[v.s] && js >= 0 && js < 4) {
      pv.x[js] = pv.x[js] + g.dt * s_fwd[(size_t)v.s * (g.nt + 1) + (it - 1)];
      dirty = true;
    }
    // p(fs-1, :) = -p(fs+1, :) (fdcore.f90:92-94).  Rows fs-1 and fs+1 share a
    // vector, or row fs-1 is in the vector above, whose rows (<= fs) this phase
    // never changes: its owner stores nothing and the owner of fs+1 writes it.
    const int jm = fs - 1 - iz0, jp = fs + 1 - iz0;
    if (g.fs_flag == 1 && jp >= 0 && jp < 4) {
      if (jm >= 0) {
        pv.x[jm] = -pv.x[jp];
        dirty = true;
      } else {
        p[(v.k4 - v.q) * 4 + (fs - 2)] = -pv.x[jp];
      }
    }
  }
  if (dirty) st4(p, v.k4, pv);
  if constexpr (SAVE) st4(dsave, v.k4, dv);
}

// Body tier of a vector in each phase: 0 = fast (deep interior: no damping, no
// range test, no special row or column), 1 = regular (every row inside the
// phase's update ranges, damping from the kappa arrays, no mirror, source,
// receiver, strip or reconstruction work), 2 = general (every test).  Every
// tier computes the same values; a higher tier only tests more.
template <class R>
__device__ __forceinline__ int tier_fwd_p(const Grid<R>& g, const VecIdx& v, bool src_here) {
  if (src_here) return 2;
  if (v.deep) return 0;
  return (v.ix >= 3 && v.ix <= g.NX - 2 && v.iz0 >= g.fs + 2 && v.iz0 + 3 <= g.NZ - 2) ? 1 : 2;
}

// The vector holds a row or column of the boundary strips (fdcore.f90:130-159).
template <class R>
__device__ __forceinline__ bool strip_vec(const Grid<R>& g, const VecIdx& v) {
  const int fs = g.fs, NZ = g.NZ, NX = g.NX, L = g.L, iz0 = v.iz0, ix = v.ix;
  return (iz0 <= fs + 2 && iz0 + 3 >= fs) || (iz0 <= NZ - L && iz0 + 3 >= NZ - L - 1) || ix == L + 1 ||
         ix == L + 2 || ix == NX - L || ix == NX - L - 1;
}

template <class R>
__device__ __forceinline__ int tier_fwd_uw(const Grid<R>& g, const VecIdx& v, bool rec_here) {
  if (rec_here) return 2;
  if (v.deep) return 0;
  return (v.ix >= 2 && v.ix <= g.NX - 2 && v.iz0 >= g.fs + 1 && v.iz0 + 3 <= g.NZ - 2 && !strip_vec(g, v)) ? 1 : 2;
}

// No row of the vector lies on the interior grid (no reconstruction work).
template <class R>
__device__ __forceinline__ bool outside_interior(const Grid<R>& g, const VecIdx& v) {
  const int jx = v.ix - g.L, jz0 = v.iz0 - g.L;
  return jx < 1 || jx > g.nx || jz0 + 3 < 1 || jz0 > g.nz;
}

template <class R>
__device__ __forceinline__ int tier_bwd_uw(const Grid<R>& g, const VecIdx& v) {
  if (v.deep) return 0;
  const bool mirror = g.fs_flag == 1 && v.iz0 <= g.fs && v.iz0 + 3 >= g.fs - 1;  // rows fs-1, fs
  return (v.ix >= 2 && v.ix <= g.NX - 2 && v.iz0 >= 2 && v.iz0 + 3 <= g.NZ - 2 && !mirror && outside_interior(g, v))
             ? 1
             : 2;
}

template <class R>
__device__ __forceinline__ int tier_bwd_p(const Grid<R>& g, const VecIdx& v, bool rec_here, bool src_here) {
  if (rec_here || src_here) return 2;
  if (v.deep) return 0;
  const bool mirror = v.iz0 <= g.fs + 1 && v.iz0 + 3 >= g.fs - 1;  // rows fs-1, fs+1
  return (v.ix >= 3 && v.ix <= g.NX - 2 && v.iz0 >= 3 && v.iz0 + 3 <= g.NZ - 2 && !mirror && outside_interior(g, v))
             ? 1
             : 2;
}

// Body of tier t (0, 1, 2) of a list entry.
#define SWIT_TIER_CALL(body, ...) \
  do {                            \
    if (t == 0)                   \
      body<R, 0>(__VA_ARGS__);    \
    else if (t == 1)              \
      body<R, 1>(__VA_ARGS__);    \
    else                          \
      body<R, 2>(__VA_ARGS__);    \
  } while (0)

template <class R>
__global__ void __launch_bounds__(SWIT_VEC_BLOCK, SWIT_VEC_MINB_FP_BLK(R)) k_fwd_p_v(Grid<R> g, VecList L, Sources src, const R* __restrict__ s_fwd, R* P,
                                                 const R* __restrict__ U, const R* __restrict__ W, int it, int shot0) {
  VecIdx v;
  int t;
  const bool ok = list_index(g, L, shot0, v, t);
  pdl_enter();
  if (!ok) return;
  const size_t off = (size_t)v.s * g.FSZ;
  SWIT_TIER_CALL(fwd_p_body, g, src, s_fwd, P + off, U + off, W + off, it, v);
}

// Forward velocity phase (fdcore.f90:97-159).
template <class R, int T>
__device__ __forceinline__ void fwd_uw_body(const Grid<R>& g, const Receivers& rec, const R* __restrict__ p, R* __restrict__ u,
                                            R* __restrict__ w, R* __restrict__ seis_t, R* __restrict__ strips, int it,
                                            const VecIdx& v) {
  constexpr bool CHK = T == 2;
  const int LD4 = g.LD >> 2, ix = v.ix, iz0 = v.iz0, fs = g.fs, NZ = g.NZ, NX = g.NX, L = g.L;
  const V4<R> p0 = ld4(p, v.k4);
  V4<R> uv = ld4(u, v.k4), wv = ld4(w, v.k4);
  bool du = false, dw = false;
  if (!CHK || (iz0 + 3 >= fs && iz0 <= NZ - 1 && ix >= 2 && ix <= NX - 1)) {
    const V4<R> b = ld4(g.B, v.kc);
    const V4<R> kw = kappa4<R, T>(g.kw, v);
    if (!CHK || ix <= NX - 2) {
      const V4<R> ku = kappa4<R, T>(g.ku, v);
      const V4<R> pp1 = ld4(p, v.k4 + LD4), pp2 = ld4(p, v.k4 + 2 * LD4), pm1 = ld4(p, v.k4 - LD4);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int iz = iz0 + j;
        if (!CHK || (iz >= fs && iz <= NZ - 1)) {
          const R kappa = T == 0 ? R(0) : ku.x[j];
          uv.x[j] = (R(1.0) - kappa) * uv.x[j] - b.x[j] * (g.c1 * (pp1.x[j] - p0.x[j]) + g.c2 * (pp2.x[j] - pm1.x[j]));
        }
      }
      du = true;
    }
    R pz[7];  // p at rows iz0-1 .. iz0+5
    col_window(p, v, LD4, p0, pz, -1, 2);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int iz = iz0 + j;
      if (!CHK || (iz >= fs && iz <= NZ - 2)) {
        const R kappa = T == 0 ? R(0) : kw.x[j];
        wv.x[j] = (R(1.0) - kappa) * wv.x[j] - b.x[j] * (g.c1 * (pz[j + 2] - pz[j + 1]) + g.c2 * (pz[j + 3] - pz[j]));
      }
    }
    dw = true;
  }
  if (CHK) {
    // w(fs-1, ix) = w(fs, ix) for every column (fdcore.f90:116-120).  If row
    // fs-1 ends the vector above, that vector (rows < fs) has no u or w update
    // and its owner stores nothing; the owner of row fs writes the mirror.
    const int jm = fs - 1 - iz0, jr = fs - iz0;
    if (g.fs_flag == 1 && jr >= 0 && jr < 4) {
      if (jm >= 0) {
        wv.x[jm] = wv.x[jr];
        dw = true;
      } else {
        w[(v.k4 - v.q) * 4 + (fs - 2)] = wv.x[jr];
      }
    }
  }
  if (du) st4(u, v.k4, uv);
  if (dw) st4(w, v.k4, wv);
  if (!CHK) return;
  // receivers (fdcore.f90:123-128)
  if (iz0 + 3 >= rec.zlo[v.s] && iz0 <= rec.zhi[v.s]) {
    const int* cp = rec.colptr + (size_t)v.s * (NX + 2);
    const int e1 = cp[ix + 1];
    for (int e = cp[ix]; e < e1; ++e) {
      const int j = rec.zrow[e] - iz0;
      // vx / vz receivers record u / w after their update (dev/solver/fdcore.f90:162-175)
      if (j >= 0 && j < 4)
        seis_t[((size_t)v.s * g.nt + (it - 1)) * g.ngmax + rec.ig[e]] =
            rec.comp == 1 ? uv.x[j] : (rec.comp == 2 ? wv.x[j] : p0.x[j]);
    }
  }
  // boundary strips of step it (fdcore.f90:130-159)
  const bool strip_rows = (iz0 <= fs + 2 && iz0 + 3 >= fs) || (iz0 <= NZ - L && iz0 + 3 >= NZ - L - 1);
  const bool strip_cols = ix == L + 1 || ix == L + 2 || ix == NX - L || ix == NX - L - 1;
  if (strips && (strip_rows || strip_cols)) {
    R* bs = strips + ((size_t)v.s * g.snt + (it - g.sit0)) * g.SL;
    const StripOff o = strip_offsets(g.nx, g.nz);
    const int jx = ix - L;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int iz = iz0 + j, jz = iz - L;
      if (jx >= 1 && jx <= g.nx) {
        if (iz == NZ - L) bs[o.B0 + jx - 1] = p0.x[j];
        if (iz == NZ - L - 1) {
          bs[o.B1 + jx - 1] = p0.x[j];
          bs[o.B2 + jx - 1] = wv.x[j];
        }
        if (iz == fs) {
          bs[o.T0 + jx - 1] = p0.x[j];
          bs[o.T3 + jx - 1] = uv.x[j];
          bs[o.T5 + jx - 1] = wv.x[j];
        }
        if (iz == fs + 1) {
          bs[o.T1 + jx - 1] = p0.x[j];
          bs[o.T4 + jx - 1] = uv.x[j];
        }
        if (iz == fs + 2) bs[o.T2 + jx - 1] = p0.x[j];
      }
      if (jz >= 1 && jz <= g.nz) {
        if (ix == L + 1) {
          bs[o.S0 + jz - 1] = p0.x[j];
          bs[o.S2 + jz - 1] = uv.x[j];
        }
        if (ix == L + 2) bs[o.S1 + jz - 1] = p0.x[j];
        if (ix == NX - L) bs[o.S3 + jz - 1] = p0.x[j];
        if (ix == NX - L - 1) {
          bs[o.S4 + jz - 1] = p0.x[j];
          bs[o.S5 + jz - 1] = uv.x[j];
        }
      }
    }
  }
}

template <class R>
__global__ void __launch_bounds__(SWIT_VEC_BLOCK, SWIT_VEC_MINB_BLK(R)) k_fwd_uw_v(Grid<R> g, VecList L, Receivers rec, const R* __restrict__ P, R* U,
                                                  R* W, R* __restrict__ seis_t, R* __restrict__ strips, int it,
                                                  int shot0) {
  VecIdx v;
  int t;
  const bool ok = list_index(g, L, shot0, v, t);
  pdl_enter();
  if (!ok) return;
  const size_t off = (size_t)v.s * g.FSZ;
  SWIT_TIER_CALL(fwd_uw_body, g, rec, P + off, U + off, W + off, seis_t, strips, it, v);
}

// ---------------------------------------------------------------------------
// Backward velocity phase: adjoint u, w (fdcore.f90:309-333) and the
// reconstruction u, w with their re-insert (fdcore.f90:220-247).
template <class R, int T>
__device__ __forceinline__ void bwd_uw_body(const Grid<R>& g, const R* __restrict__ pb, R* __restrict__ ub, R* __restrict__ wb,
                                            const R* __restrict__ pe, R* __restrict__ ue, R* __restrict__ we, const R* __restrict__ strips,
                                            int it, const VecIdx& v) {
  constexpr bool CHK = T == 2;
  const int LD4 = g.LD >> 2, ix = v.ix, iz0 = v.iz0, fs = g.fs, NZ = g.NZ, NX = g.NX, L = g.L;
  // ---- adjoint: u on ix in [2, NX-2], iz in [2, NZ-1]; w on ix in [2, NX-1], iz in [2, NZ-2]
  if (!CHK || (ix >= 2 && ix <= NX - 1 && iz0 <= NZ - 1)) {
    const V4<R> a = ld4(g.A, v.kc);
    const V4<R> p0 = ld4(pb, v.k4);
    const V4<R> kw = kappa4<R, T>(g.kw, v);
    if (!CHK || ix <= NX - 2) {
      const V4<R> ku = kappa4<R, T>(g.ku, v);
      V4<R> uv = ld4(ub, v.k4);
      const V4<R> pp1 = ld4(pb, v.k4 + LD4), pp2 = ld4(pb, v.k4 + 2 * LD4), pm1 = ld4(pb, v.k4 - LD4);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int iz = iz0 + j;
        if (!CHK || (iz >= 2 && iz <= NZ - 1)) {
          const R kappa = T == 0 ? R(0) : ku.x[j];
          uv.x[j] = (R(1.0) - kappa) * uv.x[j] - a.x[j] * (g.c1 * (pp1.x[j] - p0.x[j]) + g.c2 * (pp2.x[j] - pm1.x[j]));
        }
      }
      st4(ub, v.k4, uv);
    }
    V4<R> wv = ld4(wb, v.k4);
    R pz[7];  // pb at rows iz0-1 .. iz0+5
    col_window(pb, v, LD4, p0, pz, -1, 2);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int iz = iz0 + j;
      if (!CHK || (iz >= 2 && iz <= NZ - 2)) {
        const R kappa = T == 0 ? R(0) : kw.x[j];
        wv.x[j] = (R(1.0) - kappa) * wv.x[j] - a.x[j] * (g.c1 * (pz[j + 2] - pz[j + 1]) + g.c2 * (pz[j + 3] - pz[j]));
      }
    }
    if (!CHK) {
      st4(wb, v.k4, wv);
    } else {
      // w(fs-1, ix) = w(fs, ix) for ix in [2, NX-1] (fdcore.f90:329-333).  When
      // row fs-1 ends the vector above, the owner of row fs writes it and that
      // vector's owner stores its other three rows.
      const int jm = fs - 1 - iz0, jr = fs - iz0;
      if (g.fs_flag == 1 && jr == 0) wb[(v.k4 - v.q) * 4 + (fs - 2)] = wv.x[0];
      if (g.fs_flag == 1 && jm >= 0 && jm < 4) {
        if (jr < 4) {
          wv.x[jm] = wv.x[jr];
          st4(wb, v.k4, wv);
        } else {
          st4_except(wb, v.k4, wv, jm);
        }
      } else {
        st4(wb, v.k4, wv);
      }
    }
  }
  // ---- reconstruction on the interior
  const int jx = ix - L, jz0 = iz0 - L;
  if (T == 1 || (CHK && (jx < 1 || jx > g.nx || jz0 + 3 < 1 || jz0 > g.nz))) return;
  const int nx = g.nx, nz = g.nz, fsi = fs - L;
  const V4<R> bb = ld4(g.B, v.kc);
  const V4<R> e0 = ld4(pe, v.k4);
  V4<R> uv = ld4(ue, v.k4), wv = ld4(we, v.k4);
  if (!CHK || (jx >= 2 && jx <= nx - 2)) {
    const V4<R> ep1 = ld4(pe, v.k4 + LD4), ep2 = ld4(pe, v.k4 + 2 * LD4), em1 = ld4(pe, v.k4 - LD4);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int jz = jz0 + j;
      if (!CHK || (jz >= fsi + 1 && jz <= nz - 1))
        uv.x[j] = uv.x[j] + bb.x[j] * (g.c1 * (ep1.x[j] - e0.x[j]) + g.c2 * (ep2.x[j] - em1.x[j]));
    }
  }
  if (!CHK || (jx >= 2 && jx <= nx - 1)) {
    R ez[7];  // pe at rows iz0-1 .. iz0+5 (zero outside the interior)
    col_window(pe, v, LD4, e0, ez, -1, 2);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int jz = jz0 + j;
      if (!CHK || (jz >= fsi + 1 && jz <= nz - 2))
        wv.x[j] = wv.x[j] + bb.x[j] * (g.c1 * (ez[j + 2] - ez[j + 1]) + g.c2 * (ez[j + 3] - ez[j]));
    }
  }
  if (CHK) {
    const R* b = strips + ((size_t)v.s * g.snt + (it - 1 - g.sit0)) * g.SL;  // boundary(:, it-1)
    const StripOff o = strip_offsets(nx, nz);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int jz = jz0 + j;
      if (jz < 1 || jz > nz) continue;
      if (jz == nz - 1) wv.x[j] = b[o.B2 + jx - 1];
      if (jx == 1) uv.x[j] = b[o.S2 + jz - 1];
      if (jx == nx - 1) uv.x[j] = b[o.S5 + jz - 1];
    }
  }
  st4(ue, v.k4, uv);
  st4(we, v.k4, wv);
}

template <class R>
__global__ void __launch_bounds__(SWIT_VEC_BLOCK, SWIT_VEC_MINB_BUW_BLK(R)) k_bwd_uw_v(Grid<R> g, VecList L, const R* __restrict__ PB, R* UB, R* WB,
                                                  const R* __restrict__ PE, R* UE, R* WE,
                                                  const R* __restrict__ strips, int it, int shot0) {
  VecIdx v;
  int t;
  const bool ok = list_index(g, L, shot0, v, t);
  pdl_enter();
  if (!ok) return;
  const size_t off = (size_t)v.s * g.FSZ;
  SWIT_TIER_CALL(bwd_uw_body, g, PB + off, UB + off, WB + off, PE + off, UE + off, WE + off, strips, it, v);
}

// ---------------------------------------------------------------------------
// Backward pressure phase: adjoint p + injection + mirror (fdcore.f90:336-373),
// reconstruction p with source subtraction and re-insert (fdcore.f90:249-287),
// imaging sums (solver.f90:237-239).
template <class R, int T>
__device__ __forceinline__ void bwd_p_body(const Grid<R>& g, const Receivers& rec, const Sources& src,
                                           const R* __restrict__ s_fwd, const R* __restrict__ adj_t, R* __restrict__ pb,
                                           const R* __restrict__ ub, const R* __restrict__ wb, R* __restrict__ pe,
                                           const R* __restrict__ ue, const R* __restrict__ we, R* __restrict__ dg, R* __restrict__ dfw, R* __restrict__ dbk,
                                           const R* __restrict__ strips, int it, const VecIdx& v) {
  constexpr bool CHK = T == 2;
  const int LD4 = g.LD >> 2, ix = v.ix, iz0 = v.iz0, fs = g.fs, NZ = g.NZ, NX = g.NX, L = g.L;
  const V4<R> pold = ld4(pb, v.k4);
  V4<R> pv = pold;
  bool dirty = false;
  if (!CHK || (ix >= 3 && ix <= NX - 2 && iz0 + 3 >= 3 && iz0 <= NZ - 2)) {
    const V4<R> bcoef = ld4(g.B, v.kc);
    const V4<R> kk = kappa4<R, T>(g.kp, v);
    const V4<R> u0 = ld4(ub, v.k4), um1 = ld4(ub, v.k4 - LD4), up1 = ld4(ub, v.k4 + LD4), um2 = ld4(ub, v.k4 - 2 * LD4);
    R wz[7];  // wb at rows iz0-2 .. iz0+4
    col_window(wb, v, LD4, ld4(wb, v.k4), wz, -2, 1);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int iz = iz0 + j;
      if (!CHK || (iz >= 3 && iz <= NZ - 2)) {
        const R kappa = T == 0 ? R(0) : kk.x[j];
        pv.x[j] = (R(1.0) - kappa) * pv.x[j] -
                  bcoef.x[j] * (g.c1 * (u0.x[j] - um1.x[j] + wz[j + 2] - wz[j + 1]) +
                                g.c2 * (up1.x[j] - um2.x[j] + wz[j + 3] - wz[j]));
      }
    }
    dirty = true;
  }
  if (!CHK) {
    st4(pb, v.k4, pv);
  } else {
    if (rec.comp == 0 && iz0 + 3 >= rec.zlo[v.s] && iz0 <= rec.zhi[v.s]) {
      const int* cp = rec.colptr + (size_t)v.s * (NX + 2);
      const int e1 = cp[ix + 1];
      for (int e = cp[ix]; e < e1; ++e) {
        const int j = rec.zrow[e] - iz0;
        if (j >= 0 && j < 4) {
          pv.x[j] = pv.x[j] + g.dt * adj_t[((size_t)v.s * g.nt + (it - 1)) * g.ngmax + rec.ig[e]];
          dirty = true;
        }
      }
    }
    // p(fs-1, ix) = -p(fs+1, ix) for every column (fdcore.f90:370-373).  When
    // row fs-1 lies in the vector above, the owner of row fs+1 writes it and
    // that vector's owner stores its other rows.
    const int jm = fs - 1 - iz0, jp = fs + 1 - iz0;
    if (jp >= 0 && jp < 4 && jm < 0) pb[(v.k4 - v.q) * 4 + (fs - 2)] = -pv.x[jp];
    if (jm >= 0 && jm < 4) {
      if (jp < 4) {
        pv.x[jm] = -pv.x[jp];
        st4(pb, v.k4, pv);
      } else {
        st4_except(pb, v.k4, pv, jm);
      }
    } else if (dirty) {
      st4(pb, v.k4, pv);
    }
  }

  // ---- reconstruction p, re-insert, imaging on the interior
  const int jx = ix - L, jz0 = iz0 - L;
  if (T == 1 || (CHK && (jx < 1 || jx > g.nx || jz0 + 3 < 1 || jz0 > g.nz))) return;
  const int nx = g.nx, nz = g.nz, fsi = fs - L;
  V4<R> ev = ld4(pe, v.k4);
  if (CHK) {
    const int rj = src.risz[v.s] - jz0;
    if (jx == src.risx[v.s] && rj >= 0 && rj < 4) ev.x[rj] = ev.x[rj] - g.dt * s_fwd[(size_t)v.s * (g.nt + 1) + it];
  }
  if (!CHK || (jx >= 3 && jx <= nx - 2)) {
    const V4<R> a = ld4(g.A, v.kc);
    const V4<R> u0 = ld4(ue, v.k4), um1 = ld4(ue, v.k4 - LD4), up1 = ld4(ue, v.k4 + LD4), um2 = ld4(ue, v.k4 - 2 * LD4);
    R wz[7];  // we at rows iz0-2 .. iz0+4
    col_window(we, v, LD4, ld4(we, v.k4), wz, -2, 1);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int jz = jz0 + j;
      if (!CHK || (jz >= fsi + 2 && jz <= nz - 2))
        ev.x[j] = ev.x[j] + a.x[j] * (g.c1 * (u0.x[j] - um1.x[j] + wz[j + 2] - wz[j + 1]) +
                                      g.c2 * (up1.x[j] - um2.x[j] + wz[j + 3] - wz[j]));
    }
  }
  V4<R> g0 = ld4(dg, v.kg), f0 = ld4(dfw, v.kg), k0 = ld4(dbk, v.kg);
  const R* b = CHK ? strips + ((size_t)v.s * g.snt + (it - 1 - g.sit0)) * g.SL : nullptr;
  const StripOff o = strip_offsets(nx, nz);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int jz = jz0 + j;
    if (CHK && (jz < 1 || jz > nz)) continue;
    R pf = ev.x[j];
    if (CHK) {
      if (jz == nz) pf = b[o.B0 + jx - 1];
      if (jz == nz - 1) pf = b[o.B1 + jx - 1];
      if (jx == 1) pf = b[o.S0 + jz - 1];
      if (jx == 2) pf = b[o.S1 + jz - 1];
      if (jx == nx) pf = b[o.S3 + jz - 1];
      if (jx == nx - 1) pf = b[o.S4 + jz - 1];
      if (jz == fsi) pf = b[o.T0 + jx - 1];
      if (jz == fsi + 1) pf = b[o.T1 + jx - 1];
      if (jz == fsi + 2) pf = b[o.T2 + jx - 1];
    }
    ev.x[j] = pf;
    g0.x[j] = g0.x[j] + pf * (pold.x[j] - pv.x[j]);
    f0.x[j] = f0.x[j] + pf * pf;
    k0.x[j] = k0.x[j] + pv.x[j] * pv.x[j];
  }
  st4(pe, v.k4, ev);
  st4(dg, v.kg, g0);
  st4(dfw, v.kg, f0);
  st4(dbk, v.kg, k0);
}

// dg, dfw, dbk are the shot's imaging sums (indexed by v.kg).
template <class R>
__global__ void __launch_bounds__(SWIT_VEC_BLOCK, SWIT_VEC_MINB_BLK(R)) k_bwd_p_v(Grid<R> g, VecList L, Receivers rec, Sources src,
                                                 const R* __restrict__ s_fwd, const R* __restrict__ adj_t, R* PB,
                                                 const R* __restrict__ UB, const R* __restrict__ WB, R* PE,
                                                 const R* __restrict__ UE, const R* __restrict__ WE, R* DG, R* DFW,
                                                 R* DBK, const R* __restrict__ strips, int it, int shot0) {
  VecIdx v;
  int t;
  const bool ok = list_index(g, L, shot0, v, t);
  pdl_enter();
  if (!ok) return;
  const size_t off = (size_t)v.s * g.FSZ;
  SWIT_TIER_CALL(bwd_p_body, g, rec, src, s_fwd, adj_t, PB + off, UB + off, WB + off, PE + off, UE + off, WE + off,
                 DG + off, DFW + off, DBK + off, strips, it, v);
}

// Body tier of every vector for each phase kernel (fwd_p, fwd_uw, bwd_uw,
// bwd_p), the highest any shot needs; 3 where the phase does no work: rows
// above fs-1 in the forward (no update, mirror, source, receiver or strip
// there) and rows from NZ on.  out[k * NX * LD/4 + (ix-1) * LD/4 + q].
// vx / vz receivers: after the adjoint pressure phase of reverse step it, the
// adjoint source of step it goes into u or w at the receiver point
// (dev/solver/fdcore.f90:472-485: u(z, igx) = u(z, igx) - dt s(it, ig)), in
// receiver order; one thread per column and shot.
template <class R>
__global__ void k_inject_vel(Grid<R> g, Receivers rec, const R* __restrict__ adj_t, R* UB, R* WB, int it,
                             int shot0) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int s = shot0 + blockIdx.y;
  pdl_enter();
  if (ix > g.NX) return;
  const int* cp = rec.colptr + (size_t)s * (g.NX + 2);
  const int e1 = cp[ix + 1];
  if (cp[ix] == e1) return;
  R* f = (rec.comp == 1 ? UB : WB) + (size_t)s * g.FSZ + (size_t)(ix - 1) * g.LD;
  for (int e = cp[ix]; e < e1; ++e) {
    const int z = rec.zrow[e];
    f[z - 1] = f[z - 1] - g.dt * adj_t[((size_t)s * g.nt + (it - 1)) * g.ngmax + rec.ig[e]];
  }
}

template <class R>
__global__ void k_tiers(Grid<R> g, Sources src, Receivers rec, int ns, int* out) {
  const int LD4 = g.LD >> 2;
  const size_t n = (size_t)g.NX * LD4;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    VecIdx v;
    v.ix = (int)(t / LD4) + 1;
    v.q = (int)(t % LD4);
    v.iz0 = 4 * v.q + 1;
    vec_flags(g, v);
    int a = 0, b = 0, c = 0, d = 0;
    for (int s = 0; s < ns; ++s) {
      const bool fsrc = v.ix == src.isx[s] && src.isz[s] >= v.iz0 && src.isz[s] < v.iz0 + 4;
      const bool rh = v.iz0 + 3 >= rec.zlo[s] && v.iz0 <= rec.zhi[s];
      const int rz = src.risz[s] + g.L;
      const bool bsrc = src.risx[s] + g.L == v.ix && rz >= v.iz0 && rz < v.iz0 + 4;
      a = max(a, tier_fwd_p(g, v, fsrc));
      b = max(b, tier_fwd_uw(g, v, rh));
      c = max(c, tier_bwd_uw(g, v));
      d = max(d, tier_bwd_p(g, v, rh, bsrc));
    }
    const bool fskip = v.iz0 + 3 <= g.fs - 1 || v.iz0 >= g.NZ, bskip = v.iz0 >= g.NZ;
    out[t] = fskip ? 3 : a;
    out[n + t] = fskip ? 3 : b;
    out[2 * n + t] = bskip ? 3 : c;
    out[3 * n + t] = bskip ? 3 : d;
  }
}

}  // namespace swit
