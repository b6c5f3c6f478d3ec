// kernels_cluster.cuh -- cluster-persistent time loops: one thread-block
// cluster per shot keeps the shot's wavefields in distributed shared memory
// for the whole forward (or reverse) time loop.
//
// The NX columns of a shot are split over the C CTAs of a cluster (balanced,
// at least two columns each).  A CTA holds its columns plus two ghost columns
// on either side of every field, each column LD/4 vectors of 4 rows, so the
// vector bodies of kernels_vec.cuh run unchanged on shared-memory arrays.  After
// each phase a CTA stores its two first and two last columns of the fields the
// next phase differentiates along x into the neighbours' ghost columns
// (st.shared::cluster), and a cluster barrier (release/acquire) publishes them:
//   forward  p phase -> send p -> barrier -> u,w phase -> send u -> barrier
//   reverse  u,w phase -> send ub, ue -> barrier -> p phase -> send pb, pe -> barrier
// Reading a ghost of step t always follows the barrier after it was written,
// and rewriting it follows the barrier after its last read, so two cluster
// barriers per time step order every shared-memory access.  Every thread of
// the cluster executes every barrier (there is no early exit), so the loops
// cannot wait on a CTA that has left.
//
// Only the boundary strips, receiver traces, source samples, coefficient
// arrays (when they do not fit on chip) and the imaging sums touch global
// memory inside the loop.
#pragma once
#include <cooperative_groups.h>

#include "kernels_vec.cuh"

namespace swit {
namespace cg = cooperative_groups;

// Columns [x0, x0 + ncol) (1-based) of CTA r of C.
__host__ __device__ __forceinline__ void cl_cols(int NX, int C, int r, int& x0, int& ncol) {
  const int b = NX / C, m = NX % C;
  ncol = b + (r < m ? 1 : 0);
  x0 = 1 + r * b + (r < m ? r : m);
}

// Vector (column c of this CTA, vector q) -> index set.  Fields in shared
// memory: column c at local column c + 2.  Coefficients: a local copy without
// ghosts (ab_local) or the global arrays.  Imaging sums: the shot's global arrays.
template <class R>
__device__ __forceinline__ VecIdx cl_index(const Grid<R>& g, int s, int x0, int c, int q, bool ab_local) {
  VecIdx v;
  const int LD4 = g.LD >> 2;
  v.s = s;
  v.q = q;
  v.ix = x0 + c;
  v.iz0 = 4 * q + 1;
  v.ok = true;
  v.k4 = (size_t)(c + 2) * LD4 + q;
  v.kg = (size_t)(v.ix - 1) * LD4 + q;
  v.kc = ab_local ? (size_t)c * LD4 + q : v.kg;
  vec_flags(g, v);
  return v;
}

// Own columns 0, 1 -> left neighbour's right ghosts; own columns ncol-2,
// ncol-1 -> right neighbour's left ghosts: 4 columns of LD4 vectors.
template <class R>
__device__ __forceinline__ void cl_send(cg::cluster_group& cl, R* f, int r, int C, int ncol, int ncol_left, int LD4) {
  for (int i = threadIdx.x; i < 4 * LD4; i += blockDim.x) {
    const int j = i / LD4, q = i - j * LD4;
    int dst, mine, theirs;
    if (j < 2) {
      if (r == 0) continue;
      dst = r - 1;
      mine = 2 + j;
      theirs = ncol_left + 2 + j;
    } else {
      if (r == C - 1) continue;
      dst = r + 1;
      mine = ncol + (j - 2);
      theirs = j - 2;
    }
    R* remote = cl.map_shared_rank(f, (unsigned)dst);
    st4(remote, (size_t)theirs * LD4 + q, ld4(f, (size_t)mine * LD4 + q));
  }
}

// Task list of a CTA: its vectors (c, q), packed c << 16 | q, grouped by body
// tier cat(c, q) in {0, 1, 2} (kernels_vec.cuh), each group in column-major
// order, so 32 consecutive entries run one body; cat 3 = a vector on which the
// loop does no work, left out.  n[0] = first vector of tier 1, n[1] = first of
// tier 2, n[2] = length.  Contains __syncthreads; blockDim.x is a multiple of
// 32 and every thread calls it.
template <class Cat>
__device__ __forceinline__ void cl_tasks(uint32_t* list, int ncol, int LD4, Cat cat, int n[3]) {
  __shared__ int s_cnt[3][32];
  __shared__ int s_off[3];
  __shared__ int s_len;
  const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nthr >> 5;
  const int ntask = ncol * LD4;
  int c0 = 0, c1 = 0, c2 = 0;
  for (int t = tid; t < ntask; t += nthr) {
    const int k = cat(t / LD4, t % LD4);
    c0 += k == 0;
    c1 += k == 1;
    c2 += k == 2;
  }
  for (int o = 16; o > 0; o >>= 1) {
    c0 += __shfl_xor_sync(0xffffffffu, c0, o);
    c1 += __shfl_xor_sync(0xffffffffu, c1, o);
    c2 += __shfl_xor_sync(0xffffffffu, c2, o);
  }
  if (lane == 0) {
    s_cnt[0][wid] = c0;
    s_cnt[1][wid] = c1;
    s_cnt[2][wid] = c2;
  }
  __syncthreads();
  if (tid == 0) {
    int a = 0, b = 0, c = 0;
    for (int w = 0; w < nw; ++w) {
      a += s_cnt[0][w];
      b += s_cnt[1][w];
      c += s_cnt[2][w];
    }
    s_off[0] = 0;
    s_off[1] = a;
    s_off[2] = a + b;
    s_len = a + b + c;
  }
  __syncthreads();
  n[0] = s_off[1];
  n[1] = s_off[2];
  n[2] = s_len;
  const unsigned lt = (1u << lane) - 1u;
  for (int b = 0; b < ntask; b += nthr) {
    const int t = b + tid;
    const int k = t < ntask ? cat(t / LD4, t % LD4) : 3;
    const unsigned m0 = __ballot_sync(0xffffffffu, k == 0), m1 = __ballot_sync(0xffffffffu, k == 1),
                   m2 = __ballot_sync(0xffffffffu, k == 2);
    if (lane == 0) {
      s_cnt[0][wid] = __popc(m0);
      s_cnt[1][wid] = __popc(m1);
      s_cnt[2][wid] = __popc(m2);
    }
    __syncthreads();
    if (k < 3) {
      int o = s_off[k];
      for (int w = 0; w < wid; ++w) o += s_cnt[k][w];
      const unsigned m = k == 0 ? m0 : (k == 1 ? m1 : m2);
      list[o + __popc(m & lt)] = ((uint32_t)(t / LD4) << 16) | (uint32_t)(t % LD4);
    }
    __syncthreads();
    if (tid < 3) {
      int a = 0;
      for (int w = 0; w < nw; ++w) a += s_cnt[tid][w];
      s_off[tid] += a;
    }
    __syncthreads();
  }
}

// Dynamic schedule of a phase: warps claim groups of 32 consecutive list
// entries from an on-chip counter, the last group (general tier) first, so
// warps that finish early take more work and the strip and trace stores of the
// general vectors are issued early.  f(i) runs entry i.  The caller resets the
// counter behind a barrier before the phase runs again.
template <class F>
__device__ __forceinline__ void cl_run(int* ctr, int nlist, F f) {
  const int lane = threadIdx.x & 31, ngrp = (nlist + 31) >> 5;
  for (;;) {
    int k = 0;
    if (lane == 0) k = atomicAdd(ctr, 1);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= ngrp) break;
    const int i = (ngrp - 1 - k) * 32 + lane;
    if (i < nlist) f(i);
  }
}

template <class R>
__device__ __forceinline__ V4<R> zero4() {
  V4<R> z;
#pragma unroll
  for (int j = 0; j < 4; ++j) z.x[j] = R(0);
  return z;
}

// Shared memory of a cluster CTA (elements of R, then the task list): nf
// fields of ceil(NX/C) + 4 columns, nab coefficient arrays of ceil(NX/C)
// columns, LD values per column; ceil(NX/C) * LD/4 list entries.
__host__ __device__ __forceinline__ size_t cl_field_elems(int NX, int C, int LD, int nf, int nab) {
  const int ncmax = (NX + C - 1) / C;
  return ((size_t)nf * (ncmax + 4) + (size_t)nab * ncmax) * LD;
}
__host__ __device__ __forceinline__ size_t cl_list_entries(int NX, int C, int LD) {
  return (size_t)((NX + C - 1) / C) * (LD / 4);
}

// Forward time loop of one shot per cluster (fdcore.f90:75-160).  Launch: grid
// (C, shots), cluster (C, 1, 1), MAXT threads; dynamic shared memory for 3
// fields (+ A and B when ab_local) and the task list.  The final state is
// written to P, U, W.
template <class R, int MAXT>
__global__ void __launch_bounds__(MAXT, 1)
    k_fwd_cl(Grid<R> g, Sources src, Receivers rec, const R* __restrict__ s_fwd, R* __restrict__ P,
             R* __restrict__ U, R* __restrict__ W, R* __restrict__ seis_t, R* __restrict__ strips, int shot0,
             int ab_local) {
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks(), r = (int)cl.block_rank();
  const int s = shot0 + blockIdx.y;
  const int LD = g.LD, LD4 = LD >> 2;
  int x0, ncol, xl, ncl;
  cl_cols(g.NX, C, r, x0, ncol);
  cl_cols(g.NX, C, r > 0 ? r - 1 : 0, xl, ncl);
  const int ncmax = (g.NX + C - 1) / C, NCW = ncmax + 4;
  extern __shared__ __align__(16) unsigned char cl_smem[];
  R* p = reinterpret_cast<R*>(cl_smem);
  R* u = p + (size_t)NCW * LD;
  R* w = u + (size_t)NCW * LD;
  uint32_t* list = reinterpret_cast<uint32_t*>(p + cl_field_elems(g.NX, C, LD, 3, ab_local ? 2 : 0));
  const int tid = threadIdx.x, nthr = blockDim.x;
  for (size_t i = tid; i < (size_t)3 * NCW * LD4; i += nthr) st4(p, i, zero4<R>());
  Grid<R> gl = g;
  if (ab_local) {
    R* a = w + (size_t)NCW * LD;
    R* b = a + (size_t)ncmax * LD;
    for (int i = tid; i < ncol * LD4; i += nthr) {
      const size_t kg = (size_t)(x0 - 1) * LD4 + i;
      st4(a, (size_t)i, ld4(g.A, kg));
      st4(b, (size_t)i, ld4(g.B, kg));
    }
    gl.A = a;
    gl.B = b;
  }
  const int isx = src.isx[s], isz = src.isz[s], zlo = rec.zlo[s], zhi = rec.zhi[s];
  int nt01[3];
  cl_tasks(list, ncol, LD4, [=](int c, int q) {
    VecIdx v;
    v.ix = x0 + c;
    v.iz0 = 4 * q + 1;
    vec_flags(g, v);
    const bool src_here = v.ix == isx && isz >= v.iz0 && isz < v.iz0 + 4;
    const bool rec_here = v.iz0 + 3 >= zlo && v.iz0 <= zhi;
    // rows above fs-1 and below NZ-1 take no update, mirror, source, receiver or strip
    if (v.iz0 + 3 <= g.fs - 1 || v.iz0 >= g.NZ) return 3;
    return max(tier_fwd_p(g, v, src_here), tier_fwd_uw(g, v, rec_here));
  }, nt01);
  const int n0 = nt01[0], n1 = nt01[1], nlist = nt01[2];
  const bool abl = ab_local != 0;
  __shared__ int s_ctr[2];
  if (tid < 2) s_ctr[tid] = 0;
  cl.sync();
  for (int it = 2; it <= g.nt; ++it) {
    cl_run(&s_ctr[0], nlist, [&](int i) {
      const uint32_t e = list[i];
      const VecIdx v = cl_index(gl, s, x0, (int)(e >> 16), (int)(e & 0xffffu), abl);
      if (i < n0)
        fwd_p_body<R, 0>(gl, src, s_fwd, p, u, w, it, v);
      else if (i < n1)
        fwd_p_body<R, 1>(gl, src, s_fwd, p, u, w, it, v);
      else
        fwd_p_body<R, 2>(gl, src, s_fwd, p, u, w, it, v);
    });
    __syncthreads();
    if (tid == 0) s_ctr[0] = 0;
    cl_send(cl, p, r, C, ncol, ncl, LD4);
    cl.sync();
    cl_run(&s_ctr[1], nlist, [&](int i) {
      const uint32_t e = list[i];
      const VecIdx v = cl_index(gl, s, x0, (int)(e >> 16), (int)(e & 0xffffu), abl);
      if (i < n0)
        fwd_uw_body<R, 0>(gl, rec, p, u, w, seis_t, strips, it, v);
      else if (i < n1)
        fwd_uw_body<R, 1>(gl, rec, p, u, w, seis_t, strips, it, v);
      else
        fwd_uw_body<R, 2>(gl, rec, p, u, w, seis_t, strips, it, v);
    });
    __syncthreads();
    if (tid == 0) s_ctr[1] = 0;
    cl_send(cl, u, r, C, ncol, ncl, LD4);
    cl.sync();
  }
  const size_t off = (size_t)s * g.FSZ;
  for (int i = tid; i < ncol * LD4; i += nthr) {
    const size_t kl = (size_t)2 * LD4 + i, kg = (size_t)(x0 - 1) * LD4 + i;
    st4(P + off, kg, ld4(p, kl));
    st4(U + off, kg, ld4(u, kl));
    st4(W + off, kg, ld4(w, kl));
  }
}

// Reverse time loop of one shot per cluster (solver.f90:230-253 with
// fdcore.f90:220-287, 309-373): adjoint pb, ub, wb from zero, reconstruction
// pe, ue, we from the final forward state in PE, UE, WE (PML layout), imaging
// sums accumulated in the shot's DG, DFW, DBK.  Dynamic shared memory: 6 fields
// and the task list.
template <class R, int MAXT>
__global__ void __launch_bounds__(MAXT, 1)
    k_bwd_cl(Grid<R> g, Receivers rec, Sources src, const R* __restrict__ s_fwd, const R* __restrict__ adj_t,
             const R* __restrict__ PE, const R* __restrict__ UE, const R* __restrict__ WE, R* __restrict__ DG,
             R* __restrict__ DFW, R* __restrict__ DBK, const R* __restrict__ strips, int shot0) {
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks(), r = (int)cl.block_rank();
  const int s = shot0 + blockIdx.y;
  const int LD = g.LD, LD4 = LD >> 2;
  int x0, ncol, xl, ncl;
  cl_cols(g.NX, C, r, x0, ncol);
  cl_cols(g.NX, C, r > 0 ? r - 1 : 0, xl, ncl);
  const int ncmax = (g.NX + C - 1) / C, NCW = ncmax + 4;
  extern __shared__ __align__(16) unsigned char cl_smem[];
  const size_t F = (size_t)NCW * LD;
  R* pb = reinterpret_cast<R*>(cl_smem);
  R* ub = pb + F;
  R* wb = ub + F;
  R* pe = wb + F;
  R* ue = pe + F;
  R* we = ue + F;
  uint32_t* list = reinterpret_cast<uint32_t*>(pb + cl_field_elems(g.NX, C, LD, 6, 0));
  const int tid = threadIdx.x, nthr = blockDim.x;
  const size_t off = (size_t)s * g.FSZ;
  for (size_t i = tid; i < (size_t)3 * NCW * LD4; i += nthr) st4(pb, i, zero4<R>());
  // reconstruction state, ghosts included, from the global arrays
  for (int i = tid; i < (ncol + 4) * LD4; i += nthr) {
    const int lc = i / LD4, ix = x0 - 2 + lc;
    if (ix >= 1 && ix <= g.NX) {
      const size_t kg = (size_t)(x0 - 3) * LD4 + i;
      st4(pe, (size_t)i, ld4(PE + off, kg));
      st4(ue, (size_t)i, ld4(UE + off, kg));
      st4(we, (size_t)i, ld4(WE + off, kg));
    } else {
      st4(pe, (size_t)i, zero4<R>());
      st4(ue, (size_t)i, zero4<R>());
      st4(we, (size_t)i, zero4<R>());
    }
  }
  const int zlo = rec.zlo[s], zhi = rec.zhi[s];
  const int rsx = src.risx[s] + g.L, rsz = src.risz[s] + g.L;  // risx = 0: none
  int nt01[3];
  cl_tasks(list, ncol, LD4, [=](int c, int q) {
    VecIdx v;
    v.ix = x0 + c;
    v.iz0 = 4 * q + 1;
    vec_flags(g, v);
    const bool rec_here = v.iz0 + 3 >= zlo && v.iz0 <= zhi;
    const bool src_here = rsx == v.ix && rsz >= v.iz0 && rsz < v.iz0 + 4;
    if (v.iz0 >= g.NZ) return 3;  // rows below NZ-1 take no update
    return max(tier_bwd_uw(g, v), tier_bwd_p(g, v, rec_here, src_here));
  }, nt01);
  const int n0 = nt01[0], n1 = nt01[1], nlist = nt01[2];
  __shared__ int s_ctr[2];
  if (tid < 2) s_ctr[tid] = 0;
  cl.sync();
  R* dg = DG + off;
  R* dfw = DFW + off;
  R* dbk = DBK + off;
  for (int it = g.nt; it >= 2; --it) {
    cl_run(&s_ctr[0], nlist, [&](int i) {
      const uint32_t e = list[i];
      const VecIdx v = cl_index(g, s, x0, (int)(e >> 16), (int)(e & 0xffffu), false);
      if (i < n0)
        bwd_uw_body<R, 0>(g, pb, ub, wb, pe, ue, we, strips, it, v);
      else if (i < n1)
        bwd_uw_body<R, 1>(g, pb, ub, wb, pe, ue, we, strips, it, v);
      else
        bwd_uw_body<R, 2>(g, pb, ub, wb, pe, ue, we, strips, it, v);
    });
    __syncthreads();
    if (tid == 0) s_ctr[0] = 0;
    cl_send(cl, ub, r, C, ncol, ncl, LD4);
    cl_send(cl, ue, r, C, ncol, ncl, LD4);
    cl.sync();
    cl_run(&s_ctr[1], nlist, [&](int i) {
      const uint32_t e = list[i];
      const VecIdx v = cl_index(g, s, x0, (int)(e >> 16), (int)(e & 0xffffu), false);
      if (i < n0)
        bwd_p_body<R, 0>(g, rec, src, s_fwd, adj_t, pb, ub, wb, pe, ue, we, dg, dfw, dbk, strips, it, v);
      else if (i < n1)
        bwd_p_body<R, 1>(g, rec, src, s_fwd, adj_t, pb, ub, wb, pe, ue, we, dg, dfw, dbk, strips, it, v);
      else
        bwd_p_body<R, 2>(g, rec, src, s_fwd, adj_t, pb, ub, wb, pe, ue, we, dg, dfw, dbk, strips, it, v);
    });
    __syncthreads();
    if (tid == 0) s_ctr[1] = 0;
    cl_send(cl, pb, r, C, ncol, ncl, LD4);
    cl_send(cl, pe, r, C, ncol, ncl, LD4);
    cl.sync();
  }
}

}  // namespace swit
