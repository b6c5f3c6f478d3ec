// kernels_band.cuh -- the four phase kernels staged through shared memory by
// the bulk-copy (TMA) engine.
//
// A block owns a band of BC consecutive columns (all LD rows) of one shot.
// Columns are contiguous in the PML-grid layout, so each array the phase
// reads is one contiguous range: thread 0 issues one cp.async.bulk per array
// (global -> shared, completion counted on an mbarrier), every thread waits on
// the mbarrier once, runs the vector bodies of kernels_vec.cuh on the shared
// copies, and thread 0 writes the updated arrays back with one bulk store each
// (shared -> global).  Arrays differentiated along x are staged with two halo
// columns either side; the others hold the band only, addressed through a base
// pointer two columns before the copy so that every array uses the same local
// index.  Within a band the vectors are listed by body tier, so a warp runs one
// body.  Blocks update disjoint columns and no phase writes an array it reads
// across columns, so the in-place global update is race-free.
//
// Every wait on the mbarrier is bounded: on timeout the block records it in a
// global error word, waits (again bounded) for its copies in flight and leaves
// without computing; swit_check reports the word.
#pragma once
#include "kernels_vec.cuh"

namespace swit {

// Per-band task lists: entries e[band * stride + i] = (local column) << 16 | q,
// grouped by body tier; cnt[band] = {first tier-1 entry, first tier-2 entry, length}.
struct BandList {
  const uint32_t* __restrict__ e;
  const int4* __restrict__ cnt;
  int stride;
  int bc;         // columns per band
  unsigned wait;  // polls of the mbarrier before a block gives up (kBandWaitLimit unless set lower)
};

constexpr unsigned kBandWaitLimit = 1u << 22;  // polls of the mbarrier before a block gives up
constexpr int kErrBandTimeout = 1;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// Bounded wait for phase `parity` of the mbarrier: at most `limit` polls; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned limit = kBandWaitLimit) {
  const uint32_t a = smem_addr(bar);
  for (unsigned n = 0; n < limit; ++n) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// bytes (a multiple of 16) from global src to shared dst (both 16-byte aligned).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(dst), "r"(smem_addr(src)),
               "r"(bytes)
               : "memory");
}
// Commits the bulk stores and waits until they have completed.
__device__ __forceinline__ void bulk_commit_and_drain() {
  asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
  asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
}
// Generic-proxy shared-memory writes -> visible to the bulk-copy engine.
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// Band geometry of this block.
struct Band {
  int c0, ncol;  // first column (1-based), columns
  int h0, h1;    // halo column range inside [1, NX]
};
template <class R>
__device__ __forceinline__ Band band_of(const Grid<R>& g, int bc) {
  Band b;
  b.c0 = blockIdx.x * bc + 1;
  b.ncol = min(bc, g.NX - b.c0 + 1);
  b.h0 = max(1, b.c0 - 2);
  b.h1 = min(g.NX, b.c0 + b.ncol + 1);
  return b;
}

// List entry i of this band -> vector index set (local indices) and tier.
template <class R>
__device__ __forceinline__ void band_task(const Grid<R>& g, const BandList& L, const Band& b, int s, int i,
                                          const int4& cnt, VecIdx& v, int& t) {
  const uint32_t e = L.e[(size_t)blockIdx.x * L.stride + i];
  const int lc = (int)(e >> 16);
  v.s = s;
  v.q = (int)(e & 0xffffu);
  v.ix = b.c0 + lc;
  v.iz0 = 4 * v.q + 1;
  v.ok = true;
  v.k4 = (size_t)(lc + 2) * (g.LD >> 2) + v.q;
  v.kc = v.k4;
  v.kg = v.k4;
  t = i < cnt.x ? 0 : (i < cnt.y ? 1 : 2);
}

// Waits (at most `limit` polls) for the staged copies; on timeout every thread
// of the block learns it, thread 0 records it and waits once more, with the full
// bound, for the copies in flight, so the block never leaves with a copy still
// writing its shared memory.
__device__ __forceinline__ bool band_ready(uint64_t* bar, int* err, unsigned limit) {
  const bool ok = mbar_wait(bar, 0, limit);
  const bool bad = __syncthreads_or(!ok);
  if (bad && threadIdx.x == 0) {
    atomicOr(err, kErrBandTimeout);
    mbar_wait(bar, 0);
  }
  return !bad;
}

// Shared memory of a band kernel: nh halo arrays of bc + 4 columns and no band
// arrays of bc columns, LD values each.
__host__ __device__ __forceinline__ size_t band_smem(int bc, int LD, int nh, int no, size_t esz) {
  return ((size_t)nh * (bc + 4) + (size_t)no * bc) * LD * esz;
}

#ifndef SWIT_BAND_BLOCKS
#define SWIT_BAND_BLOCKS 4
#endif

// Stages `cols` columns starting at global column x (1-based) of array A (LD
// values per column, shot offset applied by the caller) at local column lc of
// the shared array S.
#define BAND_LOAD(S, lc, A, x, cols) \
  bulk_load((S) + (size_t)(lc) * LD, (A) + (size_t)((x) - 1) * LD, (uint32_t)((cols) * colb), &bar)


// Forward pressure phase (fdcore.f90:77-94) of one band.
template <class R>
__global__ void __launch_bounds__(256, SWIT_BAND_BLOCKS)
    k_fwd_p_b(Grid<R> g, BandList L, Sources src, const R* __restrict__ s_fwd, R* P, const R* __restrict__ U,
              const R* __restrict__ W, int it, int shot0, int* err) {
  extern __shared__ __align__(128) unsigned char band_sm[];
  __shared__ uint64_t bar;
  pdl_enter();
  const int LD = g.LD, bc = L.bc, s = shot0 + blockIdx.y;
  const Band b = band_of(g, bc);
  const size_t off = (size_t)s * g.FSZ, colb = (size_t)LD * sizeof(R);
  R* su = reinterpret_cast<R*>(band_sm);
  R* sp = su + (size_t)(bc + 4) * LD;
  R* sw = sp + (size_t)bc * LD;
  R* sa = sw + (size_t)bc * LD;
  R* sk = sa + (size_t)bc * LD;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(&bar, (uint32_t)(((b.h1 - b.h0 + 1) + 4 * b.ncol) * colb));
    BAND_LOAD(su, b.h0 - b.c0 + 2, U + off, b.h0, b.h1 - b.h0 + 1);
    BAND_LOAD(sp, 0, P + off, b.c0, b.ncol);
    BAND_LOAD(sw, 0, W + off, b.c0, b.ncol);
    BAND_LOAD(sa, 0, g.A, b.c0, b.ncol);
    BAND_LOAD(sk, 0, g.kp, b.c0, b.ncol);
  }
  const int4 cnt = L.cnt[blockIdx.x];
  if (!band_ready(&bar, err, L.wait)) return;
  Grid<R> gl = g;
  gl.A = sa - 2 * LD;
  gl.kp = sk - 2 * LD;
  for (int i = threadIdx.x; i < cnt.z; i += blockDim.x) {
    VecIdx v;
    int t;
    band_task(gl, L, b, s, i, cnt, v, t);
    SWIT_TIER_CALL(fwd_p_body, gl, src, s_fwd, sp - 2 * LD, su, sw - 2 * LD, it, v);
  }
  fence_async_shared();
  __syncthreads();
  if (threadIdx.x == 0) {
    bulk_store(P + off + (size_t)(b.c0 - 1) * LD, sp, (uint32_t)(b.ncol * colb));
    bulk_commit_and_drain();
  }
}

// Forward velocity phase (fdcore.f90:97-159) of one band.
template <class R>
__global__ void __launch_bounds__(256, SWIT_BAND_BLOCKS)
    k_fwd_uw_b(Grid<R> g, BandList L, Receivers rec, const R* __restrict__ P, R* U, R* W, R* __restrict__ seis_t,
               R* __restrict__ strips, int it, int shot0, int* err) {
  extern __shared__ __align__(128) unsigned char band_sm[];
  __shared__ uint64_t bar;
  pdl_enter();
  const int LD = g.LD, bc = L.bc, s = shot0 + blockIdx.y;
  const Band b = band_of(g, bc);
  const size_t off = (size_t)s * g.FSZ, colb = (size_t)LD * sizeof(R);
  R* sp = reinterpret_cast<R*>(band_sm);
  R* su = sp + (size_t)(bc + 4) * LD;
  R* sw = su + (size_t)bc * LD;
  R* sb = sw + (size_t)bc * LD;
  R* sku = sb + (size_t)bc * LD;
  R* skw = sku + (size_t)bc * LD;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(&bar, (uint32_t)(((b.h1 - b.h0 + 1) + 5 * b.ncol) * colb));
    BAND_LOAD(sp, b.h0 - b.c0 + 2, P + off, b.h0, b.h1 - b.h0 + 1);
    BAND_LOAD(su, 0, U + off, b.c0, b.ncol);
    BAND_LOAD(sw, 0, W + off, b.c0, b.ncol);
    BAND_LOAD(sb, 0, g.B, b.c0, b.ncol);
    BAND_LOAD(sku, 0, g.ku, b.c0, b.ncol);
    BAND_LOAD(skw, 0, g.kw, b.c0, b.ncol);
  }
  const int4 cnt = L.cnt[blockIdx.x];
  if (!band_ready(&bar, err, L.wait)) return;
  Grid<R> gl = g;
  gl.B = sb - 2 * LD;
  gl.ku = sku - 2 * LD;
  gl.kw = skw - 2 * LD;
  for (int i = threadIdx.x; i < cnt.z; i += blockDim.x) {
    VecIdx v;
    int t;
    band_task(gl, L, b, s, i, cnt, v, t);
    SWIT_TIER_CALL(fwd_uw_body, gl, rec, sp, su - 2 * LD, sw - 2 * LD, seis_t, strips, it, v);
  }
  fence_async_shared();
  __syncthreads();
  if (threadIdx.x == 0) {
    bulk_store(U + off + (size_t)(b.c0 - 1) * LD, su, (uint32_t)(b.ncol * colb));
    bulk_store(W + off + (size_t)(b.c0 - 1) * LD, sw, (uint32_t)(b.ncol * colb));
    bulk_commit_and_drain();
  }
}


// Reverse velocity phase of one band: adjoint u, w (fdcore.f90:309-333) and
// reconstruction u, w with their re-insert (fdcore.f90:220-247).
template <class R>
__global__ void __launch_bounds__(256, SWIT_BAND_BLOCKS)
    k_bwd_uw_b(Grid<R> g, BandList L, const R* __restrict__ PB, R* UB, R* WB, const R* __restrict__ PE, R* UE, R* WE,
               const R* __restrict__ strips, int it, int shot0, int* err) {
  extern __shared__ __align__(128) unsigned char band_sm[];
  __shared__ uint64_t bar;
  pdl_enter();
  const int LD = g.LD, bc = L.bc, s = shot0 + blockIdx.y;
  const Band b = band_of(g, bc);
  const size_t off = (size_t)s * g.FSZ, colb = (size_t)LD * sizeof(R), H = (size_t)(bc + 4) * LD,
               O = (size_t)bc * LD;
  R* spb = reinterpret_cast<R*>(band_sm);
  R* spe = spb + H;
  R* sub = spe + H;
  R* swb = sub + O;
  R* sue = swb + O;
  R* swe = sue + O;
  R* sa = swe + O;
  R* sb = sa + O;
  R* sku = sb + O;
  R* skw = sku + O;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nh = b.h1 - b.h0 + 1, lh = b.h0 - b.c0 + 2;
    mbar_expect_tx(&bar, (uint32_t)((2 * nh + 8 * b.ncol) * colb));
    BAND_LOAD(spb, lh, PB + off, b.h0, nh);
    BAND_LOAD(spe, lh, PE + off, b.h0, nh);
    BAND_LOAD(sub, 0, UB + off, b.c0, b.ncol);
    BAND_LOAD(swb, 0, WB + off, b.c0, b.ncol);
    BAND_LOAD(sue, 0, UE + off, b.c0, b.ncol);
    BAND_LOAD(swe, 0, WE + off, b.c0, b.ncol);
    BAND_LOAD(sa, 0, g.A, b.c0, b.ncol);
    BAND_LOAD(sb, 0, g.B, b.c0, b.ncol);
    BAND_LOAD(sku, 0, g.ku, b.c0, b.ncol);
    BAND_LOAD(skw, 0, g.kw, b.c0, b.ncol);
  }
  const int4 cnt = L.cnt[blockIdx.x];
  if (!band_ready(&bar, err, L.wait)) return;
  Grid<R> gl = g;
  gl.A = sa - 2 * LD;
  gl.B = sb - 2 * LD;
  gl.ku = sku - 2 * LD;
  gl.kw = skw - 2 * LD;
  for (int i = threadIdx.x; i < cnt.z; i += blockDim.x) {
    VecIdx v;
    int t;
    band_task(gl, L, b, s, i, cnt, v, t);
    SWIT_TIER_CALL(bwd_uw_body, gl, spb, sub - 2 * LD, swb - 2 * LD, spe, sue - 2 * LD, swe - 2 * LD, strips, it, v);
  }
  fence_async_shared();
  __syncthreads();
  if (threadIdx.x == 0) {
    const size_t go = off + (size_t)(b.c0 - 1) * LD;
    const uint32_t nb = (uint32_t)(b.ncol * colb);
    bulk_store(UB + go, sub, nb);
    bulk_store(WB + go, swb, nb);
    bulk_store(UE + go, sue, nb);
    bulk_store(WE + go, swe, nb);
    bulk_commit_and_drain();
  }
}

// Reverse pressure phase of one band: adjoint p with injection and mirror
// (fdcore.f90:336-373), reconstruction p with source subtraction and re-insert
// (fdcore.f90:249-287), imaging sums (solver.f90:237-239).
template <class R>
__global__ void __launch_bounds__(256, SWIT_BAND_BLOCKS)
    k_bwd_p_b(Grid<R> g, BandList L, Receivers rec, Sources src, const R* __restrict__ s_fwd,
              const R* __restrict__ adj_t, R* PB, const R* __restrict__ UB, const R* __restrict__ WB, R* PE,
              const R* __restrict__ UE, const R* __restrict__ WE, R* DG, R* DFW, R* DBK, const R* __restrict__ strips,
              int it, int shot0, int* err) {
  extern __shared__ __align__(128) unsigned char band_sm[];
  __shared__ uint64_t bar;
  pdl_enter();
  const int LD = g.LD, bc = L.bc, s = shot0 + blockIdx.y;
  const Band b = band_of(g, bc);
  const size_t off = (size_t)s * g.FSZ, colb = (size_t)LD * sizeof(R), H = (size_t)(bc + 4) * LD,
               O = (size_t)bc * LD;
  R* sub = reinterpret_cast<R*>(band_sm);
  R* sue = sub + H;
  R* spb = sue + H;
  R* swb = spb + O;
  R* spe = swb + O;
  R* swe = spe + O;
  R* sa = swe + O;
  R* sb = sa + O;
  R* sk = sb + O;
  R* sg = sk + O;
  R* sf = sg + O;
  R* sd = sf + O;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nh = b.h1 - b.h0 + 1, lh = b.h0 - b.c0 + 2;
    mbar_expect_tx(&bar, (uint32_t)((2 * nh + 10 * b.ncol) * colb));
    BAND_LOAD(sub, lh, UB + off, b.h0, nh);
    BAND_LOAD(sue, lh, UE + off, b.h0, nh);
    BAND_LOAD(spb, 0, PB + off, b.c0, b.ncol);
    BAND_LOAD(swb, 0, WB + off, b.c0, b.ncol);
    BAND_LOAD(spe, 0, PE + off, b.c0, b.ncol);
    BAND_LOAD(swe, 0, WE + off, b.c0, b.ncol);
    BAND_LOAD(sa, 0, g.A, b.c0, b.ncol);
    BAND_LOAD(sb, 0, g.B, b.c0, b.ncol);
    BAND_LOAD(sk, 0, g.kp, b.c0, b.ncol);
    BAND_LOAD(sg, 0, DG + off, b.c0, b.ncol);
    BAND_LOAD(sf, 0, DFW + off, b.c0, b.ncol);
    BAND_LOAD(sd, 0, DBK + off, b.c0, b.ncol);
  }
  const int4 cnt = L.cnt[blockIdx.x];
  if (!band_ready(&bar, err, L.wait)) return;
  Grid<R> gl = g;
  gl.A = sa - 2 * LD;
  gl.B = sb - 2 * LD;
  gl.kp = sk - 2 * LD;
  for (int i = threadIdx.x; i < cnt.z; i += blockDim.x) {
    VecIdx v;
    int t;
    band_task(gl, L, b, s, i, cnt, v, t);
    SWIT_TIER_CALL(bwd_p_body, gl, rec, src, s_fwd, adj_t, spb - 2 * LD, sub, swb - 2 * LD, spe - 2 * LD, sue,
                   swe - 2 * LD, sg - 2 * LD, sf - 2 * LD, sd - 2 * LD, strips, it, v);
  }
  fence_async_shared();
  __syncthreads();
  if (threadIdx.x == 0) {
    const size_t go = off + (size_t)(b.c0 - 1) * LD;
    const uint32_t nb = (uint32_t)(b.ncol * colb);
    bulk_store(PB + go, spb, nb);
    bulk_store(PE + go, spe, nb);
    bulk_store(DG + go, sg, nb);
    bulk_store(DFW + go, sf, nb);
    bulk_store(DBK + go, sd, nb);
    bulk_commit_and_drain();
  }
}

}  // namespace swit
