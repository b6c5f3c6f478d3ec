// kernels_multi.cuh -- the four phase kernels over many independent problems
// (instances) of different grids, shot counts and record lengths in one launch.
//
// Each instance is a regular engine (its own arrays); a device table holds per
// instance the grid description, receiver and source tables and array
// pointers.  Per phase kernel, every instance's own task list (kernels_vec.cuh)
// is padded to whole blocks of kMultiBlock entries and the blocks of a wave's
// (instance, shot) pairs are listed in the wave's block table, instances ordered
// by record length nt, longest first.  Within a wave all forward loops start
// together and all reverse loops start together, so at a given step the blocks
// of the pairs still running are a prefix of the table and a launch covers
// exactly that prefix.  A block
// belongs to one instance and one shot: it stages the instance's description in
// shared memory once, and skips its work when the instance is switched off for
// this call.  The vector bodies are those of the single-instance kernels, so
// every instance computes the bits its own engine would.
#pragma once
#include "kernels_vec.cuh"

namespace swit {

template <class R>
struct Inst {
  Grid<R> g;
  Receivers rec;
  Sources src;
  int ns;
  const R* s_fwd;
  R *p, *u, *w, *seis_t, *strips;
  R *pb, *ub, *wb, *pe, *ue, *we, *dg, *dfw, *dbk;
  const R* adj_t;
};

constexpr uint32_t kMultiPad = 0xffffffffu;  // padding entry of a block
// Threads (list entries) per block of the multi-instance kernels. 128-entry blocks
// (as the single-instance vec kernels use) measured no faster on uneven batches.
#ifndef SWIT_MULTI_BLOCK
#define SWIT_MULTI_BLOCK 256
#endif
constexpr int kMultiBlock = SWIT_MULTI_BLOCK;

// Block table entry: x = instance << 16 | shot, y = first list entry of the block.
// List entries: tier << 30 | (ix - 1) << 16 | q, or kMultiPad.
struct MultiLaunch {
  const uint2* __restrict__ blocks;
  const uint32_t* __restrict__ list;
  const int* __restrict__ on;  // per instance: 0 = skip in this call
  int nblocks;                 // active prefix
};

// Stages this block's instance description in shared memory; returns it, or
// null when the block is past the active prefix or its instance is off (uniform
// over the block).  *e = this thread's list entry.
template <class R>
__device__ __forceinline__ const Inst<R>* multi_block(const Inst<R>* __restrict__ tab, const MultiLaunch& L,
                                                      Inst<R>* sI, uint32_t* e, int* s) {
  if ((int)blockIdx.x >= L.nblocks) return nullptr;
  const uint2 b = L.blocks[blockIdx.x];
  const int r = (int)(b.x >> 16);
  if (!L.on[r]) return nullptr;
  *s = (int)(b.x & 0xffffu);
  *e = L.list[b.y + threadIdx.x];
  const int* src = reinterpret_cast<const int*>(tab + r);
  int* dst = reinterpret_cast<int*>(sI);
  for (int k = threadIdx.x; k < (int)(sizeof(Inst<R>) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
  __syncthreads();
  return sI;
}

__device__ __forceinline__ void multi_vec(const int LD, uint32_t e, int s, VecIdx& v, int& t) {
  t = (int)(e >> 30);
  v.s = s;
  v.ix = (int)((e >> 16) & 0x3fffu) + 1;
  v.q = (int)(e & 0xffffu);
  v.iz0 = 4 * v.q + 1;
  v.ok = true;
  v.k4 = (size_t)(v.ix - 1) * (LD >> 2) + v.q;
  v.kc = v.k4;
  v.kg = v.k4;
}

// The instance description is a block-uniform early exit, so __syncthreads in
// multi_block is reached by all threads or none.
#define SWIT_MULTI_PROLOGUE                                          \
  __shared__ __align__(16) unsigned char inst_sm[sizeof(Inst<R>)];   \
  uint32_t e = kMultiPad;                                            \
  int s = 0;                                                         \
  const Inst<R>* I = multi_block(tab, L, reinterpret_cast<Inst<R>*>(inst_sm), &e, &s); \
  pdl_enter();                                                       \
  if (!I || e == kMultiPad) return;                                  \
  VecIdx v;                                                          \
  int t;                                                             \
  multi_vec(I->g.LD, e, s, v, t);                                    \
  const size_t off = (size_t)s * I->g.FSZ;

// Forward phases at step it (the same step for every running instance).
template <class R>
__global__ void __launch_bounds__(kMultiBlock) k_fwd_p_m(const Inst<R>* __restrict__ tab, MultiLaunch L, int it) {
  SWIT_MULTI_PROLOGUE
  SWIT_TIER_CALL(fwd_p_body, I->g, I->src, I->s_fwd, I->p + off, I->u + off, I->w + off, it, v);
}

template <class R>
__global__ void __launch_bounds__(kMultiBlock) k_fwd_uw_m(const Inst<R>* __restrict__ tab, MultiLaunch L, int it, int store) {
  SWIT_MULTI_PROLOGUE
  SWIT_TIER_CALL(fwd_uw_body, I->g, I->rec, I->p + off, I->u + off, I->w + off, I->seis_t, store ? I->strips : nullptr,
                 it, v);
}

// Reverse phases at reverse index jr: instance step it = nt - jr.
template <class R>
__global__ void __launch_bounds__(kMultiBlock) k_bwd_uw_m(const Inst<R>* __restrict__ tab, MultiLaunch L, int jr) {
  SWIT_MULTI_PROLOGUE
  SWIT_TIER_CALL(bwd_uw_body, I->g, I->pb + off, I->ub + off, I->wb + off, I->pe + off, I->ue + off, I->we + off,
                 I->strips, I->g.nt - jr, v);
}

template <class R>
__global__ void __launch_bounds__(kMultiBlock) k_bwd_p_m(const Inst<R>* __restrict__ tab, MultiLaunch L, int jr) {
  SWIT_MULTI_PROLOGUE
  SWIT_TIER_CALL(bwd_p_body, I->g, I->rec, I->src, I->s_fwd, I->adj_t, I->pb + off, I->ub + off, I->wb + off,
                 I->pe + off, I->ue + off, I->we + off, I->dg + off, I->dfw + off, I->dbk + off, I->strips,
                 I->g.nt - jr, v);
}

}  // namespace swit
