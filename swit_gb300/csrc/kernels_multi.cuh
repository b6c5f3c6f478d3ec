// kernels_multi.cuh -- the four phase kernels over many independent problems
// (instances) of different grids, shot counts and record lengths in one launch.
//
// Each instance is a regular engine (its own arrays); a device table holds per
// instance the grid description, receiver and source tables and array
// pointers.  One combined task list per phase kernel concatenates the
// instances' own task lists (kernels_vec.cuh), instances ordered by record
// length nt, longest first, each entry (instance << 40 | tier << 32 |
// (ix - 1) << 16 | q).  All forward loops start together and all reverse loops
// start together, so at a given step the instances still running are a prefix
// of the list and a launch covers exactly that prefix.  blockIdx.y is the
// shot; threads past an instance's shot count return at once.  The vector
// bodies are those of the single-instance kernels, so every instance computes
// the bits its own engine would.
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

// List entry i -> instance, vector index set and tier; null past the active
// prefix or past the instance's shots.
template <class R>
__device__ __forceinline__ const Inst<R>* multi_index(const Inst<R>* __restrict__ tab,
                                                       const uint64_t* __restrict__ list, int len, VecIdx& v, int& t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return nullptr;
  const uint64_t e = list[i];
  const Inst<R>* I = tab + (e >> 40);
  const int s = blockIdx.y;
  if (s >= I->ns) return nullptr;
  t = (int)((e >> 32) & 3u);
  v.s = s;
  v.ix = (int)((e >> 16) & 0xffffu) + 1;
  v.q = (int)(e & 0xffffu);
  v.iz0 = 4 * v.q + 1;
  v.ok = true;
  v.k4 = (size_t)(v.ix - 1) * (I->g.LD >> 2) + v.q;
  v.kc = v.k4;
  v.kg = v.k4;
  return I;
}

// Forward phases at step it (the same step for every running instance).
template <class R>
__global__ void __launch_bounds__(256) k_fwd_p_m(const Inst<R>* __restrict__ tab, const uint64_t* __restrict__ list,
                                                 int len, int it) {
  VecIdx v;
  int t;
  const Inst<R>* I = multi_index(tab, list, len, v, t);
  pdl_enter();
  if (!I) return;
  const size_t off = (size_t)v.s * I->g.FSZ;
  SWIT_TIER_CALL(fwd_p_body, I->g, I->src, I->s_fwd, I->p + off, I->u + off, I->w + off, it, v);
}

template <class R>
__global__ void __launch_bounds__(256) k_fwd_uw_m(const Inst<R>* __restrict__ tab, const uint64_t* __restrict__ list,
                                                  int len, int it, int store) {
  VecIdx v;
  int t;
  const Inst<R>* I = multi_index(tab, list, len, v, t);
  pdl_enter();
  if (!I) return;
  const size_t off = (size_t)v.s * I->g.FSZ;
  SWIT_TIER_CALL(fwd_uw_body, I->g, I->rec, I->p + off, I->u + off, I->w + off, I->seis_t, store ? I->strips : nullptr,
                 it, v);
}

// Reverse phases at reverse index jr: instance step it = nt - jr.
template <class R>
__global__ void __launch_bounds__(256) k_bwd_uw_m(const Inst<R>* __restrict__ tab, const uint64_t* __restrict__ list,
                                                  int len, int jr) {
  VecIdx v;
  int t;
  const Inst<R>* I = multi_index(tab, list, len, v, t);
  pdl_enter();
  if (!I) return;
  const size_t off = (size_t)v.s * I->g.FSZ;
  SWIT_TIER_CALL(bwd_uw_body, I->g, I->pb + off, I->ub + off, I->wb + off, I->pe + off, I->ue + off, I->we + off,
                 I->strips, I->g.nt - jr, v);
}

template <class R>
__global__ void __launch_bounds__(256) k_bwd_p_m(const Inst<R>* __restrict__ tab, const uint64_t* __restrict__ list,
                                                 int len, int jr) {
  VecIdx v;
  int t;
  const Inst<R>* I = multi_index(tab, list, len, v, t);
  pdl_enter();
  if (!I) return;
  const size_t off = (size_t)v.s * I->g.FSZ;
  SWIT_TIER_CALL(bwd_p_body, I->g, I->rec, I->src, I->s_fwd, I->adj_t, I->pb + off, I->ub + off, I->wb + off,
                 I->pe + off, I->ue + off, I->we + off, I->dg + off, I->dfw + off, I->dbk + off, I->strips,
                 I->g.nt - jr, v);
}

}  // namespace swit
