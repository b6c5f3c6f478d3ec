// engine.cu -- C ABI (include/swit_gb300.h) and device workspace of the GB300
// forward/adjoint engine.  Kernels are in kernels.cuh.
//
// Build: nvcc -gencode arch=compute_103a,code=sm_103a --fmad=false
//        -Xcompiler -ffp-contract=off (see swit_gb300/build.py).  --fmad=false and
// the host flag keep every floating-point operation in the reference's order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/swit_gb300.h"
#include "kernels.cuh"
#include "kernels_walk.cuh"
#include "kernels_vec.cuh"
#include "kernels_cluster.cuh"
#include "kernels_band.cuh"
#include "kernels_multi.cuh"
#include "kernels_exact.cuh"

using namespace swit;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t _e = (call);                                                                  \
    if (_e != cudaSuccess) return fail(SWIT_E_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, __LINE__); \
  } while (0)

inline int round_up(int a, int m) { return (a + m - 1) / m * m; }

}  // namespace

namespace swit {
// Lets other translation units of the library report through swit_last_error.
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace swit

constexpr int kCapStreamsMax = 4;  // concurrent branches of a captured graph, at most

struct swit_engine {
  // problem
  int nx, nz, L, nt, NX, NZ, LD, LDI, fs, fs_flag, ns, ngmax, SL, prec, path;
  float dx32, dt32;
  int batch, bx;
  int variant;  // 1 = split, 2 = walk (one kernel per step, ping-pong), 3 = vec (split, 4 rows per thread),
                // 4 = cluster (one persistent cluster per shot, wavefields in distributed shared memory),
                // 5 = hybrid (cluster forward, vec reverse loop), 6 = band (vec bodies on bands of
                // columns staged through shared memory by bulk copies)
  // cluster variant: cluster sizes, threads per CTA, A and B on chip, dynamic shared memory
  int clf = 0, clb = 0, maxt_f = 0, maxt_b = 0, ab_local = 0;
  int vbx = 32;  // columns per CTA of the vec kernels (block_x for variant 3)
  bool pdl = false;  // programmatic dependent launch between the vec step kernels (batched path)
  // task lists of the four vec kernels (fwd_p, fwd_uw, bwd_uw, bwd_p), kernels_vec.cuh
  uint32_t* d_list = nullptr;
  size_t list_stride = 0;
  int list_n0[4] = {0, 0, 0, 0}, list_n1[4] = {0, 0, 0, 0}, list_len[4] = {0, 0, 0, 0};
  // the device lists of the single-instance kernels: the full lists above minus
  // the tier-0 rectangle of each kernel, whose vectors the first rect_nb blocks
  // map arithmetically (VecList); the multi-instance engine uses the full lists
  int dl_n0[4] = {0, 0, 0, 0}, dl_n1[4] = {0, 0, 0, 0}, dl_len[4] = {0, 0, 0, 0};
  int rect_x0[4] = {0, 0, 0, 0}, rect_q0[4] = {0, 0, 0, 0}, rect_nq[4] = {1, 1, 1, 1}, rect_n[4] = {0, 0, 0, 0};
  uint32_t* d_dlist = nullptr;
  std::vector<uint32_t> h_list;  // host copy of the four lists (multi-instance engines combine them)
  // band variant: columns per band, bands, per-band task lists and counts of the four kernels
  int band_bc = 0, nbands = 0, band_stride = 0;
  unsigned band_wait = 0;  // mbarrier polls before a band block gives up (SWIT_BAND_WAIT_POLLS lowers it)
  uint32_t* d_blist = nullptr;
  int4* d_bcnt = nullptr;
  size_t band_sm[4] = {0, 0, 0, 0};
  int* d_err = nullptr;  // device error word (kernels_band.cuh), read by swit_check
  // checkpointed recomputation: every ckpt_k steps, ckpt_m segments; strip buffer of snt steps per shot whose
  // slot 0 holds step sit0; ckpt = ckpt_m slots x {p, u, w} x ns x FSZ (slot m: state after segment m)
  int ckpt_k = 0, ckpt_m = 0, snt = 0, sit0 = 1;
  void* ckpt = nullptr;
  size_t smf = 0, smb = 0;
  int IL;       // interior fields: row/column offset into their layout (npml for vec, else 0)
  int device;
  size_t esz;  // sizeof(R)
  std::vector<int> ng, isx, isz, risx, risz, colptr, ent_ig, ent_zr, zlo, zhi;
  // device tables
  int *d_ng = nullptr, *d_isx = nullptr, *d_isz = nullptr, *d_risx = nullptr, *d_risz = nullptr;
  int *d_colptr = nullptr, *d_ig = nullptr, *d_zr = nullptr, *d_live = nullptr, *d_zlo = nullptr, *d_zhi = nullptr;
  int4* d_rcol = nullptr;  // per shot and column: first receiver entry {ig, row, count, entry}
  double* d_mtrace = nullptr;
  // device arrays of type R (float or double)
  void *A = nullptr, *B = nullptr, *damp = nullptr, *cint = nullptr;
  void *kp = nullptr, *ku = nullptr, *kw = nullptr;  // damping factors per point (vec and cluster kernels)
  void *p = nullptr, *u = nullptr, *w = nullptr, *pb = nullptr, *ub = nullptr, *wb = nullptr;
  void *pe = nullptr, *ue = nullptr, *we = nullptr, *dg = nullptr, *dfw = nullptr, *dbk = nullptr;
  void *strips = nullptr, *src = nullptr, *seis_t = nullptr, *adj_t = nullptr;
  // second state set of the walk variant
  void *p2 = nullptr, *u2 = nullptr, *w2 = nullptr, *pb2 = nullptr, *ub2 = nullptr, *wb2 = nullptr;
  void *pe2 = nullptr, *ue2 = nullptr, *we2 = nullptr;
  float* d_in = nullptr;     // float staging: sources / obs / adjoint sources from the host
  void* d_stage = nullptr;   // output staging for host outputs
  size_t bytes = 0;
  bool model_set = false, fwd_ready = false;
  cudaStream_t cap = nullptr;
  // further capture streams: batches run round-robin over the branches of the graphs (capture_fork)
  cudaStream_t capx[kCapStreamsMax - 1] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[kCapStreamsMax - 1] = {};
  // host observed data of swit_gradient_l2: copied into d_in on `cpy` while the
  // forward loop runs (ev_in: the call's start on the caller's stream; ev_cpy: copy done)
  cudaStream_t cpy = nullptr;
  cudaEvent_t ev_in = nullptr, ev_cpy = nullptr;
  float* d_src_in = nullptr;  // source staging (ns x nt floats), apart from d_in
  int branches = 2;  // graph branches in use (swit_desc.graph_branches)
  // captured loops, each a sequence of graphs of at most kGraphNodes nodes (capture_chunked)
  std::vector<cudaGraphExec_t> gfwd[2];
  std::vector<cudaGraphExec_t> gbwd;
  int launches_fwd = 0, launches_bwd = 0;
  // exact discrete adjoint (adjoint_mode 1, kernels_exact.cuh): the strip buffer holds the forward's D of
  // every step (SL = NX * LD); mirror rows, source gradient, dA/dc; graph of its reverse loop
  int exact = 0;
  int rcomp = 0;  // recorded component: 0 = p, 1 = vx, 2 = vz (swit_desc.receiver_component)
  void *xm = nullptr, *xsrc = nullptr, *xdadc = nullptr;
  std::vector<cudaGraphExec_t> gxb;
  size_t graph_nodes = 0;  // node bound per captured graph (kGraphNodes; SWIT_GRAPH_NODES overrides)
};

namespace {

template <class T>
int dalloc(swit_engine* e, T** ptr, size_t n) {
  if (n == 0) n = 1;
  cudaError_t rc = cudaMalloc((void**)ptr, n * sizeof(T));
  if (rc != cudaSuccess) {
    *ptr = nullptr;
    return fail(SWIT_E_NOMEM, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(rc));
  }
  e->bytes += n * sizeof(T);
  return 0;
}

int valloc(swit_engine* e, void** ptr, size_t n) {
  if (n == 0) n = 1;
  cudaError_t rc = cudaMalloc(ptr, n * e->esz);
  if (rc != cudaSuccess) {
    *ptr = nullptr;
    return fail(SWIT_E_NOMEM, "cudaMalloc of %zu bytes failed: %s", n * e->esz, cudaGetErrorString(rc));
  }
  e->bytes += n * e->esz;
  return 0;
}

void release(swit_engine* e) {
  for (auto* v : {&e->gfwd[0], &e->gfwd[1], &e->gbwd, &e->gxb}) {
    for (cudaGraphExec_t x : *v) cudaGraphExecDestroy(x);
    v->clear();
  }
  if (e->cap) cudaStreamDestroy(e->cap);
  for (int i = 0; i < kCapStreamsMax - 1; ++i) {
    if (e->capx[i]) cudaStreamDestroy(e->capx[i]);
    if (e->ev_join[i]) cudaEventDestroy(e->ev_join[i]);
  }
  if (e->ev_fork) cudaEventDestroy(e->ev_fork);
  if (e->cpy) cudaStreamDestroy(e->cpy);
  if (e->ev_in) cudaEventDestroy(e->ev_in);
  if (e->ev_cpy) cudaEventDestroy(e->ev_cpy);
  void* ptrs[] = {e->d_rcol, e->d_zlo, e->d_zhi, e->d_ng, e->d_isx, e->d_isz, e->d_risx, e->d_risz, e->d_colptr, e->d_ig, e->d_zr, e->d_live,
                  e->d_mtrace, e->A, e->B, e->damp, e->cint, e->kp, e->ku, e->kw, e->p, e->u, e->w, e->pb, e->ub, e->wb, e->pe,
                  e->ue, e->we, e->dg, e->dfw, e->dbk, e->strips, e->src, e->seis_t, e->adj_t, e->d_in, e->d_src_in,
                  e->d_stage, e->p2, e->u2, e->w2, e->pb2, e->ub2, e->wb2, e->pe2, e->ue2, e->we2, e->d_list, e->d_dlist, e->d_blist, e->d_bcnt, e->d_err, e->ckpt,
                  e->xm, e->xsrc, e->xdadc};
  for (void* q : ptrs)
    if (q) cudaFree(q);
}

template <class R>
Grid<R> make_grid(const swit_engine* e) {
  Grid<R> g;
  g.nx = e->nx;
  g.nz = e->nz;
  g.L = e->L;
  g.NX = e->NX;
  g.NZ = e->NZ;
  g.LD = e->LD;
  g.LDI = e->LDI;
  g.fs = e->fs;
  g.fs_flag = e->fs_flag;
  g.nt = e->nt;
  g.ngmax = e->ngmax;
  g.SL = e->SL;
  g.snt = e->snt;
  g.sit0 = e->sit0;
  g.FSZ = (size_t)e->NX * e->LD;
  g.FSI = e->variant >= 2 ? g.FSZ : (size_t)e->nx * e->LDI;
  g.IL = e->IL;
  if (e->variant >= 2) g.LDI = e->LD;
  g.dt = (R)e->dt32;
  g.c1 = R(9.0) / R(8.0);    // global.f90:34
  g.c2 = R(-1.0) / R(24.0);  // global.f90:35
  g.A = (const R*)e->A;
  g.B = (const R*)e->B;
  g.damp = (const R*)e->damp;
  g.kp = (const R*)e->kp;
  g.ku = (const R*)e->ku;
  g.kw = (const R*)e->kw;
  return g;
}

inline Receivers make_rec(const swit_engine* e) {
  return Receivers{e->d_colptr, e->d_ig, e->d_zr, e->d_zlo, e->d_zhi, e->rcomp, e->d_rcol};
}
inline Sources make_src(const swit_engine* e) { return Sources{e->d_isx, e->d_isz, e->d_risx, e->d_risz}; }

// Launch shape of the stencil kernels for a batch of nb shots.
inline void stencil_shape(const swit_engine* e, int nb, dim3& grid, dim3& block) {
  block = dim3(32, e->bx, 1);
  grid = dim3((e->NZ + 31) / 32, (e->NX + e->bx - 1) / e->bx, nb);
}

// Launch with programmatic stream serialization when pdl is set: the next
// kernel's blocks may be scheduled during this one's tail and wait on chip
// (griddepcontrol.wait in pdl_enter) until it has completed.
template <class... P, class... A>
void launch_pdl_sm(bool pdl, void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...);
}
template <class... P, class... A>
void launch_pdl(bool pdl, void (*k)(P...), dim3 grid, dim3 block, cudaStream_t st, A&&... args) {
  launch_pdl_sm(pdl, k, grid, block, 0, st, std::forward<A>(args)...);
}

// Band variant: one block per band of e->band_bc columns and shot.
inline BandList band_list(const swit_engine* e, int k) {
  return BandList{e->d_blist + (size_t)k * e->nbands * e->band_stride, e->d_bcnt + (size_t)k * e->nbands,
                  e->band_stride, e->band_bc, e->band_wait};
}

// Vec kernels: SWIT_VEC_BLOCK threads per block over the kernel's task list k (the tier-0
// rectangle first, mapped arithmetically, then the device list), nb shots.
inline VecList vec_list(const swit_engine* e, int k) {
  return VecList{e->d_dlist + (size_t)k * e->list_stride, e->dl_n0[k], e->dl_n1[k], e->dl_len[k], e->rect_x0[k],
                 e->rect_q0[k], e->rect_nq[k], e->rect_n[k], (e->rect_n[k] + SWIT_VEC_BLOCK - 1) / SWIT_VEC_BLOCK};
}
inline dim3 vec_block(const swit_engine*) { return dim3(SWIT_VEC_BLOCK); }
inline dim3 vec_grid(const swit_engine* e, int k, int nb) {
  constexpr int B = SWIT_VEC_BLOCK;
  return dim3((unsigned)std::max(1, (e->rect_n[k] + B - 1) / B + (e->dl_len[k] + B - 1) / B), nb);
}

// Cluster variant: one launch runs the whole time loop of nb shots, one
// cluster of e->clf (forward) or e->clb (reverse) CTAs per shot.
inline cudaLaunchConfig_t cluster_config(int C, int nb, int threads, size_t smem, cudaStream_t st,
                                         cudaLaunchAttribute* at) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C, nb, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cfg;
}

template <class R, int MAXT>
void launch_cluster_fwd_t(swit_engine* e, bool store, int shot0, int nb, cudaStream_t st) {
  cudaLaunchAttribute at[1];
  const cudaLaunchConfig_t cfg = cluster_config(e->clf, nb, e->maxt_f, e->smf, st, at);
  R* strips = store ? (R*)e->strips : nullptr;
  cudaLaunchKernelEx(&cfg, k_fwd_cl<R, MAXT>, make_grid<R>(e), make_src(e), make_rec(e), (const R*)e->src, (R*)e->p,
                     (R*)e->u, (R*)e->w, (R*)e->seis_t, strips, shot0, e->ab_local);
}

template <class R, int MAXT>
void launch_cluster_bwd_t(swit_engine* e, int shot0, int nb, cudaStream_t st) {
  cudaLaunchAttribute at[1];
  const cudaLaunchConfig_t cfg = cluster_config(e->clb, nb, e->maxt_b, e->smb, st, at);
  cudaLaunchKernelEx(&cfg, k_bwd_cl<R, MAXT>, make_grid<R>(e), make_rec(e), make_src(e), (const R*)e->src,
                     (const R*)e->adj_t, (const R*)e->pe, (const R*)e->ue, (const R*)e->we, (R*)e->dg, (R*)e->dfw,
                     (R*)e->dbk, (const R*)e->strips, shot0);
}

// Walk variant (kernels_walk.cuh): one launch per step and batch; a CTA is
// kWalkWarps of the ceil(LD/4/28) warps of one tile of e->bx columns of one
// shot (grid: tiles x shots x warp groups).  State is
// double-buffered: forward step it reads set A (p, u, w) when it is even and
// set B (p2, u2, w2) when it is odd; reverse step it reads set A when nt - it
// is even.
inline dim3 walk_block(const swit_engine*) { return dim3(32, kWalkWarps); }
inline dim3 walk_grid(const swit_engine* e, int nb) {
  const int nw = (e->LD / 4 + kWalkOwn - 1) / kWalkOwn;  // warps per column
  return dim3((e->NX + e->bx - 1) / e->bx, nb, (nw + kWalkWarps - 1) / kWalkWarps);
}

template <class R>
void launch_fwd_walk(swit_engine* e, bool store, int shot0, int nb, int it, cudaStream_t st) {
  Grid<R> g = make_grid<R>(e);
  const bool a = (it - 2) % 2 == 0;
  launch_pdl(e->pdl, k_fwd_walk<R>, walk_grid(e, nb), walk_block(e), st, g, make_src(e), make_rec(e),
             (const R*)e->src, (const R*)(a ? e->p : e->p2), (const R*)(a ? e->u : e->u2),
             (const R*)(a ? e->w : e->w2), (R*)(a ? e->p2 : e->p), (R*)(a ? e->u2 : e->u), (R*)(a ? e->w2 : e->w),
             (R*)e->seis_t, store ? (R*)e->strips : (R*)nullptr, it, shot0, e->bx);
}

template <class R>
void launch_bwd_walk(swit_engine* e, int shot0, int nb, int it, cudaStream_t st) {
  Grid<R> g = make_grid<R>(e);
  const bool a = (e->nt - it) % 2 == 0;
  launch_pdl(e->pdl, k_bwd_walk<R>, walk_grid(e, nb), walk_block(e), st, g, make_src(e), make_rec(e),
             (const R*)e->src, (const R*)e->adj_t, (const R*)(a ? e->pb : e->pb2), (const R*)(a ? e->ub : e->ub2),
             (const R*)(a ? e->wb : e->wb2), (R*)(a ? e->pb2 : e->pb), (R*)(a ? e->ub2 : e->ub),
             (R*)(a ? e->wb2 : e->wb), (const R*)(a ? e->pe : e->pe2), (const R*)(a ? e->ue : e->ue2),
             (const R*)(a ? e->we : e->we2), (R*)(a ? e->pe2 : e->pe), (R*)(a ? e->ue2 : e->ue),
             (R*)(a ? e->we2 : e->we), (R*)e->dg, (R*)e->dfw, (R*)e->dbk, (const R*)e->strips, it, shot0, e->bx);
}

// Forward time loop of shots [shot0, shot0+nb): fdcore.f90:75-160.
template <class R>
void launch_forward_steps(swit_engine* e, bool store, int shot0, int nb, cudaStream_t st, int it_lo = 2,
                          int it_hi = -1) {
  if (it_hi < 0) it_hi = e->nt;
  if (e->variant == 4 || e->variant == 5) {
    if (e->maxt_f == 512)
      launch_cluster_fwd_t<R, 512>(e, store, shot0, nb, st);
    else
      launch_cluster_fwd_t<R, 1024>(e, store, shot0, nb, st);
    return;
  }
  if (e->variant == 6) {
    Grid<R> g = make_grid<R>(e);
    R* strips = store ? (R*)e->strips : nullptr;
    const dim3 grid(e->nbands, nb), block(256);
    const BandList l0 = band_list(e, 0), l1 = band_list(e, 1);
    for (int it = it_lo; it <= it_hi; ++it) {
      launch_pdl_sm(e->pdl, k_fwd_p_b<R>, grid, block, e->band_sm[0], st, g, l0, make_src(e), (const R*)e->src,
                    (R*)e->p, (const R*)e->u, (const R*)e->w, it, shot0, e->d_err);
      launch_pdl_sm(e->pdl, k_fwd_uw_b<R>, grid, block, e->band_sm[1], st, g, l1, make_rec(e), (const R*)e->p,
                    (R*)e->u, (R*)e->w, (R*)e->seis_t, strips, it, shot0, e->d_err);
    }
    return;
  }
  if (e->variant == 3) {
    Grid<R> g = make_grid<R>(e);
    // exact adjoint: the pressure phase stores D instead of the velocity phase storing strips
    R* strips = store && !e->exact ? (R*)e->strips : nullptr;
    const dim3 block = vec_block(e), g0 = vec_grid(e, 0, nb), g1 = vec_grid(e, 1, nb);
    const VecList l0 = vec_list(e, 0), l1 = vec_list(e, 1);
    for (int it = it_lo; it <= it_hi; ++it) {
      if (store && e->exact)
        launch_pdl(e->pdl, k_fwd_p_vx<R>, g0, block, st, g, l0, make_src(e), (const R*)e->src, (R*)e->p,
                   (const R*)e->u, (const R*)e->w, it, shot0, (R*)e->strips);
      else
        launch_pdl(e->pdl, k_fwd_p_v<R>, g0, block, st, g, l0, make_src(e), (const R*)e->src, (R*)e->p,
                   (const R*)e->u, (const R*)e->w, it, shot0);
      launch_pdl(e->pdl, k_fwd_uw_v<R>, g1, block, st, g, l1, make_rec(e), (const R*)e->p, (R*)e->u, (R*)e->w,
                 (R*)e->seis_t, strips, it, shot0);
    }
    return;
  }
  if (e->variant == 2) {
    for (int it = it_lo; it <= it_hi; ++it) launch_fwd_walk<R>(e, store, shot0, nb, it, st);
    return;
  }
  Grid<R> g = make_grid<R>(e);
  dim3 grid, block;
  stencil_shape(e, nb, grid, block);
  R* strips = store ? (R*)e->strips : nullptr;
  for (int it = it_lo; it <= it_hi; ++it) {
    k_fwd_p<R><<<grid, block, 0, st>>>(g, make_src(e), (const R*)e->src, (R*)e->p, (const R*)e->u, (const R*)e->w, it,
                                       shot0);
    k_fwd_uw<R><<<grid, block, 0, st>>>(g, make_rec(e), (const R*)e->p, (R*)e->u, (R*)e->w, (R*)e->seis_t, strips, it,
                                        shot0);
  }
}

// Reverse time loop of shots [shot0, shot0+nb): solver.f90:230-253.
template <class R>
void launch_backward_steps(swit_engine* e, int shot0, int nb, cudaStream_t st, int it_hi = -1, int it_lo = 2) {
  if (it_hi < 0) it_hi = e->nt;
  if (e->variant == 4) {
    if (e->maxt_b == 512)
      launch_cluster_bwd_t<R, 512>(e, shot0, nb, st);
    else
      launch_cluster_bwd_t<R, 1024>(e, shot0, nb, st);
    return;
  }
  if (e->variant == 6) {
    Grid<R> g = make_grid<R>(e);
    const dim3 grid(e->nbands, nb), block(256);
    const BandList l2 = band_list(e, 2), l3 = band_list(e, 3);
    for (int it = it_hi; it >= it_lo; --it) {
      launch_pdl_sm(e->pdl, k_bwd_uw_b<R>, grid, block, e->band_sm[2], st, g, l2, (const R*)e->pb, (R*)e->ub,
                    (R*)e->wb, (const R*)e->pe, (R*)e->ue, (R*)e->we, (const R*)e->strips, it, shot0, e->d_err);
      launch_pdl_sm(e->pdl, k_bwd_p_b<R>, grid, block, e->band_sm[3], st, g, l3, make_rec(e), make_src(e),
                    (const R*)e->src, (const R*)e->adj_t, (R*)e->pb, (const R*)e->ub, (const R*)e->wb, (R*)e->pe,
                    (const R*)e->ue, (const R*)e->we, (R*)e->dg, (R*)e->dfw, (R*)e->dbk, (const R*)e->strips, it,
                    shot0, e->d_err);
    }
    return;
  }
  if (e->variant == 3 || e->variant == 5) {
    Grid<R> g = make_grid<R>(e);
    const dim3 block = vec_block(e), g2 = vec_grid(e, 2, nb), g3 = vec_grid(e, 3, nb);
    const VecList l2 = vec_list(e, 2), l3 = vec_list(e, 3);
    for (int it = it_hi; it >= it_lo; --it) {
      launch_pdl(e->pdl, k_bwd_uw_v<R>, g2, block, st, g, l2, (const R*)e->pb, (R*)e->ub, (R*)e->wb,
                 (const R*)e->pe, (R*)e->ue, (R*)e->we, (const R*)e->strips, it, shot0);
      launch_pdl(e->pdl, k_bwd_p_v<R>, g3, block, st, g, l3, make_rec(e), make_src(e), (const R*)e->src,
                 (const R*)e->adj_t, (R*)e->pb, (const R*)e->ub, (const R*)e->wb, (R*)e->pe, (const R*)e->ue,
                 (const R*)e->we, (R*)e->dg, (R*)e->dfw, (R*)e->dbk, (const R*)e->strips, it, shot0);
      if (e->rcomp)  // vx / vz receivers: adjoint source into u / w
        launch_pdl(e->pdl, k_inject_vel<R>, dim3((e->NX + 255) / 256, nb), dim3(256), st, g, make_rec(e),
                   (const R*)e->adj_t, (R*)e->ub, (R*)e->wb, it, shot0);
    }
    return;
  }
  if (e->variant == 2) {
    for (int it = it_hi; it >= it_lo; --it) launch_bwd_walk<R>(e, shot0, nb, it, st);
    return;
  }
  Grid<R> g = make_grid<R>(e);
  dim3 grid, block;
  stencil_shape(e, nb, grid, block);
  for (int it = it_hi; it >= it_lo; --it) {
    k_bwd_uw<R><<<grid, block, 0, st>>>(g, (const R*)e->pb, (R*)e->ub, (R*)e->wb, (const R*)e->pe, (R*)e->ue,
                                        (R*)e->we, (const R*)e->strips, it, shot0);
    k_bwd_p<R><<<grid, block, 0, st>>>(g, make_rec(e), make_src(e), (const R*)e->src, (const R*)e->adj_t, (R*)e->pb,
                                       (const R*)e->ub, (const R*)e->wb, (R*)e->pe, (const R*)e->ue,
                                       (const R*)e->we, (R*)e->dg, (R*)e->dfw, (R*)e->dbk, (const R*)e->strips, it,
                                       shot0);
  }
}

// Shots per forward launch: the hybrid variant runs every shot in one cluster
// launch (the hardware schedules the clusters); the others use the batch.
inline int fwd_batch(const swit_engine* e) { return e->variant == 5 ? e->ns : e->batch; }

// Checkpointed recomputation.  Segment m (m = 0 .. ckpt_m-1, ckpt_m =
// ceil(nt/k)) is the forward steps [max(2, m k + 1), min(nt, (m+1) k)]; the
// reverse steps that read its strips are [m k + 2, min(nt, (m+1) k + 1)]
// (reverse step it reads the strips of step it-1; none for the last segment
// when m k + 2 > nt).  Checkpoint slot m holds (p, u, w) after segment m (the
// last slot is the final state); the state before segment 0 is zero.
// it_after: the forward step after which the state is saved or restored (the
// walk variant keeps the state after step it in set B when it is even).
inline void ckpt_copy(swit_engine* e, int slot, int s0, int nb, bool save, int it_after, cudaStream_t st) {
  const size_t fsz = (size_t)e->NX * e->LD * e->esz;
  const bool b = e->variant == 2 && it_after % 2 == 0;
  void* f[3] = {b ? e->p2 : e->p, b ? e->u2 : e->u, b ? e->w2 : e->w};
  for (int q = 0; q < 3; ++q) {
    char* c = (char*)e->ckpt + (((size_t)slot * 3 + q) * e->ns + s0) * fsz;
    char* a = (char*)f[q] + (size_t)s0 * fsz;
    cudaMemcpyAsync(save ? c : a, save ? a : c, (size_t)nb * fsz, cudaMemcpyDeviceToDevice, st);
  }
}

// Forward of shots [s0, s0+nb) keeping checkpoints instead of strips.
template <class R>
void forward_checkpointed(swit_engine* e, int s0, int nb, cudaStream_t st) {
  const int k = e->ckpt_k;
  for (int m = 0; m < e->ckpt_m; ++m) {
    launch_forward_steps<R>(e, false, s0, nb, st, std::max(2, m * k + 1), std::min(e->nt, (m + 1) * k));
    ckpt_copy(e, m, s0, nb, true, std::min(e->nt, (m + 1) * k), st);
  }
}

// Reverse loop of shots [s0, s0+nb): per segment, last first, restore the
// state before it, re-run its forward steps into the k-step strip buffer
// (the same kernels, so the same strips as a boundary-saving run), then run
// the reverse steps that read them.  Leaves sit0 = 1.
template <class R>
void backward_checkpointed(swit_engine* e, int s0, int nb, cudaStream_t st) {
  const int k = e->ckpt_k;
  const size_t fsz = (size_t)e->NX * e->LD * e->esz;
  for (int m = e->ckpt_m - 1; m >= 0; --m) {
    if (m * k + 2 > e->nt) continue;
    if (m > 0) {
      ckpt_copy(e, m - 1, s0, nb, false, m * k, st);
    } else {
      cudaMemsetAsync((char*)e->p + (size_t)s0 * fsz, 0, (size_t)nb * fsz, st);
      cudaMemsetAsync((char*)e->u + (size_t)s0 * fsz, 0, (size_t)nb * fsz, st);
      cudaMemsetAsync((char*)e->w + (size_t)s0 * fsz, 0, (size_t)nb * fsz, st);
      // the strips of step 1 (slot 0 of segment 0) are zero: no forward step 1 runs
      cudaMemsetAsync((char*)e->strips + (size_t)s0 * e->snt * e->SL * e->esz, 0,
                      (size_t)nb * e->snt * e->SL * e->esz, st);
    }
    e->sit0 = m * k + 1;
    launch_forward_steps<R>(e, true, s0, nb, st, std::max(2, m * k + 1), std::min(e->nt, (m + 1) * k));
    launch_backward_steps<R>(e, s0, nb, st, std::min(e->nt, (m + 1) * k + 1), m * k + 2);
  }
  e->sit0 = 1;
}

// Exact adjoint (kernels_exact.cuh): reverse steps it_hi .. it_lo of shots
// [shot0, shot0+nb), two launches per step over the forward kernels' task lists.
template <class R>
XAdj<R> make_xadj(swit_engine* e) {
  return XAdj<R>{(R*)e->pb, (R*)e->ub, (R*)e->wb, (R*)e->dg, (R*)e->xm, (R*)e->xsrc, (const R*)e->strips,
                 (const R*)e->adj_t};
}

template <class R>
void launch_exact_steps(swit_engine* e, int shot0, int nb, cudaStream_t st, int it_hi, int it_lo) {
  Grid<R> g = make_grid<R>(e);
  const XAdj<R> x = make_xadj<R>(e);
  const dim3 block = vec_block(e), g0 = vec_grid(e, 0, nb), g1 = vec_grid(e, 1, nb);
  const VecList l0 = vec_list(e, 0), l1 = vec_list(e, 1);
  for (int it = it_hi; it >= it_lo; --it) {
    if (e->rcomp)
      launch_pdl(e->pdl, k_xinject_vel<R>, dim3((e->NX + 255) / 256, nb), dim3(256), st, g, make_rec(e), x, it,
                 shot0);
    launch_pdl(e->pdl, k_xadj_p<R>, g0, block, st, g, l0, make_rec(e), make_src(e), x, it, shot0);
    launch_pdl(e->pdl, k_xadj_uw<R>, g1, block, st, g, l1, x, it, shot0);
  }
}

// Exact adjoint of shots [s0, s0+nb).  Boundary saving: the forward stored D of
// every step.  Checkpoints: per segment, last first, restore the state before
// it, re-run its forward steps storing D into the k-step buffer, then run the
// same steps in reverse.  Leaves sit0 = 1.
template <class R>
void exact_reverse(swit_engine* e, int s0, int nb, cudaStream_t st) {
  if (!e->ckpt_k) {
    launch_exact_steps<R>(e, s0, nb, st, e->nt, 2);
    return;
  }
  const int k = e->ckpt_k;
  const size_t fsz = (size_t)e->NX * e->LD * e->esz;
  for (int m = e->ckpt_m - 1; m >= 0; --m) {
    const int lo = std::max(2, m * k + 1), hi = std::min(e->nt, (m + 1) * k);
    if (lo > hi) continue;
    if (m > 0) {
      ckpt_copy(e, m - 1, s0, nb, false, m * k, st);
    } else {
      cudaMemsetAsync((char*)e->p + (size_t)s0 * fsz, 0, (size_t)nb * fsz, st);
      cudaMemsetAsync((char*)e->u + (size_t)s0 * fsz, 0, (size_t)nb * fsz, st);
      cudaMemsetAsync((char*)e->w + (size_t)s0 * fsz, 0, (size_t)nb * fsz, st);
    }
    e->sit0 = m * k + 1;
    launch_forward_steps<R>(e, true, s0, nb, st, lo, hi);
    launch_exact_steps<R>(e, s0, nb, st, hi, lo);
  }
  e->sit0 = 1;
}

// Inside a capture on e->cap: the other capture streams join (fork) and are
// joined back (join), so batches issued round-robin on the streams form
// concurrent branches of the graph; kernels of different branches fill each
// other's tails and launch gaps.  Batches share no array (each shot owns its
// wavefields, strips and sums), so the order between them does not matter.
// What counts is the state of the shots in flight against the L2 and equal work
// per branch (auto_batches): at 481x141, 127.6 shot-gradients/s with three
// branches of 9-shot batches, 126.0 with two of 13, 105.3 with 13-shot batches
// on three branches (one branch runs two batches) and 101.6 with one chain.
inline cudaStream_t capture_stream(swit_engine* e, int b, cudaStream_t origin) {
  const int k = b % e->branches;
  return k ? e->capx[k - 1] : origin;
}
inline void capture_fork(swit_engine* e, cudaStream_t origin) {
  cudaEventRecord(e->ev_fork, origin);
  for (int i = 0; i < e->branches - 1; ++i) cudaStreamWaitEvent(e->capx[i], e->ev_fork, 0);
}
inline void capture_join(swit_engine* e, cudaStream_t origin) {
  for (int i = 0; i < e->branches - 1; ++i) {
    cudaEventRecord(e->ev_join[i], e->capx[i]);
    cudaStreamWaitEvent(origin, e->ev_join[i], 0);
  }
}

// A captured loop is split into graphs of at most about kGraphNodes nodes,
// each a whole number of rounds of the branches.  Observed on GB300: a 200-shot,
// nt 6000 survey in one-shot batches captured as one graph of 2.4 M kernel
// nodes per loop returned a NaN gradient, and capturing a 4.8 M-node loop
// crashed the process, where graphs of up to 0.5 M nodes ran correctly.
constexpr size_t kGraphNodes = size_t(1) << 18;

// Upper bound of the nodes one batch adds to a captured loop.
inline size_t loop_nodes(const swit_engine* e) {
  return 2 * (size_t)(e->nt - 1) * (e->ckpt_k ? 2 : 1) + 8 * (size_t)e->ckpt_m + 8;
}

inline void destroy_graphs(std::vector<cudaGraphExec_t>& ex) {
  for (cudaGraphExec_t x : ex) cudaGraphExecDestroy(x);
  ex.clear();
}

inline int launch_graphs(const std::vector<cudaGraphExec_t>& ex, cudaStream_t st) {
  for (cudaGraphExec_t x : ex) CK(cudaGraphLaunch(x, st));
  return 0;
}

// Captures batches 0 .. nbatch-1 (issue(b, stream) launches batch b's work on
// the given capture stream) into ex: consecutive chunks of batches, each chunk
// one graph with the batches on concurrent branches.  ex is left empty on error.
template <class F>
int capture_chunked(swit_engine* e, std::vector<cudaGraphExec_t>& ex, int nbatch, size_t nodes_per_batch,
                    const char* what, F&& issue) {
  int chunk = (int)std::max<size_t>(1, e->graph_nodes / std::max<size_t>(1, nodes_per_batch));
  if (chunk >= e->branches) chunk -= chunk % e->branches;
  for (int b0 = 0; b0 < nbatch; b0 += chunk) {
    cudaError_t rc = cudaStreamBeginCapture(e->cap, cudaStreamCaptureModeThreadLocal);
    if (rc != cudaSuccess) {
      destroy_graphs(ex);
      return fail(SWIT_E_CUDA, "%s graph capture: %s", what, cudaGetErrorString(rc));
    }
    capture_fork(e, e->cap);
    for (int b = b0; b < std::min(nbatch, b0 + chunk); ++b) issue(b, capture_stream(e, b - b0, e->cap));
    capture_join(e, e->cap);
    cudaGraph_t graph = nullptr;
    rc = cudaStreamEndCapture(e->cap, &graph);
    if (rc != cudaSuccess) {
      destroy_graphs(ex);
      return fail(SWIT_E_CUDA, "%s graph capture: %s", what, cudaGetErrorString(rc));
    }
    cudaGraphExec_t x = nullptr;
    rc = cudaGraphInstantiate(&x, graph, 0);
    cudaGraphDestroy(graph);
    if (rc != cudaSuccess) {
      destroy_graphs(ex);
      return fail(SWIT_E_CUDA, "%s graph instantiate: %s", what, cudaGetErrorString(rc));
    }
    ex.push_back(x);
  }
  return 0;
}

// True while the caller is capturing `st` into a graph of its own: the loops
// are then issued straight onto st (the branches forked from and joined back
// to it), since a graph launch cannot be captured.
inline bool caller_capturing(cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive;
}

template <class F>
int issue_into_capture(swit_engine* e, cudaStream_t st, int nbatch, F&& issue) {
  // the caller's graph gets every node of the loop: keep it under the same bound
  // as the engine's own graphs
  const size_t nodes = (size_t)nbatch * loop_nodes(e);
  if (nodes > e->graph_nodes)
    return fail(SWIT_E_LIMIT,
                "capturing this loop into the caller's graph would add about %zu kernel nodes, above the %zu-node "
                "bound of one graph; run it uncaptured (the engine then splits it into bounded graphs itself)",
                nodes, e->graph_nodes);
  capture_fork(e, st);
  for (int b = 0; b < nbatch; ++b) issue(b, capture_stream(e, b, st));
  capture_join(e, st);
  CK(cudaGetLastError());
  return 0;
}


template <class R>
int run_forward_loop(swit_engine* e, bool store, cudaStream_t st) {
  if (e->path == 1) {
    for (int s = 0; s < e->ns; ++s) {
      if (store && e->ckpt_k)
        forward_checkpointed<R>(e, s, 1, st);
      else
        launch_forward_steps<R>(e, store, s, 1, st);
    }
    CK(cudaGetLastError());
    return 0;
  }
  std::vector<cudaGraphExec_t>& ex = e->gfwd[store ? 1 : 0];
  const int fb = fwd_batch(e), nbatch = (e->ns + fb - 1) / fb;
  auto issue = [&](int b, cudaStream_t cs) {
    const int s0 = b * fb, nb = std::min(fb, e->ns - s0);
    if (store && e->ckpt_k)
      forward_checkpointed<R>(e, s0, nb, cs);
    else
      launch_forward_steps<R>(e, store, s0, nb, cs);
  };
  if (caller_capturing(st)) return issue_into_capture(e, st, nbatch, issue);
  if (ex.empty()) {
    int rc = capture_chunked(e, ex, nbatch, loop_nodes(e), "forward", issue);
    if (rc) return rc;
  }
  return launch_graphs(ex, st);
}

template <class R>
int run_backward_loop(swit_engine* e, cudaStream_t st) {
  if (e->path == 1) {
    for (int s = 0; s < e->ns; ++s) {
      if (e->ckpt_k)
        backward_checkpointed<R>(e, s, 1, st);
      else
        launch_backward_steps<R>(e, s, 1, st);
    }
    CK(cudaGetLastError());
    return 0;
  }
  const int nbatch = (e->ns + e->batch - 1) / e->batch;
  auto issue = [&](int b, cudaStream_t cs) {
    const int s0 = b * e->batch, nb = std::min(e->batch, e->ns - s0);
    if (e->ckpt_k)
      backward_checkpointed<R>(e, s0, nb, cs);
    else
      launch_backward_steps<R>(e, s0, nb, cs);
  };
  if (caller_capturing(st)) return issue_into_capture(e, st, nbatch, issue);
  if (e->gbwd.empty()) {
    int rc = capture_chunked(e, e->gbwd, nbatch, loop_nodes(e), "backward", issue);
    if (rc) return rc;
  }
  return launch_graphs(e->gbwd, st);
}

template <class R>
__global__ void k_src_in(const float* __restrict__ in, R* out, int ns, int nt) {
  const size_t n = (size_t)ns * (nt + 1);
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(t / (nt + 1)), i = (int)(t - (size_t)s * (nt + 1));
    out[t] = i < nt ? (R)in[(size_t)s * nt + i] : R(0);  // s(nt+1) = 0
  }
}

inline int nblocks(size_t n, int bs = 256);

// Final forward state -> reconstruction fields (set A), fdcore.f90:164-166.
template <class R>
void copy_end(swit_engine* e, cudaStream_t st) {
  Grid<R> g = make_grid<R>(e);
  const bool in_b = e->variant == 2 && (e->nt - 2) % 2 == 0;  // the last step wrote set B
  const R* P = (const R*)(in_b ? e->p2 : e->p);
  const R* U = (const R*)(in_b ? e->u2 : e->u);
  const R* W = (const R*)(in_b ? e->w2 : e->w);
  if (e->ckpt_k) {  // the reverse loop reuses p, u, w; the final state is checkpoint slot ckpt_m-1
    const size_t f = (size_t)e->ns * e->NX * e->LD;
    const R* c = (const R*)e->ckpt + (size_t)(e->ckpt_m - 1) * 3 * f;
    P = c;
    U = c + f;
    W = c + 2 * f;
  }
  k_copy_end<R><<<nblocks((size_t)e->ns * e->nx * e->nz), 256, 0, st>>>(g, P, U, W, (R*)e->pe, (R*)e->ue,
                                                                        (R*)e->we, e->ns);
}

inline int nblocks(size_t n, int bs) {
  size_t b = (n + bs - 1) / bs;
  return (int)std::min<size_t>(b, 152 * 16);
}

// Copies a float input of n values to device staging (or uses it in place).
int stage_input(swit_engine* e, const float* in, size_t n, int on_device, cudaStream_t st, const float** out) {
  if (on_device) {
    *out = in;
    return 0;
  }
  CK(cudaMemcpyAsync(e->d_in, in, n * sizeof(float), cudaMemcpyHostToDevice, st));
  *out = e->d_in;
  return 0;
}

template <class R>
int forward_impl(swit_engine* e, const float* src, void* seis, bool store, int on_device, cudaStream_t st,
                 bool run_loop = true) {
  Grid<R> g = make_grid<R>(e);
  const float* dsrc = src;
  if (!on_device) {
    CK(cudaMemcpyAsync(e->d_src_in, src, (size_t)e->ns * e->nt * sizeof(float), cudaMemcpyHostToDevice, st));
    dsrc = e->d_src_in;
  }
  k_src_in<R><<<nblocks((size_t)e->ns * (e->nt + 1)), 256, 0, st>>>(dsrc, (R*)e->src, e->ns, e->nt);
  const size_t fb = (size_t)e->ns * g.FSZ * e->esz;
  CK(cudaMemsetAsync(e->p, 0, fb, st));
  CK(cudaMemsetAsync(e->u, 0, fb, st));
  CK(cudaMemsetAsync(e->w, 0, fb, st));
  if (e->variant == 2) {
    CK(cudaMemsetAsync(e->p2, 0, fb, st));
    CK(cudaMemsetAsync(e->u2, 0, fb, st));
    CK(cudaMemsetAsync(e->w2, 0, fb, st));
  }
  if (run_loop) {  // a multi-instance engine runs the loops of all its instances itself
    const int rc = run_forward_loop<R>(e, store, st);
    if (rc) return rc;
  }
  if (seis) {
    dim3 grid((e->nt + 31) / 32, (e->ngmax + 31) / 32, e->ns), block(32, 8);
    void* out = on_device ? seis : e->d_stage;
    if (e->prec == 0)
      k_seis_out<R, float><<<grid, block, 0, st>>>((const R*)e->seis_t, (float*)out, e->ns, e->nt, e->ngmax);
    else
      k_seis_out<R, double><<<grid, block, 0, st>>>((const R*)e->seis_t, (double*)out, e->ns, e->nt, e->ngmax);
    if (!on_device)
      CK(cudaMemcpyAsync(seis, e->d_stage, (size_t)e->ns * e->ngmax * e->nt * e->esz, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaGetLastError());
  e->fwd_ready = store;
  return 0;
}

// Reverse loop of the exact adjoint over all shots: plain path one shot at a
// time, batched path captured once into bounded graphs (batches on concurrent
// branches), or issued straight into a caller's capture.
template <class R>
int run_exact_loop(swit_engine* e, cudaStream_t st) {
  if (e->path == 1) {
    for (int s = 0; s < e->ns; ++s) exact_reverse<R>(e, s, 1, st);
    CK(cudaGetLastError());
    return 0;
  }
  const int nbatch = (e->ns + e->batch - 1) / e->batch;
  auto issue = [&](int b, cudaStream_t cs) {
    exact_reverse<R>(e, b * e->batch, std::min(e->batch, e->ns - b * e->batch), cs);
  };
  if (caller_capturing(st)) return issue_into_capture(e, st, nbatch, issue);
  if (e->gxb.empty()) {
    int rc = capture_chunked(e, e->gxb, nbatch, loop_nodes(e), "exact adjoint", issue);
    if (rc) return rc;
  }
  return launch_graphs(e->gxb, st);
}

// Exact adjoint after a storing forward run: adjoint sources already staged in
// adj_t; grad = dJ/dvp (nx, nz), gsrc = dJ/dsrc (ns, nt), either may be null.
template <class R>
int exact_core(swit_engine* e, void* grad, void* gsrc, int on_device, cudaStream_t st) {
  Grid<R> g = make_grid<R>(e);
  const size_t fb = (size_t)e->ns * g.FSZ * e->esz;
  CK(cudaMemsetAsync(e->pb, 0, fb, st));
  CK(cudaMemsetAsync(e->ub, 0, fb, st));
  CK(cudaMemsetAsync(e->wb, 0, fb, st));
  CK(cudaMemsetAsync(e->dg, 0, fb, st));
  CK(cudaMemsetAsync(e->xm, 0, (size_t)e->ns * 2 * e->NX * e->esz, st));
  CK(cudaMemsetAsync(e->xsrc, 0, (size_t)e->ns * e->nt * e->esz, st));
  int rc = run_exact_loop<R>(e, st);
  if (rc) return rc;
  const size_t NI = (size_t)e->nx * e->nz;
  if (grad) {
    void* og = on_device ? grad : e->d_stage;
    if (e->prec == 0)
      k_xgrad<R, float><<<nblocks(NI), 256, 0, st>>>(g, (const R*)e->dg, (const R*)e->xdadc, e->ns, (float*)og);
    else
      k_xgrad<R, double><<<nblocks(NI), 256, 0, st>>>(g, (const R*)e->dg, (const R*)e->xdadc, e->ns, (double*)og);
    CK(cudaGetLastError());
    if (!on_device) CK(cudaMemcpyAsync(grad, og, NI * e->esz, cudaMemcpyDeviceToHost, st));
  }
  if (gsrc)
    CK(cudaMemcpyAsync(gsrc, e->xsrc, (size_t)e->ns * e->nt * e->esz,
                       on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
  return 0;
}

template <class R>
int backward_end(swit_engine* e, void* grad, void* fw, void* bk, int on_device, cudaStream_t st);

// Zeroed adjoint state and imaging sums, reconstruction start: everything of
// the reverse job before its time loop (vec kernels).
template <class R>
int backward_begin(swit_engine* e, cudaStream_t st) {
  Grid<R> g = make_grid<R>(e);
  const size_t fb = (size_t)e->ns * g.FSZ * e->esz, ib = (size_t)e->ns * g.FSI * e->esz;
  CK(cudaMemsetAsync(e->pb, 0, fb, st));
  CK(cudaMemsetAsync(e->ub, 0, fb, st));
  CK(cudaMemsetAsync(e->wb, 0, fb, st));
  CK(cudaMemsetAsync(e->dg, 0, ib, st));
  CK(cudaMemsetAsync(e->dfw, 0, ib, st));
  CK(cudaMemsetAsync(e->dbk, 0, ib, st));
  copy_end<R>(e, st);
  return 0;
}

template <class R>
int backward_core(swit_engine* e, void* grad, void* fw, void* bk, int on_device, cudaStream_t st) {
  Grid<R> g = make_grid<R>(e);
  const size_t fb = (size_t)e->ns * g.FSZ * e->esz, ib = (size_t)e->ns * g.FSI * e->esz;
  CK(cudaMemsetAsync(e->pb, 0, fb, st));
  CK(cudaMemsetAsync(e->ub, 0, fb, st));
  CK(cudaMemsetAsync(e->wb, 0, fb, st));
  if (e->variant == 2) {
    void* z2[] = {e->pb2, e->ub2, e->wb2, e->pe2, e->ue2, e->we2};
    for (void* q : z2) CK(cudaMemsetAsync(q, 0, fb, st));
  }
  CK(cudaMemsetAsync(e->dg, 0, ib, st));
  CK(cudaMemsetAsync(e->dfw, 0, ib, st));
  CK(cudaMemsetAsync(e->dbk, 0, ib, st));
  // the reverse loop starts from the final forward state, which the forward
  // buffers keep until the next forward: every backward sees the same start
  copy_end<R>(e, st);
  int rc = run_backward_loop<R>(e, st);
  if (rc) return rc;
  return backward_end<R>(e, grad, fw, bk, on_device, st);
}

// Shot sum, scaling and outputs after the reverse loop (solver.f90:263-279).
template <class R>
int backward_end(swit_engine* e, void* grad, void* fw, void* bk, int on_device, cudaStream_t st) {
  Grid<R> g = make_grid<R>(e);
  const size_t NI = (size_t)e->nx * e->nz;
  char* stage = (char*)e->d_stage;
  void* og = on_device ? grad : (grad ? stage : nullptr);
  void* of = on_device ? fw : (fw ? stage + NI * e->esz : nullptr);
  void* ob = on_device ? bk : (bk ? stage + 2 * NI * e->esz : nullptr);
  if (e->prec == 0)
    k_reduce<R, float><<<nblocks(NI), 256, 0, st>>>(g, (const R*)e->dg, (const R*)e->dfw, (const R*)e->dbk,
                                                    (const R*)e->cint, e->ns, (float*)og, (float*)of, (float*)ob);
  else
    k_reduce<R, double><<<nblocks(NI), 256, 0, st>>>(g, (const R*)e->dg, (const R*)e->dfw, (const R*)e->dbk,
                                                     (const R*)e->cint, e->ns, (double*)og, (double*)of,
                                                     (double*)ob);
  CK(cudaGetLastError());
  if (!on_device) {
    if (grad) CK(cudaMemcpyAsync(grad, og, NI * e->esz, cudaMemcpyDeviceToHost, st));
    if (fw) CK(cudaMemcpyAsync(fw, of, NI * e->esz, cudaMemcpyDeviceToHost, st));
    if (bk) CK(cudaMemcpyAsync(bk, ob, NI * e->esz, cudaMemcpyDeviceToHost, st));
  }
  return 0;
}

template <class R>
int backward_impl(swit_engine* e, const float* adj, void* grad, void* fw, void* bk, int on_device, cudaStream_t st) {
  const float* dadj;
  int rc = stage_input(e, adj, (size_t)e->ns * e->ngmax * e->nt, on_device, st, &dadj);
  if (rc) return rc;
  dim3 grid((e->nt + 31) / 32, (e->ngmax + 31) / 32, e->ns), block(32, 8);
  k_adj_in<R><<<grid, block, 0, st>>>(dadj, (R*)e->adj_t, e->ns, e->nt, e->ngmax);
  return backward_core<R>(e, grad, fw, bk, on_device, st);
}

template <class R>
int exact_impl(swit_engine* e, const float* adj, void* grad, void* gsrc, int on_device, cudaStream_t st) {
  const float* dadj;
  int rc = stage_input(e, adj, (size_t)e->ns * e->ngmax * e->nt, on_device, st, &dadj);
  if (rc) return rc;
  dim3 grid((e->nt + 31) / 32, (e->ngmax + 31) / 32, e->ns), block(32, 8);
  k_adj_in<R><<<grid, block, 0, st>>>(dadj, (R*)e->adj_t, e->ns, e->nt, e->ngmax);
  return exact_core<R>(e, grad, gsrc, on_device, st);
}

// Waveform misfit per trace and its adjoint source syn - obs for live traces
// (misfit.py:128-148, 263-282), from the synthetics of the last forward run.
template <class R>
int residual_l2(swit_engine* e, const float* obs, int on_device, cudaStream_t st) {
  const float* dobs;
  int rc = stage_input(e, obs, (size_t)e->ns * e->ngmax * e->nt, on_device, st, &dobs);
  if (rc) return rc;
  k_trace_stats<R><<<dim3(e->ngmax, e->ns), 256, 0, st>>>((const R*)e->seis_t, dobs, e->d_ng, e->nt, e->ngmax,
                                                          e->dt32, e->d_live, e->d_mtrace);
  dim3 grid((e->nt + 31) / 32, (e->ngmax + 31) / 32, e->ns), block(32, 8);
  k_residual<R><<<grid, block, 0, st>>>((const R*)e->seis_t, dobs, e->d_live, (R*)e->adj_t, e->nt, e->ngmax);
  CK(cudaGetLastError());
  return 0;
}

// Sum of the per-trace misfits on the host (waits for the stream).
int misfit_sum(swit_engine* e, cudaStream_t st, double* misfit) {
  std::vector<double> mt((size_t)e->ns * e->ngmax);
  CK(cudaMemcpyAsync(mt.data(), e->d_mtrace, mt.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  double acc = 0.0;
  for (double v : mt) acc += v;
  *misfit = acc;
  return 0;
}

template <class R>
int gradient_impl(swit_engine* e, const float* src, const float* obs, void* grad, void* fw, void* bk, void* seis,
                  double* misfit, int on_device, cudaStream_t st) {
  // Host observed data: copied into d_in on the engine's copy stream while the
  // forward loop runs (the copy waits for everything queued on st before this
  // call, e.g. the previous call's residual reading d_in), and the residual
  // waits for the copy.
  const float* dobs = obs;
  if (!on_device) {
    CK(cudaEventRecord(e->ev_in, st));
    CK(cudaStreamWaitEvent(e->cpy, e->ev_in, 0));
  }
  int rc = forward_impl<R>(e, src, seis, true, on_device, st);
  if (rc) return rc;
  if (!on_device) {
    CK(cudaMemcpyAsync(e->d_in, obs, (size_t)e->ns * e->ngmax * e->nt * sizeof(float), cudaMemcpyHostToDevice,
                       e->cpy));
    CK(cudaEventRecord(e->ev_cpy, e->cpy));
    CK(cudaStreamWaitEvent(st, e->ev_cpy, 0));
    dobs = e->d_in;
  }
  rc = residual_l2<R>(e, dobs, 1, st);
  if (rc) return rc;
  rc = e->exact ? exact_core<R>(e, grad, nullptr, on_device, st) : backward_core<R>(e, grad, fw, bk, on_device, st);
  if (rc) return rc;
  return misfit ? misfit_sum(e, st, misfit) : 0;
}

// Model setup on the host, in R: padding (io.f90:231-300), vmin
// (math.f90:342-361), damping table (pml.f90:80-87) and coefficients.
template <class R>
int set_model_impl(swit_engine* e, const float* vp, const float* rho, cudaStream_t st) {
  const int nx = e->nx, nz = e->nz, L = e->L, NX = e->NX, NZ = e->NZ, LD = e->LD;
  double vmax = 0.0;
  for (size_t i = 0; i < (size_t)nx * nz; ++i) {
    if (!std::isfinite(vp[i]) || !(vp[i] > 0.f) || !std::isfinite(rho[i]) || !(rho[i] > 0.f))
      return fail(SWIT_E_MODEL, "vp/rho must be finite and positive (index %zu: vp=%g rho=%g)", i, vp[i], rho[i]);
    vmax = std::max(vmax, (double)vp[i]);
  }
  // toolbox/base.py:42, 58-59: dt < sqrt(3/8) dx / vmax
  const double dt_req = std::sqrt(3.0 / 8.0) * (double)e->dx32 / vmax;
  if (dt_req <= (double)e->dt32)
    return fail(SWIT_E_CFL, "modeling stability: dt = %.4f ms > dt_required = %.4f ms", e->dt32 * 1000.0,
                dt_req * 1000.0);
  std::vector<R> c((size_t)NX * NZ), den((size_t)NX * NZ);
  auto at = [&](std::vector<R>& m, int iz, int ix) -> R& { return m[(size_t)(ix - 1) * NZ + (iz - 1)]; };
  auto pad = [&](std::vector<R>& m, const float* in) {
    for (int ix = 1; ix <= nx; ++ix)
      for (int iz = 1; iz <= nz; ++iz) at(m, L + iz, L + ix) = (R)in[(size_t)(ix - 1) * nz + (iz - 1)];
    for (int ix = 1; ix <= L; ++ix)
      for (int iz = L + 1; iz <= L + nz; ++iz) {
        at(m, iz, ix) = at(m, iz, L + 1);
        at(m, iz, NX - L + ix) = at(m, iz, NX - L);
      }
    for (int iz = 1; iz <= L; ++iz)
      for (int ix = 1; ix <= NX; ++ix) {
        at(m, iz, ix) = at(m, L + 1, ix);
        at(m, NZ - L + iz, ix) = at(m, NZ - L, ix);
      }
  };
  pad(c, vp);
  pad(den, rho);
  // vmin over interior rows i > fs(j) - npml = 1 (flat free surface)
  R vmin = R(10000000000.0);
  for (int i = 1; i <= nz; ++i)
    for (int j = 1; j <= nx; ++j)
      if (i > e->fs - L && vmin > at(c, L + i, L + j)) vmin = at(c, L + i, L + j);
  const R dx = (R)e->dx32, dt = (R)e->dt32;
  std::vector<R> damp(L + 1, R(0));
  {
    const R a = (R)(L - 1) * dx;
    const R kappa = R(3.0) * vmin * (R)std::log(1000.0) / (R(2.0) * a);
    for (int i = 1; i <= L; ++i) {
      const R xa = (R)(i - 1) * dx / a;
      damp[i] = kappa * xa * xa;
    }
  }
  const int LDI = e->variant >= 2 ? LD : e->LDI, IL = e->IL;
  const size_t nci = e->variant >= 2 ? (size_t)NX * LD : (size_t)nx * e->LDI;
  std::vector<R> A((size_t)NX * LD, R(0)), B((size_t)NX * LD, R(0)), ci(nci, R(1));
  for (int ix = 1; ix <= NX; ++ix)
    for (int iz = 1; iz <= NZ; ++iz) {
      const R dn = at(den, iz, ix), cc = at(c, iz, ix);
      A[(size_t)(ix - 1) * LD + (iz - 1)] = dn * cc * cc * dt / dx;  // fdcore.f90:79
      B[(size_t)(ix - 1) * LD + (iz - 1)] = dt / (dn * dx);          // fdcore.f90:99
    }
  for (int jx = 1; jx <= nx; ++jx)
    for (int jz = 1; jz <= nz; ++jz) ci[(size_t)(jx - 1 + IL) * LDI + (jz - 1 + IL)] = at(c, L + jz, L + jx);
  CK(cudaMemcpyAsync(e->A, A.data(), A.size() * sizeof(R), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(e->B, B.data(), B.size() * sizeof(R), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(e->damp, damp.data(), damp.size() * sizeof(R), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(e->cint, ci.data(), ci.size() * sizeof(R), cudaMemcpyHostToDevice, st));
  std::vector<R> dadc;
  if (e->exact) {  // dA/dc of the exact adjoint's vp gradient
    dadc.assign((size_t)NX * LD, R(0));
    for (int ix = 1; ix <= NX; ++ix)
      for (int iz = 1; iz <= NZ; ++iz)
        dadc[(size_t)(ix - 1) * LD + (iz - 1)] = R(2.0) * at(den, iz, ix) * at(c, iz, ix) * dt / dx;
    CK(cudaMemcpyAsync(e->xdadc, dadc.data(), dadc.size() * sizeof(R), cudaMemcpyHostToDevice, st));
  }
  if (e->kp) {
    Grid<R> g = make_grid<R>(e);
    k_kappa<R><<<nblocks((size_t)NX * LD), 256, 0, st>>>(g, (R*)e->kp, (R*)e->ku, (R*)e->kw);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(st));  // host vectors go out of scope
  e->model_set = true;
  e->fwd_ready = false;
  return 0;
}

template <class R>
int export_impl(swit_engine* e, void* boundary, void* pend, void* uend, void* wend, int on_device, cudaStream_t st) {
  if (e->ckpt_k) return fail(SWIT_E_STATE, "this call needs boundary saving (checkpoint_every = 0)");
  Grid<R> g = make_grid<R>(e);
  copy_end<R>(e, st);
  const size_t NB = (size_t)e->ns * e->nt * e->SL, NI = (size_t)e->ns * e->nx * e->nz;
  auto one = [&](void* dst, size_t n, auto&& launch) -> int {
    if (!dst) return 0;
    void* out = dst;
    void* tmp = nullptr;
    if (!on_device) {
      CK(cudaMallocAsync(&tmp, n * e->esz, st));
      out = tmp;
    }
    launch(out);
    CK(cudaGetLastError());
    if (!on_device) {
      CK(cudaMemcpyAsync(dst, tmp, n * e->esz, cudaMemcpyDeviceToHost, st));
      CK(cudaFreeAsync(tmp, st));
    }
    return 0;
  };
  int rc = one(boundary, NB, [&](void* out) {
    if (e->prec == 0)
      k_strips_out<R, float><<<nblocks(NB), 256, 0, st>>>(g, (const R*)e->strips, (float*)out, e->ns);
    else
      k_strips_out<R, double><<<nblocks(NB), 256, 0, st>>>(g, (const R*)e->strips, (double*)out, e->ns);
  });
  if (rc) return rc;
  void* outs[3] = {pend, uend, wend};
  void* fields[3] = {e->pe, e->ue, e->we};
  for (int q = 0; q < 3; ++q) {
    rc = one(outs[q], NI, [&](void* out) {
      if (e->prec == 0)
        k_interior_out<R, float><<<nblocks(NI), 256, 0, st>>>(g, (const R*)fields[q], (float*)out, e->ns);
      else
        k_interior_out<R, double><<<nblocks(NI), 256, 0, st>>>(g, (const R*)fields[q], (double*)out, e->ns);
    });
    if (rc) return rc;
  }
  if (!on_device) CK(cudaStreamSynchronize(st));
  return 0;
}

// Per-launch timing of the stencil kernels with CUDA events.
//
// Per-kernel cost under the conditions of the captured loop: for each of the
// four vec kernels, one graph holding only that kernel's launches -- S steps of
// every batch, batches round-robin on the graph branches as in capture_chunked
// -- timed with CUDA events around one replay.  mean_ms = replay time / launches,
// so mean_ms x (batches per step) is the kernel's time per step, and the four
// kernels' times per step add up to about the loop's time per step (the other
// kernels of a step are absent from each graph, so their overlap is not).  The
// wavefields are left with meaningless values; every forward starts from zero.
template <class R>
int profile_vec_graphs(swit_engine* e, int32_t launches[4], double mean_ms[4], cudaStream_t st) {
  Grid<R> g = make_grid<R>(e);
  const int B = e->batch, nbatch = (e->ns + B - 1) / B;
  const int S = std::min(e->nt - 1, 256);
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  CK(cudaEventCreate(&t0));
  CK(cudaEventCreate(&t1));
  int rc = 0;
  for (int k = 0; k < 4 && !rc; ++k) {
    auto issue = [&](int b, cudaStream_t cs) {
      const int s0 = b * B, nb = std::min(B, e->ns - s0);
      for (int i = 0; i < S; ++i) {
        const int it = k < 2 ? 2 + i : e->nt - i;
        if (k == 0)
          launch_pdl(e->pdl, k_fwd_p_v<R>, vec_grid(e, 0, nb), vec_block(e), cs, g, vec_list(e, 0), make_src(e),
                     (const R*)e->src, (R*)e->p, (const R*)e->u, (const R*)e->w, it, s0);
        else if (k == 1)
          launch_pdl(e->pdl, k_fwd_uw_v<R>, vec_grid(e, 1, nb), vec_block(e), cs, g, vec_list(e, 1), make_rec(e),
                     (const R*)e->p, (R*)e->u, (R*)e->w, (R*)e->seis_t, (R*)e->strips, it, s0);
        else if (k == 2)
          launch_pdl(e->pdl, k_bwd_uw_v<R>, vec_grid(e, 2, nb), vec_block(e), cs, g, vec_list(e, 2),
                     (const R*)e->pb, (R*)e->ub, (R*)e->wb, (const R*)e->pe, (R*)e->ue, (R*)e->we,
                     (const R*)e->strips, it, s0);
        else
          launch_pdl(e->pdl, k_bwd_p_v<R>, vec_grid(e, 3, nb), vec_block(e), cs, g, vec_list(e, 3), make_rec(e),
                     make_src(e), (const R*)e->src, (const R*)e->adj_t, (R*)e->pb, (const R*)e->ub,
                     (const R*)e->wb, (R*)e->pe, (const R*)e->ue, (const R*)e->we, (R*)e->dg, (R*)e->dfw,
                     (R*)e->dbk, (const R*)e->strips, it, s0);
      }
    };
    std::vector<cudaGraphExec_t> ex;
    const size_t saved = e->graph_nodes;
    e->graph_nodes = (size_t)(nbatch + 1) * S;  // one graph per kernel (all batches in one chunk)
    rc = capture_chunked(e, ex, nbatch, (size_t)S, "profile", issue);
    e->graph_nodes = saved;
    if (rc) break;
    float ms = 0.f;
    if ((rc = launch_graphs(ex, st)) == 0) {  // warm-up replay
      cudaEventRecord(t0, st);
      rc = launch_graphs(ex, st);
      cudaEventRecord(t1, st);
      cudaError_t ce = cudaEventSynchronize(t1);
      if (!rc && ce != cudaSuccess) rc = fail(SWIT_E_CUDA, "profile: %s", cudaGetErrorString(ce));
      if (!rc) cudaEventElapsedTime(&ms, t0, t1);
    }
    destroy_graphs(ex);
    launches[k] = nbatch * S;
    mean_ms[k] = (double)ms / (nbatch * S);
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  return rc;
}

template <class R>
int profile_impl(swit_engine* e, int32_t launches[4], double mean_ms[4], cudaStream_t st) {
  if (e->ckpt_k) return fail(SWIT_E_STATE, "this call needs boundary saving (checkpoint_every = 0)");
  if (e->variant == 3 && e->path == 0) return profile_vec_graphs<R>(e, launches, mean_ms, st);
  Grid<R> g = make_grid<R>(e);
  const int nshot_launch = e->path == 1 ? 1 : e->batch;
  std::vector<cudaEvent_t> ev[4];
  auto record = [&](int which) {
    cudaEvent_t a;
    cudaEventCreate(&a);
    ev[which].push_back(a);
    cudaEventRecord(a, st);
  };
  const size_t fb = (size_t)e->ns * g.FSZ * e->esz, ib = (size_t)e->ns * g.FSI * e->esz;
  void* fz[] = {e->p, e->u, e->w, e->p2, e->u2, e->w2};
  for (void* q : fz)
    if (q) CK(cudaMemsetAsync(q, 0, fb, st));
  const int nshot_fwd = e->path == 1 ? 1 : fwd_batch(e);
  for (int s0 = 0; s0 < e->ns; s0 += nshot_fwd) {
    const int nb = std::min(nshot_fwd, e->ns - s0);
    if (e->variant == 4 || e->variant == 5) {
      record(0);
      launch_forward_steps<R>(e, true, s0, nb, st);
      record(0);
      continue;
    }
    dim3 grid, block;
    stencil_shape(e, nb, grid, block);
    for (int it = 2; it <= e->nt; ++it) {
      if (e->variant == 2) {
        record(0);
        launch_fwd_walk<R>(e, true, s0, nb, it, st);
        record(0);
        continue;
      }
      if (e->variant == 6) {
        const dim3 bg(e->nbands, nb), bb(256);
        record(0);
        launch_pdl_sm(false, k_fwd_p_b<R>, bg, bb, e->band_sm[0], st, g, band_list(e, 0), make_src(e),
                      (const R*)e->src, (R*)e->p, (const R*)e->u, (const R*)e->w, it, s0, e->d_err);
        record(0);
        record(1);
        launch_pdl_sm(false, k_fwd_uw_b<R>, bg, bb, e->band_sm[1], st, g, band_list(e, 1), make_rec(e),
                      (const R*)e->p, (R*)e->u, (R*)e->w, (R*)e->seis_t, (R*)e->strips, it, s0, e->d_err);
        record(1);
        continue;
      }
      if (e->variant == 3) {
        record(0);
        k_fwd_p_v<R><<<vec_grid(e, 0, nb), vec_block(e), 0, st>>>(g, vec_list(e, 0), make_src(e), (const R*)e->src,
                                                                (R*)e->p, (const R*)e->u, (const R*)e->w, it, s0);
        record(0);
        record(1);
        k_fwd_uw_v<R><<<vec_grid(e, 1, nb), vec_block(e), 0, st>>>(g, vec_list(e, 1), make_rec(e), (const R*)e->p,
                                                                 (R*)e->u, (R*)e->w, (R*)e->seis_t, (R*)e->strips,
                                                                 it, s0);
        record(1);
        continue;
      }
      record(0);
      k_fwd_p<R><<<grid, block, 0, st>>>(g, make_src(e), (const R*)e->src, (R*)e->p, (const R*)e->u,
                                         (const R*)e->w, it, s0);
      record(0);
      record(1);
      k_fwd_uw<R><<<grid, block, 0, st>>>(g, make_rec(e), (const R*)e->p, (R*)e->u, (R*)e->w, (R*)e->seis_t,
                                          (R*)e->strips, it, s0);
      record(1);
    }
  }
  void* bz[] = {e->pb, e->ub, e->wb, e->pb2, e->ub2, e->wb2};
  for (void* q : bz)
    if (q) CK(cudaMemsetAsync(q, 0, fb, st));
  CK(cudaMemsetAsync(e->dg, 0, ib, st));
  CK(cudaMemsetAsync(e->dfw, 0, ib, st));
  CK(cudaMemsetAsync(e->dbk, 0, ib, st));
  copy_end<R>(e, st);
  for (int s0 = 0; s0 < e->ns; s0 += nshot_launch) {
    const int nb = std::min(nshot_launch, e->ns - s0);
    if (e->variant == 4) {
      record(2);
      launch_backward_steps<R>(e, s0, nb, st);
      record(2);
      continue;
    }
    dim3 grid, block;
    stencil_shape(e, nb, grid, block);
    for (int it = e->nt; it >= 2; --it) {
      if (e->variant == 2) {
        record(2);
        launch_bwd_walk<R>(e, s0, nb, it, st);
        record(2);
        continue;
      }
      if (e->variant == 6) {
        const dim3 bg(e->nbands, nb), bb(256);
        record(2);
        launch_pdl_sm(false, k_bwd_uw_b<R>, bg, bb, e->band_sm[2], st, g, band_list(e, 2), (const R*)e->pb,
                      (R*)e->ub, (R*)e->wb, (const R*)e->pe, (R*)e->ue, (R*)e->we, (const R*)e->strips, it, s0,
                      e->d_err);
        record(2);
        record(3);
        launch_pdl_sm(false, k_bwd_p_b<R>, bg, bb, e->band_sm[3], st, g, band_list(e, 3), make_rec(e), make_src(e),
                      (const R*)e->src, (const R*)e->adj_t, (R*)e->pb, (const R*)e->ub, (const R*)e->wb, (R*)e->pe,
                      (const R*)e->ue, (const R*)e->we, (R*)e->dg, (R*)e->dfw, (R*)e->dbk, (const R*)e->strips, it,
                      s0, e->d_err);
        record(3);
        continue;
      }
      if (e->variant == 3 || e->variant == 5) {
        record(2);
        k_bwd_uw_v<R><<<vec_grid(e, 2, nb), vec_block(e), 0, st>>>(g, vec_list(e, 2), (const R*)e->pb, (R*)e->ub,
                                                                 (R*)e->wb, (const R*)e->pe, (R*)e->ue, (R*)e->we,
                                                                 (const R*)e->strips, it, s0);
        record(2);
        record(3);
        k_bwd_p_v<R><<<vec_grid(e, 3, nb), vec_block(e), 0, st>>>(
            g, vec_list(e, 3), make_rec(e), make_src(e), (const R*)e->src, (const R*)e->adj_t, (R*)e->pb,
            (const R*)e->ub, (const R*)e->wb, (R*)e->pe, (const R*)e->ue, (const R*)e->we, (R*)e->dg, (R*)e->dfw,
            (R*)e->dbk, (const R*)e->strips, it, s0);
        record(3);
        continue;
      }
      record(2);
      k_bwd_uw<R><<<grid, block, 0, st>>>(g, (const R*)e->pb, (R*)e->ub, (R*)e->wb, (const R*)e->pe, (R*)e->ue,
                                          (R*)e->we, (const R*)e->strips, it, s0);
      record(2);
      record(3);
      k_bwd_p<R><<<grid, block, 0, st>>>(g, make_rec(e), make_src(e), (const R*)e->src, (const R*)e->adj_t,
                                         (R*)e->pb, (const R*)e->ub, (const R*)e->wb, (R*)e->pe, (const R*)e->ue,
                                         (const R*)e->we, (R*)e->dg, (R*)e->dfw, (R*)e->dbk, (const R*)e->strips,
                                         it, s0);
      record(3);
    }
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  for (int q = 0; q < 4; ++q) {
    double tot = 0.0;
    const size_t n = ev[q].size() / 2;
    for (size_t i = 0; i < n; ++i) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[q][2 * i], ev[q][2 * i + 1]);
      tot += ms;
    }
    for (cudaEvent_t x : ev[q]) cudaEventDestroy(x);
    launches[q] = (int32_t)n;
    mean_ms[q] = n ? tot / n : 0.0;
  }
  return 0;
}

// Saved forward run -> source, strips and final forward state (the buffers copy_end reads).
template <class R>
int import_impl(swit_engine* e, const float* src, const float* boundary, const float* pend, const float* uend,
                const float* wend, int on_device, cudaStream_t st) {
  if (e->ckpt_k) return fail(SWIT_E_STATE, "this call needs boundary saving (checkpoint_every = 0)");
  Grid<R> g = make_grid<R>(e);
  const size_t NB = (size_t)e->ns * e->nt * e->SL, NI = (size_t)e->ns * e->nx * e->nz;
  const bool in_b = e->variant == 2 && (e->nt - 2) % 2 == 0;
  void* finals[3] = {in_b ? e->p2 : e->p, in_b ? e->u2 : e->u, in_b ? e->w2 : e->w};
  const float* ends[3] = {pend, uend, wend};
  auto staged = [&](const float* in, size_t n, float** tmp) -> int {
    *tmp = nullptr;
    if (on_device) return 0;
    CK(cudaMallocAsync((void**)tmp, n * sizeof(float), st));
    CK(cudaMemcpyAsync(*tmp, in, n * sizeof(float), cudaMemcpyHostToDevice, st));
    return 0;
  };
  float* tmp = nullptr;
  int rc = staged(src, (size_t)e->ns * e->nt, &tmp);
  if (rc) return rc;
  k_src_in<R><<<nblocks((size_t)e->ns * (e->nt + 1)), 256, 0, st>>>(tmp ? tmp : src, (R*)e->src, e->ns, e->nt);
  if (tmp) CK(cudaFreeAsync(tmp, st));
  if ((rc = staged(boundary, NB, &tmp))) return rc;
  k_strips_in<R><<<nblocks(NB), 256, 0, st>>>(g, tmp ? tmp : boundary, (R*)e->strips, e->ns);
  if (tmp) CK(cudaFreeAsync(tmp, st));
  for (int q = 0; q < 3; ++q) {
    if ((rc = staged(ends[q], NI, &tmp))) return rc;
    k_end_in<R><<<nblocks(NI), 256, 0, st>>>(g, tmp ? tmp : ends[q], (R*)finals[q], e->ns);
    if (tmp) CK(cudaFreeAsync(tmp, st));
  }
  CK(cudaGetLastError());
  if (!on_device) CK(cudaStreamSynchronize(st));
  e->fwd_ready = true;
  return 0;
}

// Task lists of the vec kernels from the body tier of every vector (k_tiers):
// per kernel the tier groups 0, 1, 2 (no-work vectors dropped), each ordered by
// tiles of 256/vbx vectors x vbx columns, q fastest, so a warp covers
// 32 * vbx / 256 columns of 256 / vbx vectors as a 2-D block of the grid would.
template <class R>
int vector_tiers(swit_engine* e, std::vector<int>& t) {
  const size_t n = (size_t)e->NX * (e->LD / 4);
  int* d_t = nullptr;
  CK(cudaMalloc(&d_t, 4 * n * sizeof(int)));
  k_tiers<R><<<nblocks(n), 256>>>(make_grid<R>(e), make_src(e), make_rec(e), e->ns, d_t);
  t.resize(4 * n);
  cudaError_t ce = cudaMemcpy(t.data(), d_t, 4 * n * sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d_t);
  if (ce != cudaSuccess) return fail(SWIT_E_CUDA, "task tiers: %s", cudaGetErrorString(ce));
  return 0;
}

template <class R>
int build_lists(swit_engine* e) {
  const int LD4 = e->LD / 4, NX = e->NX;
  const size_t n = (size_t)NX * LD4;
  std::vector<int> t;
  int rt = vector_tiers<R>(e, t);
  if (rt) return rt;
  const int TX = e->vbx, TQ = 256 / e->vbx;
  std::vector<uint32_t> L(4 * n);
  for (int k = 0; k < 4; ++k) {
    uint32_t* out = &L[k * n];
    const int* tk = &t[k * n];
    int m = 0;
    for (int tier = 0; tier < 3; ++tier) {
      if (tier == 1) e->list_n0[k] = m;
      if (tier == 2) e->list_n1[k] = m;
      for (int x0 = 0; x0 < NX; x0 += TX)
        for (int q0 = 0; q0 < LD4; q0 += TQ)
          for (int x = x0; x < std::min(x0 + TX, NX); ++x)
            for (int q = q0; q < std::min(q0 + TQ, LD4); ++q)
              if (tk[(size_t)x * LD4 + q] == tier) out[m++] = ((uint32_t)x << 16) | (uint32_t)q;
    }
    e->list_len[k] = m;
  }
  e->list_stride = n;
  e->h_list = L;
  int rc = dalloc(e, &e->d_list, 4 * n);
  if (rc) return rc;
  CK(cudaMemcpy(e->d_list, L.data(), 4 * n * sizeof(uint32_t), cudaMemcpyHostToDevice));
  // Tier-0 rectangle of each kernel: the deep interior (columns [L+3, NX-L-3],
  // vectors wholly in rows [L+4, NZ-L-3]; vec_flags), when every vector in it
  // has tier 0 for that kernel (a deep source or receiver makes a hole: no
  // rectangle then).  Its vectors leave the device list.
  const int L0 = e->L, NZ = e->NZ;
  const int xa = L0 + 2, xb = NX - L0 - 4;       // 0-based columns
  const int qa = (L0 + 3 + 3) / 4, qb = (NZ - L0 - 7) / 4;  // 4q+1 >= L+4, 4q+4 <= NZ-L-3
  bool use_rect = xb >= xa && qb >= qa;
  if (const char* rv = std::getenv("SWIT_VEC_RECT")) use_rect = use_rect && std::atoi(rv) != 0;
  std::vector<uint32_t> D(4 * n, 0u);
  for (int k = 0; k < 4; ++k) {
    const int* tk = &t[k * n];
    bool ok = use_rect;
    for (int x = xa; ok && x <= xb; ++x)
      for (int q = qa; q <= qb; ++q)
        if (tk[(size_t)x * LD4 + q] != 0) {
          ok = false;
          break;
        }
    const uint32_t* src = &L[k * n];
    uint32_t* dst = &D[k * n];
    int m = 0;
    for (int i = 0; i < e->list_len[k]; ++i) {
      const int x = (int)(src[i] >> 16), q = (int)(src[i] & 0xffffu);
      if (ok && x >= xa && x <= xb && q >= qa && q <= qb) continue;
      dst[m++] = src[i];
    }
    const int rn = ok ? (xb - xa + 1) * (qb - qa + 1) : 0;
    e->rect_x0[k] = xa;
    e->rect_q0[k] = qa;
    e->rect_nq[k] = qb - qa + 1 > 0 ? qb - qa + 1 : 1;
    e->rect_n[k] = rn;
    e->dl_n0[k] = e->list_n0[k] - rn;  // the rectangle's vectors are tier-0 entries
    e->dl_n1[k] = e->list_n1[k] - rn;
    e->dl_len[k] = m;
  }
  if ((rc = dalloc(e, &e->d_dlist, 4 * n))) return rc;
  CK(cudaMemcpy(e->d_dlist, D.data(), 4 * n * sizeof(uint32_t), cudaMemcpyHostToDevice));
  return 0;
}

// Band variant: per kernel and band of band_bc columns, the band's vectors by
// body tier (no-work vectors dropped), column-major within a tier; counts
// {first tier-1 entry, first tier-2 entry, length}.  Also sets the kernels'
// shared-memory sizes.
template <class R>
int build_band_lists(swit_engine* e) {
  const int LD4 = e->LD / 4, NX = e->NX, bc = e->band_bc;
  const size_t n = (size_t)NX * LD4;
  std::vector<int> t;
  int rt = vector_tiers<R>(e, t);
  if (rt) return rt;
  e->nbands = (NX + bc - 1) / bc;
  e->band_stride = bc * LD4;
  const size_t per = (size_t)e->nbands * e->band_stride;
  std::vector<uint32_t> L(4 * per, 0u);
  std::vector<int4> cnt(4 * (size_t)e->nbands);
  for (int k = 0; k < 4; ++k) {
    const int* tk = &t[k * n];
    for (int b = 0; b < e->nbands; ++b) {
      uint32_t* out = &L[k * per + (size_t)b * e->band_stride];
      int m = 0, n0 = 0, n1 = 0;
      for (int tier = 0; tier < 3; ++tier) {
        if (tier == 1) n0 = m;
        if (tier == 2) n1 = m;
        for (int x = b * bc; x < std::min((b + 1) * bc, NX); ++x)
          for (int q = 0; q < LD4; ++q)
            if (tk[(size_t)x * LD4 + q] == tier) out[m++] = ((uint32_t)(x - b * bc) << 16) | (uint32_t)q;
      }
      cnt[k * (size_t)e->nbands + b] = make_int4(n0, n1, m, 0);
    }
  }
  int rc = dalloc(e, &e->d_blist, 4 * per);
  if (!rc) rc = dalloc(e, &e->d_bcnt, 4 * (size_t)e->nbands);
  if (rc) return rc;
  CK(cudaMemcpy(e->d_blist, L.data(), L.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(e->d_bcnt, cnt.data(), cnt.size() * sizeof(int4), cudaMemcpyHostToDevice));
  return 0;
}

// Band variant geometry: columns per band (want, or as many as 256 threads
// cover), shared memory of each kernel checked against the device limit.
template <class R>
int setup_band(swit_engine* e, int want) {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || optin <= 0)
    return fail(SWIT_E_CUDA, "cannot query the shared memory per block");
  const int LD4 = e->LD / 4;
  if (want < 0 || want > 64) return fail(SWIT_E_ARG, "block_x of the band kernels (columns per band) must be 0..64");
  const int bc = want ? want : std::max(1, 256 / LD4);
  e->band_bc = bc;
  e->bx = bc;
  e->band_sm[0] = band_smem(bc, e->LD, 1, 4, e->esz);
  e->band_sm[1] = band_smem(bc, e->LD, 1, 5, e->esz);
  e->band_sm[2] = band_smem(bc, e->LD, 2, 8, e->esz);
  e->band_sm[3] = band_smem(bc, e->LD, 2, 10, e->esz);
  for (size_t b : e->band_sm)
    if (b + 64 > (size_t)optin)
      return fail(SWIT_E_LIMIT, "a band of %d columns needs %zu bytes of shared memory per block (> %d)", bc, b, optin);
  cudaError_t rc = cudaFuncSetAttribute(k_fwd_p_b<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->band_sm[0]);
  if (rc == cudaSuccess)
    rc = cudaFuncSetAttribute(k_fwd_uw_b<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->band_sm[1]);
  if (rc == cudaSuccess)
    rc = cudaFuncSetAttribute(k_bwd_uw_b<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->band_sm[2]);
  if (rc == cudaSuccess)
    rc = cudaFuncSetAttribute(k_bwd_p_b<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->band_sm[3]);
  if (rc != cudaSuccess) return fail(SWIT_E_CUDA, "band kernel attributes: %s", cudaGetErrorString(rc));
  return 0;
}

// Grid index npml + int(x/dx) + 1 in single precision (fdcore.f90:70, 124).
inline int gidx(int L, float x, float dx) { return L + (int)(x / dx) + 1; }

// Dynamic shared memory of a cluster CTA: nf fields, nab coefficient arrays
// and the task list (kernels_cluster.cuh).
inline size_t cluster_smem(const swit_engine* e, int C, int nf, int nab) {
  return cl_field_elems(e->NX, C, e->LD, nf, nab) * e->esz + cl_list_entries(e->NX, C, e->LD) * sizeof(uint32_t);
}

// Attributes and a one-cluster occupancy check of the forward (fwd) and/or the
// reverse (bwd) cluster kernel with MAXT threads.
template <class R, int MAXT>
int cluster_attrs(swit_engine* e, bool fwd, bool bwd) {
  cudaError_t rc = cudaSuccess;
  cudaLaunchAttribute at[1];
  int n = 1;
  if (fwd) {
    rc = cudaFuncSetAttribute(k_fwd_cl<R, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->smf);
    if (rc == cudaSuccess) rc = cudaFuncSetAttribute(k_fwd_cl<R, MAXT>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaLaunchConfig_t cf = cluster_config(e->clf, 1, MAXT, e->smf, nullptr, at);
    if (rc == cudaSuccess) rc = cudaOccupancyMaxActiveClusters(&n, k_fwd_cl<R, MAXT>, &cf);
  }
  if (bwd && rc == cudaSuccess && n >= 1) {
    rc = cudaFuncSetAttribute(k_bwd_cl<R, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->smb);
    if (rc == cudaSuccess) rc = cudaFuncSetAttribute(k_bwd_cl<R, MAXT>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaLaunchConfig_t cb = cluster_config(e->clb, 1, MAXT, e->smb, nullptr, at);
    if (rc == cudaSuccess) rc = cudaOccupancyMaxActiveClusters(&n, k_bwd_cl<R, MAXT>, &cb);
  }
  if (rc != cudaSuccess) return fail(SWIT_E_CUDA, "cluster kernel setup: %s", cudaGetErrorString(rc));
  if (n < 1)
    return fail(SWIT_E_LIMIT, "clusters of %d / %d CTAs with %zu / %zu bytes of shared memory do not fit the device",
                e->clf, e->clb, e->smf, e->smb);
  return 0;
}

// Cluster variant geometry.  want = requested cluster size (0: 16); the
// forward uses it (A and B on chip when they fit too), the reverse loop the
// smallest size >= want whose six fields fit.  Every CTA needs >= 2 columns.
template <class R>
int setup_cluster(swit_engine* e, int want) {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || optin <= 0)
    return fail(SWIT_E_CUDA, "cannot query the shared memory per block");
  const int LD4 = e->LD / 4;
  // 64 registers per thread hold the FP32 bodies, FP64 needs 128
  e->maxt_f = e->maxt_b = e->prec ? 512 : 1024;
#ifdef SWIT_CLUSTER_THREADS_F
  e->maxt_f = SWIT_CLUSTER_THREADS_F;
#endif
#ifdef SWIT_CLUSTER_THREADS_B
  e->maxt_b = SWIT_CLUSTER_THREADS_B;
#endif
  if (LD4 > 512) return fail(SWIT_E_LIMIT, "the cluster kernels need NZ + 2 npml <= 2048");
  if (want < 0 || want > 16) return fail(SWIT_E_ARG, "block_x of the cluster kernels (cluster size) must be 0..16");
  int C = want ? want : 16;
  if (e->NX / C < 2) C = std::max(1, e->NX / 2);
  if (cluster_smem(e, C, 3, 0) > (size_t)optin)
    return fail(SWIT_E_LIMIT, "a cluster of %d CTAs cannot hold the forward wavefields (%zu bytes per CTA > %d)", C,
                cluster_smem(e, C, 3, 0), optin);
  e->clf = C;
  e->ab_local = cluster_smem(e, C, 3, 2) <= (size_t)optin ? 1 : 0;
  e->smf = cluster_smem(e, C, 3, e->ab_local ? 2 : 0);
  int Cb = C;
  while (Cb < 16 && e->NX / (Cb + 1) >= 2 && cluster_smem(e, Cb, 6, 0) > (size_t)optin) ++Cb;
  if (cluster_smem(e, Cb, 6, 0) > (size_t)optin) {
    if (e->variant == 4)
      return fail(SWIT_E_LIMIT, "no cluster of <= 16 CTAs holds the reverse wavefields (%zu bytes per CTA > %d)",
                  cluster_smem(e, Cb, 6, 0), optin);
    Cb = C;  // hybrid: the reverse loop runs the vec kernels; the cluster reverse kernel is never launched
  }
  e->clb = Cb;
  e->smb = std::min(cluster_smem(e, Cb, 6, 0), (size_t)optin);
  e->bx = C;
  int rc = e->maxt_f == 512 ? cluster_attrs<R, 512>(e, true, false) : cluster_attrs<R, 1024>(e, true, false);
  if (rc == 0 && e->variant == 4)
    rc = e->maxt_b == 512 ? cluster_attrs<R, 512>(e, false, true) : cluster_attrs<R, 1024>(e, false, true);
  return rc;
}

}  // namespace

// Many independent problems stepped together (kernels_multi.cuh).
struct swit_multi {
  std::vector<swit_engine*> eng;  // owned, caller order
  std::vector<int> order;         // caller indices by record length, longest first (table order)
  int max_nt = 0;
  Inst<float>* d_tab = nullptr;
  uint32_t* d_list[4] = {nullptr, nullptr, nullptr, nullptr};
  uint2* d_blocks[4] = {nullptr, nullptr, nullptr, nullptr};  // the waves' block tables, one after another
  int* d_on = nullptr;  // per table row: instance switched on for this call
  // A wave is a group of (instance, shot) pairs, in table order, whose reverse-loop state fits its share of
  // the L2; waves run their loops on concurrent branch streams.  act[k][s]: active blocks of kernel k at forward
  // step s (k = 0, 1) or reverse index s (k = 2, 3).
  struct Wave {
    int max_nt = 0;
    double state = 0.0;    // reverse-loop bytes of its pairs (the work of one launch)
    double work = 0.0;     // state bytes x steps summed over its pairs (the work of one loop)
    bool graphed = false;  // its loops are captured graphs; otherwise launched step by step on each call
    size_t boff[4] = {0, 0, 0, 0};
    std::vector<int> act[4];
    std::vector<int> rows;         // table rows with a pair in this wave
    // a wave of one instance runs that instance's own vec kernels on its shots [s0, s0 + nb)
    int s0 = 0, nb = 0;
    cudaGraphExec_t g[3] = {nullptr, nullptr, nullptr};  // its forward (no strips, strips) and reverse loops
  };
  std::vector<Wave> waves;
  size_t graph_nodes = size_t(1) << 20;  // kernel nodes per loop held in the waves' graphs, at most
  int branches = 3;
  cudaStream_t cap = nullptr, capx[2] = {nullptr, nullptr};
  cudaEvent_t ev_fork = nullptr, ev_join[2] = {nullptr, nullptr};
};

namespace {

void multi_release(swit_multi* m) {
  for (auto& w : m->waves)
    for (cudaGraphExec_t& x : w.g)
      if (x) cudaGraphExecDestroy(x);
  if (m->cap) cudaStreamDestroy(m->cap);
  for (int i = 0; i < 2; ++i) {
    if (m->capx[i]) cudaStreamDestroy(m->capx[i]);
    if (m->ev_join[i]) cudaEventDestroy(m->ev_join[i]);
  }
  if (m->ev_fork) cudaEventDestroy(m->ev_fork);
  if (m->d_tab) cudaFree(m->d_tab);
  if (m->d_on) cudaFree(m->d_on);
  for (int k = 0; k < 4; ++k) {
    if (m->d_list[k]) cudaFree(m->d_list[k]);
    if (m->d_blocks[k]) cudaFree(m->d_blocks[k]);
  }
  for (swit_engine* e : m->eng) {
    release(e);
    delete e;
  }
}

// Instance table, padded task lists, waves with their block tables and active
// prefixes.  A wave's reverse-loop state stays under 0.7 L2 / branches (as the
// single-instance engine sizes its batches); its (instance, shot) pairs are in
// table order (record length, longest first).  The waves with the least
// work per launch (where launch overhead weighs most) get captured graphs, up
// to m->graph_nodes kernel nodes per loop over all waves; the others are
// launched step by step, interleaved over the branch streams.
int multi_build(swit_multi* m) {
  const int n = (int)m->eng.size();
  m->order.resize(n);
  for (int i = 0; i < n; ++i) m->order[i] = i;
  std::stable_sort(m->order.begin(), m->order.end(), [&](int a, int b) { return m->eng[a]->nt > m->eng[b]->nt; });
  m->max_nt = m->eng[m->order[0]]->nt;
  std::vector<Inst<float>> tab(n);
  for (int r = 0; r < n; ++r) {
    swit_engine* e = m->eng[m->order[r]];
    Inst<float>& I = tab[r];
    I.g = make_grid<float>(e);
    I.rec = make_rec(e);
    I.src = make_src(e);
    I.ns = e->ns;
    I.s_fwd = (const float*)e->src;
    I.p = (float*)e->p;
    I.u = (float*)e->u;
    I.w = (float*)e->w;
    I.seis_t = (float*)e->seis_t;
    I.strips = (float*)e->strips;
    I.pb = (float*)e->pb;
    I.ub = (float*)e->ub;
    I.wb = (float*)e->wb;
    I.pe = (float*)e->pe;
    I.ue = (float*)e->ue;
    I.we = (float*)e->we;
    I.dg = (float*)e->dg;
    I.dfw = (float*)e->dfw;
    I.dbk = (float*)e->dbk;
    I.adj_t = (const float*)e->adj_t;
  }
  CK(cudaMalloc(&m->d_tab, n * sizeof(Inst<float>)));
  CK(cudaMemcpy(m->d_tab, tab.data(), n * sizeof(Inst<float>), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&m->d_on, n * sizeof(int)));
  // padded task lists of every instance, one array per kernel
  std::vector<uint32_t> base[4], chunks[4];
  for (int k = 0; k < 4; ++k) {
    std::vector<uint32_t> L;
    for (int r = 0; r < n; ++r) {
      const swit_engine* e = m->eng[m->order[r]];
      const uint32_t* src = &e->h_list[(size_t)k * e->list_stride];
      base[k].push_back((uint32_t)L.size());
      for (int i = 0; i < e->list_len[k]; ++i) {
        const uint32_t t = i < e->list_n0[k] ? 0u : (i < e->list_n1[k] ? 1u : 2u);
        L.push_back((t << 30) | src[i]);
      }
      while (L.size() % kMultiBlock) L.push_back(kMultiPad);
      chunks[k].push_back((uint32_t)((L.size() - base[k][r]) / kMultiBlock));
    }
    CK(cudaMalloc(&m->d_list[k], std::max<size_t>(L.size(), 1) * sizeof(uint32_t)));
    CK(cudaMemcpy(m->d_list[k], L.data(), L.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
  }
  // waves of (row, shot) pairs
  int dev = 0, l2 = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess ||
      l2 <= 0)
    l2 = 64 << 20;
  std::vector<double> state(n);
  for (int r = 0; r < n; ++r) {
    const swit_engine* e = m->eng[m->order[r]];
    state[r] = (3.0 * e->NX * e->NZ + 6.0 * e->nx * e->nz) * sizeof(float);
  }
  double budget = 0.7 * l2 / m->branches;
  if (const char* wb = std::getenv("SWIT_MULTI_WAVE_BYTES")) {  // smaller waves, e.g. to test them
    const double v = std::atof(wb);
    if (v > 0) budget = v;
  }
  if (const char* gn = std::getenv("SWIT_MULTI_GRAPH_NODES")) {  // e.g. 0: every wave launched step by step
    const long long v = std::atoll(gn);
    if (v >= 0) m->graph_nodes = (size_t)v;
  }
  // A problem's shots form waves of their own, equal parts of at most budget / state shots (so that its
  // waves run its single-instance kernels; fewer, larger waves than the engine's own batches, which spread
  // one problem over the branches); problems whose shots all fit in half the budget share waves with the
  // next such problems, in table order (the shared kernels).
  std::vector<std::vector<std::pair<int, int>>> groups, shared(1);
  double used = 0.0;
  for (int r = 0; r < n; ++r) {
    const int ns = m->eng[m->order[r]]->ns;
    if (ns * state[r] <= 0.5 * budget) {
      if (used + ns * state[r] > budget && !shared.back().empty()) {
        shared.emplace_back();
        used = 0.0;
      }
      for (int sh = 0; sh < ns; ++sh) shared.back().emplace_back(r, sh);
      used += ns * state[r];
      continue;
    }
    const int per = std::max(1, (int)std::min<double>(ns, budget / state[r]));
    const int nw = (ns + per - 1) / per;
    for (int i = 0; i < nw; ++i) {
      groups.emplace_back();
      for (int sh = (int)((long long)ns * i / nw); sh < (int)((long long)ns * (i + 1) / nw); ++sh)
        groups.back().emplace_back(r, sh);
    }
  }
  for (auto& gr : shared)
    if (!gr.empty()) groups.push_back(std::move(gr));
  std::vector<uint2> B[4];
  for (auto& gr : groups) {
    swit_multi::Wave w;
    w.max_nt = m->eng[m->order[gr.front().first]]->nt;
    for (auto& pr : gr) {
      w.state += state[pr.first];
      w.work += state[pr.first] * (m->eng[m->order[pr.first]]->nt - 1);
      if (w.rows.empty() || w.rows.back() != pr.first) w.rows.push_back(pr.first);
    }
    if (w.rows.size() == 1) {  // the pairs of one instance are consecutive shots
      w.s0 = gr.front().second;
      w.nb = (int)gr.size();
    }
    for (int k = 0; k < 4; ++k) {
      w.boff[k] = B[k].size();
      std::vector<int> cum;  // blocks up to and including each pair
      for (auto& pr : gr) {
        const int r = pr.first;
        for (uint32_t c = 0; c < chunks[k][r]; ++c)
          B[k].push_back(make_uint2(((uint32_t)r << 16) | (uint32_t)pr.second, base[k][r] + (uint32_t)kMultiBlock * c));
        cum.push_back((int)(B[k].size() - w.boff[k]));
      }
      // pairs whose instance has nt >= s run forward step s and reverse index s - 2: a prefix of the wave
      w.act[k].assign(w.max_nt + 1, 0);
      for (int s = 2; s <= w.max_nt; ++s) {
        size_t np = 0;
        while (np < gr.size() && m->eng[m->order[gr[np].first]]->nt >= s) ++np;
        const int a = np ? cum[np - 1] : 0;
        if (k < 2)
          w.act[k][s] = a;
        else
          w.act[k][s - 2] = a;
      }
    }
    m->waves.push_back(std::move(w));
  }
  std::vector<int> by_work(m->waves.size());
  for (size_t i = 0; i < by_work.size(); ++i) by_work[i] = (int)i;
  std::stable_sort(by_work.begin(), by_work.end(),
                   [&](int a, int b) { return m->waves[a].state < m->waves[b].state; });
  size_t nodes = 0;
  for (int i : by_work) {
    const size_t wn = 2 * (size_t)(m->waves[i].max_nt - 1);
    if (nodes + wn > m->graph_nodes) break;
    nodes += wn;
    m->waves[i].graphed = true;
  }
  for (int k = 0; k < 4; ++k) {
    CK(cudaMalloc(&m->d_blocks[k], std::max<size_t>(B[k].size(), 1) * sizeof(uint2)));
    CK(cudaMemcpy(m->d_blocks[k], B[k].data(), B[k].size() * sizeof(uint2), cudaMemcpyHostToDevice));
  }
  m->branches = std::max(1, std::min(m->branches, (int)m->waves.size()));
  CK(cudaStreamCreateWithFlags(&m->cap, cudaStreamNonBlocking));
  for (int i = 0; i < 2; ++i) {
    CK(cudaStreamCreateWithFlags(&m->capx[i], cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&m->ev_join[i], cudaEventDisableTiming));
  }
  CK(cudaEventCreateWithFlags(&m->ev_fork, cudaEventDisableTiming));
  return 0;
}

// Steps [q0, q1) of wave w's forward (which = 0: no strips, 1: with strips) or
// reverse (which = 2) loop on st; step q is forward step it = q + 2, reverse
// index jr = q (instance step nt - q).  One launch per phase and step covers
// every pair of the wave still running.
void wave_steps(swit_multi* m, swit_multi::Wave& w, int which, int q0, int q1, cudaStream_t st) {
  if (w.rows.size() == 1) {
    // one instance: its own single-instance kernels (same bodies, same bits), without
    // the instance table or the per-instance block padding of the shared kernels
    swit_engine* e = m->eng[m->order[w.rows[0]]];
    if (which < 2)
      launch_forward_steps<float>(e, which == 1, w.s0, w.nb, st, q0 + 2, q1 + 1);
    else
      launch_backward_steps<float>(e, w.s0, w.nb, st, e->nt - q0, e->nt - q1 + 1);
    return;
  }
  const dim3 block(kMultiBlock);
  const Inst<float>* tab = m->d_tab;
  auto grid = [](int nb) { return dim3((unsigned)std::max(1, nb)); };
  auto ml = [&](int k, int nb) { return MultiLaunch{m->d_blocks[k] + w.boff[k], m->d_list[k], m->d_on, nb}; };
  for (int q = q0; q < q1; ++q) {
    if (which < 2) {
      const int it = q + 2;
      launch_pdl(true, k_fwd_p_m<float>, grid(w.act[0][it]), block, st, tab, ml(0, w.act[0][it]), it);
      launch_pdl(true, k_fwd_uw_m<float>, grid(w.act[1][it]), block, st, tab, ml(1, w.act[1][it]), it, which);
    } else {
      launch_pdl(true, k_bwd_uw_m<float>, grid(w.act[2][q]), block, st, tab, ml(2, w.act[2][q]), q);
      launch_pdl(true, k_bwd_p_m<float>, grid(w.act[3][q]), block, st, tab, ml(3, w.act[3][q]), q);
    }
  }
}

// The forward (which = 0: no strips, 1: with strips) or reverse (which = 2)
// loop of every switched-on instance.  A graphed wave's loop is captured once
// into a graph of its own.  A call spreads the waves that hold a switched-on
// instance over the concurrent branch streams, largest first onto the least
// loaded branch, launches the graphs, and then the other waves step by step, a
// few steps per branch in turn so that every branch has work queued.  on[i]
// (caller order) switches instance i on.
int multi_loop(swit_multi* m, int which, const std::vector<int>& on, cudaStream_t st) {
  std::vector<int> rows(m->eng.size());
  for (size_t r = 0; r < rows.size(); ++r) rows[r] = on[m->order[r]];
  CK(cudaMemcpyAsync(m->d_on, rows.data(), rows.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  std::vector<int> active;
  for (int wi = 0; wi < (int)m->waves.size(); ++wi)
    for (int r : m->waves[wi].rows)
      if (rows[r]) {
        active.push_back(wi);
        break;
      }
  for (int wi : active) {
    swit_multi::Wave& w = m->waves[wi];
    if (!w.graphed || w.g[which]) continue;
    cudaError_t rc = cudaStreamBeginCapture(m->cap, cudaStreamCaptureModeThreadLocal);
    if (rc != cudaSuccess) return fail(SWIT_E_CUDA, "multi-instance graph capture: %s", cudaGetErrorString(rc));
    wave_steps(m, w, which, 0, w.max_nt - 1, m->cap);
    cudaGraph_t graph = nullptr;
    rc = cudaStreamEndCapture(m->cap, &graph);
    if (rc == cudaSuccess) {
      rc = cudaGraphInstantiate(&w.g[which], graph, 0);
      cudaGraphDestroy(graph);
    }
    if (rc != cudaSuccess) {
      w.g[which] = nullptr;
      return fail(SWIT_E_CUDA, "multi-instance graph: %s", cudaGetErrorString(rc));
    }
  }
  // the waves on the branch streams, forked from and joined back to st
  const int br = std::max(1, std::min(m->branches, (int)active.size()));
  auto branch = [&](int b) { return b ? m->capx[b - 1] : st; };
  CK(cudaEventRecord(m->ev_fork, st));
  for (int i = 0; i < br - 1; ++i) CK(cudaStreamWaitEvent(m->capx[i], m->ev_fork, 0));
  std::vector<int> by_work = active;
  std::stable_sort(by_work.begin(), by_work.end(),
                   [&](int a, int b) { return m->waves[a].work > m->waves[b].work; });
  std::vector<double> load(br, 0.0);
  std::vector<std::vector<int>> direct(br);
  for (int wi : by_work) {
    const int b = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    load[b] += m->waves[wi].work;
    if (m->waves[wi].graphed)
      CK(cudaGraphLaunch(m->waves[wi].g[which], branch(b)));
    else
      direct[b].push_back(wi);
  }
  // per branch: position (wave, next step) in its list of directly launched waves
  constexpr int kStepsPerTurn = 8;
  std::vector<size_t> wpos(br, 0);
  std::vector<int> qpos(br, 0);
  for (bool more = true; more;) {
    more = false;
    for (int b = 0; b < br; ++b) {
      if (wpos[b] >= direct[b].size()) continue;
      swit_multi::Wave& w = m->waves[direct[b][wpos[b]]];
      const int q1 = std::min(w.max_nt - 1, qpos[b] + kStepsPerTurn);
      wave_steps(m, w, which, qpos[b], q1, branch(b));
      qpos[b] = q1;
      if (q1 == w.max_nt - 1) {
        ++wpos[b];
        qpos[b] = 0;
      }
      more = true;
    }
  }
  CK(cudaGetLastError());
  for (int i = 0; i < br - 1; ++i) {
    CK(cudaEventRecord(m->ev_join[i], m->capx[i]));
    CK(cudaStreamWaitEvent(st, m->ev_join[i], 0));
  }
  return 0;
}

}  // namespace

extern "C" {

const char* swit_last_error(void) { return g_err.c_str(); }

// Automatic shots per launch and graph branches of the vec kernels.  The
// reverse loop touches per shot 3 wavefields on the PML grid and 6 interior
// arrays; the step kernels are fastest when the shots of the branches in flight
// keep that state in L2 (about 0.7 of it, the rest holding strips, traces and
// coefficients) and when the branches carry equal work.  So: shots in flight T =
// 0.7 L2 / state, branches br (3 unless given), batches k = br * ceil(ns / T)
// (a multiple of br, so the branches get the same number of launches) and
// ceil(ns / k) shots per batch.  At 481x141 (npml 40) on GB300: 28 shots in
// flight, 6 batches of 9 on 3 branches.
void auto_batches(swit_engine* e, int branches) {
  int dev = 0, l2 = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess ||
      l2 <= 0)
    l2 = 64 << 20;
  // reverse-loop state per shot: adjoint fields on the PML grid, reconstruction
  // fields and imaging sums on the interior; the walk kernels keep two sets
  const double state = e->variant == 2 ? (6.0 * e->NX * e->NZ + 9.0 * e->nx * e->nz) * e->esz
                                       : (3.0 * e->NX * e->NZ + 6.0 * e->nx * e->nz) * e->esz;
  const int inflight = std::max(1, (int)(0.7 * l2 / state));
  const int br = std::max(1, std::min(branches ? branches : 3, e->ns));
  const int per_branch = std::max(1, inflight / br);
  const int rounds = (e->ns + br * per_branch - 1) / (br * per_branch);
  // and at most about 1 M kernel nodes per captured loop (grids whose state
  // does not fit the L2 would otherwise run one shot per launch)
  const int kmax = std::max(br, (int)(((size_t)1 << 20) / (2 * (size_t)(e->nt - 1))) / br * br);
  const int k = std::min(std::min(e->ns, br * rounds), kmax);
  e->batch = (e->ns + k - 1) / k;
  e->branches = br;
}

int swit_create(const swit_desc* d, swit_engine** out) {
  if (!d || !out) return fail(SWIT_E_ARG, "null argument");
  *out = nullptr;
  if (d->nx < 8 || d->nz < 8) return fail(SWIT_E_ARG, "nx and nz must be >= 8 (got %d, %d)", d->nx, d->nz);
  if (d->npml < 2) return fail(SWIT_E_ARG, "npml must be >= 2 (got %d)", d->npml);
  if (d->nt < 2) return fail(SWIT_E_ARG, "nt must be >= 2 (got %d)", d->nt);
  if (d->ns < 1 || d->ng_max < 1) return fail(SWIT_E_ARG, "ns and ng_max must be >= 1");
  if (!(d->dx > 0.f) || !(d->dt > 0.f)) return fail(SWIT_E_ARG, "dx and dt must be > 0");
  if (d->precision != 0 && d->precision != 1) return fail(SWIT_E_ARG, "precision must be 0 or 1");
  if (d->path != 0 && d->path != 1) return fail(SWIT_E_ARG, "path must be 0 (batched) or 1 (plain)");
  if (!d->ng || !d->src_x || !d->src_z || !d->rec_x || !d->rec_z) return fail(SWIT_E_ARG, "null geometry array");
  if (d->ns > 65535) return fail(SWIT_E_LIMIT, "at most 65535 shots per engine");

  swit_engine* e = new swit_engine();
  e->nx = d->nx;
  e->nz = d->nz;
  e->L = d->npml;
  e->nt = d->nt;
  e->NX = d->nx + 2 * d->npml;
  e->NZ = d->nz + 2 * d->npml;
  e->LD = round_up(e->NZ, 32);
  e->LDI = round_up(e->nz, 32);
  e->fs = d->npml + 1;  // io.f90:792, flat topography
  e->fs_flag = d->free_surface == 1 ? 1 : 0;
  e->ns = d->ns;
  e->ngmax = d->ng_max;
  e->SL = 9 * d->nx + 6 * d->nz;
  e->prec = d->precision;
  e->path = d->path;
  e->dx32 = d->dx;
  e->dt32 = d->dt;
  e->esz = e->prec ? sizeof(double) : sizeof(float);
  e->batch = d->shots_per_batch > 0 ? std::min(d->shots_per_batch, d->ns) : d->ns;
  if (d->kernel_variant < 0 || d->kernel_variant > 6) {
    delete e;
    return fail(SWIT_E_ARG, "kernel_variant must be 0..6");
  }
  e->variant = d->kernel_variant ? d->kernel_variant : 3;
  if (d->adjoint_mode < 0 || d->adjoint_mode > 1) {
    delete e;
    return fail(SWIT_E_ARG, "adjoint_mode must be 0 (fd2dmpi's adjoint) or 1 (exact) (got %d)", d->adjoint_mode);
  }
  if (d->adjoint_mode == 1 && e->variant != 3) {
    delete e;
    return fail(SWIT_E_ARG, "the exact adjoint runs on the vec kernels (kernel_variant 0 or 3)");
  }
  e->exact = d->adjoint_mode;
  if (d->receiver_component < 0 || d->receiver_component > 2) {
    delete e;
    return fail(SWIT_E_ARG, "receiver_component must be 0 (p), 1 (vx) or 2 (vz) (got %d)", d->receiver_component);
  }
  if (d->receiver_component && e->variant != 2 && e->variant != 3) {
    delete e;
    return fail(SWIT_E_ARG, "vx / vz receivers run on the walk or vec kernels (kernel_variant 0, 2 or 3)");
  }
  e->rcomp = d->receiver_component;
  if (e->exact) e->SL = e->NX * e->LD;  // the strip buffer holds D of each step
  if (e->variant == 2) {
    e->bx = d->block_x > 0 ? d->block_x : 8;  // columns per tile
    if (e->bx < 2 || e->bx > 256) {
      delete e;
      return fail(SWIT_E_ARG, "block_x (columns per tile) of the walk kernels must be 2..256 (got %d)", e->bx);
    }
  } else if (e->variant == 6) {
    int rc6 = e->prec ? setup_band<double>(e, d->block_x) : setup_band<float>(e, d->block_x);
    if (rc6) {
      delete e;
      return rc6;
    }
  } else if (e->variant == 4 || e->variant == 5) {
    int rc4 = e->prec ? setup_cluster<double>(e, d->block_x) : setup_cluster<float>(e, d->block_x);
    if (rc4) {
      delete e;
      return rc4;
    }
  } else if (e->variant == 3) {
    // one thread per 4-row vector; task lists ordered by tiles of 256 / block_x vectors x block_x columns
    e->bx = e->vbx = d->block_x > 0 ? d->block_x : 4;
    if (e->bx > 64 || (e->bx & (e->bx - 1))) {
      delete e;
      return fail(SWIT_E_ARG, "block_x of the vec kernels must be a power of two <= 64");
    }
  } else {
    e->bx = d->block_x > 0 ? d->block_x : 4;
    if (32 * e->bx > 256 || (e->bx & (e->bx - 1))) {
      delete e;
      return fail(SWIT_E_ARG, "block_x of the split kernels must be a power of two <= 8");
    }
  }
  e->IL = e->variant >= 2 ? e->L : 0;
  if (d->checkpoint_every < 0) {
    delete e;
    return fail(SWIT_E_ARG, "checkpoint_every must be >= 0 (got %d)", d->checkpoint_every);
  }
  if (d->checkpoint_every > 0 && e->variant != 2 && e->variant != 3 && e->variant != 6) {
    delete e;
    return fail(SWIT_E_ARG,
                "checkpointed recomputation needs the walk, vec or band kernels (kernel_variant 0, 2, 3 or 6)");
  }
  e->ckpt_k = std::min(d->checkpoint_every, e->nt);
  if (d->graph_branches < 0 || d->graph_branches > kCapStreamsMax) {
    delete e;
    return fail(SWIT_E_ARG, "graph_branches must be 0 (automatic) or 1..%d (got %d)", kCapStreamsMax,
                d->graph_branches);
  }
  e->branches = d->graph_branches ? d->graph_branches : 2;
  e->graph_nodes = kGraphNodes;
  e->band_wait = kBandWaitLimit;
  if (const char* bw = std::getenv("SWIT_BAND_WAIT_POLLS")) {  // a shorter wait, e.g. to test the timeout path
    const long long v = std::atoll(bw);
    if (v >= 0 && v < (long long)kBandWaitLimit) e->band_wait = (unsigned)v;
  }
  if (const char* gn = std::getenv("SWIT_GRAPH_NODES")) {  // smaller graphs, e.g. to test the chunking
    const long long v = std::atoll(gn);
    if (v > 0) e->graph_nodes = (size_t)v;
  }
  if (d->shots_per_batch == 0 && e->path == 0 && (e->variant == 2 || e->variant == 3))
    auto_batches(e, d->graph_branches);
  e->ckpt_m = e->ckpt_k ? (e->nt + e->ckpt_k - 1) / e->ckpt_k : 0;
  e->snt = e->ckpt_k ? e->ckpt_k : e->nt;
  e->sit0 = 1;
#ifdef SWIT_NO_PDL
  e->pdl = false;
#else
  e->pdl = e->path == 0;
#endif
  cudaGetDevice(&e->device);

  // geometry: indices exactly as fdcore.f90:70-72, 124-126, 217-218, 349-359
  const int L = e->L, nx = e->nx, nz = e->nz, NX = e->NX, ns = e->ns, ngm = e->ngmax, fs = e->fs;
  e->ng.assign(d->ng, d->ng + ns);
  e->isx.resize(ns);
  e->isz.resize(ns);
  e->risx.resize(ns);
  e->risz.resize(ns);
  e->colptr.assign((size_t)ns * (NX + 2), 0);
  e->ent_ig.clear();
  e->ent_zr.clear();
  auto inside = [&](float x, int n) { return x >= -0.0f && (int)(x / d->dx) <= n - 1; };
  for (int s = 0; s < ns; ++s) {
    if (e->ng[s] < 0 || e->ng[s] > ngm) {
      delete e;
      return fail(SWIT_E_ARG, "ng[%d] = %d outside [0, ng_max]", s, d->ng[s]);
    }
    const float xs = d->src_x[s], zs = d->src_z[s];
    if (!inside(xs, nx) || !inside(zs, nz)) {
      delete e;
      return fail(SWIT_E_GEOM, "source %d at (%g, %g) m is outside the model", s + 1, xs, zs);
    }
    e->isx[s] = gidx(L, xs, d->dx);
    e->isz[s] = gidx(L, zs, d->dx);
    if (e->isz[s] == fs) e->isz[s] += 1;
    // reconstruction-side source subtraction, fdcore.f90:217-218, 250-256
    const int rx = (int)(xs / d->dx) + 1, rz = (int)(zs / d->dx) + 1;
    const bool act = rx > 2 && rx < nx - 1 && rz > 3 && rz < nz - 1;
    e->risx[s] = act ? rx : 0;
    e->risz[s] = act ? (rz > fs - L ? rz : fs - L + 1) : 0;
    // receivers grouped by column, in receiver order within a column
    std::vector<std::pair<int, int>> cols;  // (igx, ig)
    for (int ig = 0; ig < e->ng[s]; ++ig) {
      const float xg = d->rec_x[(size_t)s * ngm + ig], zg = d->rec_z[(size_t)s * ngm + ig];
      if (!inside(xg, nx) || !inside(zg, nz)) {
        delete e;
        return fail(SWIT_E_GEOM, "receiver %d of shot %d at (%g, %g) m is outside the model", ig + 1, s + 1, xg, zg);
      }
      cols.push_back({gidx(L, xg, d->dx), ig});
    }
    std::stable_sort(cols.begin(), cols.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    int* cp = &e->colptr[(size_t)s * (NX + 2)];
    const int base = (int)e->ent_ig.size();
    std::vector<int> cnt(NX + 2, 0);
    for (auto& c : cols) {
      const int ig = c.second;
      const float zg = d->rec_z[(size_t)s * ngm + ig];
      int igz = gidx(L, zg, d->dx);
      // forward gather moves igz == fs down one node (fdcore.f90:126); the
      // adjoint injects at igz if igz > fs else fs+1 (fdcore.f90:355-359).  For
      // z >= 0 both give the same row.
      if (igz == fs) igz += 1;
      e->ent_ig.push_back(ig);
      e->ent_zr.push_back(igz);
      cnt[c.first] += 1;
    }
    int acc = base;
    for (int ix = 0; ix <= NX + 1; ++ix) {
      cp[ix] = acc;
      acc += cnt[ix];
    }
    int lo = 1 << 30, hi = -1;
    for (size_t q = (size_t)base; q < e->ent_zr.size(); ++q) {
      lo = std::min(lo, e->ent_zr[q]);
      hi = std::max(hi, e->ent_zr[q]);
    }
    e->zlo.push_back(lo);
    e->zhi.push_back(hi);
  }
  const size_t nent = std::max<size_t>(e->ent_ig.size(), 1);
  std::vector<int4> rcol((size_t)ns * (NX + 2));
  for (int s = 0; s < ns; ++s)
    for (int c = 0; c <= NX + 1; ++c) {
      const int* cp = &e->colptr[(size_t)s * (NX + 2)];
      const int e0 = cp[c], n = (c <= NX ? cp[c + 1] : e0) - e0;
      rcol[(size_t)s * (NX + 2) + c] = n ? make_int4(e->ent_ig[e0], e->ent_zr[e0], n, e0) : make_int4(-1, -1, 0, e0);
    }
  const size_t FSZ = (size_t)e->NX * e->LD, FSI = (size_t)e->nx * e->LDI;
  int rc = 0;
#define AL(expr)    \
  if ((rc = (expr))) { \
    release(e);      \
    delete e;        \
    return rc;       \
  }
  AL(dalloc(e, &e->d_ng, ns));
  AL(dalloc(e, &e->d_isx, ns));
  AL(dalloc(e, &e->d_isz, ns));
  AL(dalloc(e, &e->d_risx, ns));
  AL(dalloc(e, &e->d_risz, ns));
  AL(dalloc(e, &e->d_colptr, (size_t)ns * (NX + 2)));
  AL(dalloc(e, &e->d_rcol, (size_t)ns * (NX + 2)));
  AL(dalloc(e, &e->d_zlo, ns));
  AL(dalloc(e, &e->d_zhi, ns));
  AL(dalloc(e, &e->d_ig, nent));
  AL(dalloc(e, &e->d_zr, nent));
  AL(dalloc(e, &e->d_live, (size_t)ns * ngm));
  AL(dalloc(e, &e->d_mtrace, (size_t)ns * ngm));
  AL(dalloc(e, &e->d_err, 1));
  AL(valloc(e, &e->A, FSZ));
  AL(valloc(e, &e->B, FSZ));
  AL(valloc(e, &e->damp, (size_t)L + 1));
  AL(valloc(e, &e->cint, e->variant >= 2 ? FSZ : FSI));
  if (e->variant >= 2) {
    AL(valloc(e, &e->kp, FSZ));
    AL(valloc(e, &e->ku, FSZ));
    AL(valloc(e, &e->kw, FSZ));
  }
  void** fields[] = {&e->p, &e->u, &e->w, &e->pb, &e->ub, &e->wb};
  for (void** f : fields) AL(valloc(e, f, (size_t)ns * FSZ));
  void** ifields[] = {&e->pe, &e->ue, &e->we, &e->dg, &e->dfw, &e->dbk};
  for (void** f : ifields) AL(valloc(e, f, (size_t)ns * (e->variant >= 2 ? FSZ : FSI)));
  if (e->variant == 2) {  // second state set of the walk kernels
    void** f2[] = {&e->p2, &e->u2, &e->w2, &e->pb2, &e->ub2, &e->wb2, &e->pe2, &e->ue2, &e->we2};
    for (void** f : f2) AL(valloc(e, f, (size_t)ns * FSZ));
  }
  AL(valloc(e, &e->strips, (size_t)ns * e->snt * e->SL));
  if (e->ckpt_k) AL(valloc(e, &e->ckpt, (size_t)e->ckpt_m * 3 * ns * FSZ));
  if (e->exact) {
    AL(valloc(e, &e->xm, (size_t)ns * 2 * e->NX));
    AL(valloc(e, &e->xsrc, (size_t)ns * e->nt));
    AL(valloc(e, &e->xdadc, FSZ));
  }
  AL(valloc(e, &e->src, (size_t)ns * (e->nt + 1)));
  AL(valloc(e, &e->seis_t, (size_t)ns * e->nt * ngm));
  AL(valloc(e, &e->adj_t, (size_t)ns * e->nt * ngm));
  AL(dalloc(e, &e->d_in, (size_t)ns * ngm * e->nt));
  AL(dalloc(e, &e->d_src_in, (size_t)ns * e->nt));
  AL(valloc(e, &e->d_stage, std::max((size_t)ns * ngm * e->nt, (size_t)3 * nx * nz)));
#undef AL
  auto h2d = [&](void* dst, const void* src, size_t bytes) -> int {
    CK(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return 0;
  };
  if ((rc = h2d(e->d_ng, e->ng.data(), ns * sizeof(int))) || (rc = h2d(e->d_isx, e->isx.data(), ns * sizeof(int))) ||
      (rc = h2d(e->d_isz, e->isz.data(), ns * sizeof(int))) ||
      (rc = h2d(e->d_risx, e->risx.data(), ns * sizeof(int))) ||
      (rc = h2d(e->d_risz, e->risz.data(), ns * sizeof(int))) ||
      (rc = h2d(e->d_colptr, e->colptr.data(), e->colptr.size() * sizeof(int))) ||
      (rc = h2d(e->d_rcol, rcol.data(), rcol.size() * sizeof(int4))) ||
      (rc = h2d(e->d_zlo, e->zlo.data(), ns * sizeof(int))) || (rc = h2d(e->d_zhi, e->zhi.data(), ns * sizeof(int))) ||
      (e->ent_ig.size() && ((rc = h2d(e->d_ig, e->ent_ig.data(), e->ent_ig.size() * sizeof(int))) ||
                            (rc = h2d(e->d_zr, e->ent_zr.data(), e->ent_zr.size() * sizeof(int)))))) {
    release(e);
    delete e;
    return rc;
  }
  if (e->variant == 6) {
    rc = e->prec ? build_band_lists<double>(e) : build_band_lists<float>(e);
    if (rc) {
      release(e);
      delete e;
      return rc;
    }
  }
  if (e->variant == 3 || e->variant == 5) {
    rc = e->prec ? build_lists<double>(e) : build_lists<float>(e);
    if (rc) {
      release(e);
      delete e;
      return rc;
    }
  }
  // Entries never written by the kernels must read as zero: step 1 of the
  // seismograms (fdcore.f90 starts at it = 2), traces beyond ng(is), and the
  // strips of step 1 that the reconstruction inserts at it = 2.
  cudaError_t ce = cudaMemset(e->seis_t, 0, (size_t)ns * e->nt * ngm * e->esz);
  if (ce == cudaSuccess) ce = cudaMemset(e->d_err, 0, sizeof(int));
  if (ce == cudaSuccess) ce = cudaMemset(e->strips, 0, (size_t)ns * e->snt * e->SL * e->esz);
  if (ce == cudaSuccess) ce = cudaMemset(e->adj_t, 0, (size_t)ns * e->nt * ngm * e->esz);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&e->cap, cudaStreamNonBlocking);
  for (int i = 0; i < kCapStreamsMax - 1 && ce == cudaSuccess; ++i) {
    ce = cudaStreamCreateWithFlags(&e->capx[i], cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->ev_join[i], cudaEventDisableTiming);
  }
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&e->cpy, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->ev_in, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->ev_cpy, cudaEventDisableTiming);
  if (ce != cudaSuccess) {
    rc = fail(SWIT_E_CUDA, "engine initialisation: %s", cudaGetErrorString(ce));
    release(e);
    delete e;
    return rc;
  }
  const int waves = (ns + e->batch - 1) / e->batch;
  const int per = e->path == 1 ? ns : waves;
  const int per_step = e->variant == 2 ? 1 : 2;
  const int fwaves = e->path == 1 ? ns : (ns + fwd_batch(e) - 1) / fwd_batch(e);
  e->launches_fwd = (e->variant == 4 || e->variant == 5) ? fwaves : per * (e->nt - 1) * per_step;
  e->launches_bwd = e->variant == 4 ? per : per * (e->nt - 1) * per_step * (e->ckpt_k ? 2 : 1);
  *out = e;
  return 0;
}

int swit_set_model(swit_engine* e, const float* vp, const float* rho, int on_device, void* stream) {
  if (!e || !vp || !rho) return fail(SWIT_E_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = (size_t)e->nx * e->nz;
  std::vector<float> hv, hr;
  if (on_device) {
    hv.resize(n);
    hr.resize(n);
    CK(cudaMemcpyAsync(hv.data(), vp, n * sizeof(float), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hr.data(), rho, n * sizeof(float), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    vp = hv.data();
    rho = hr.data();
  }
  return e->prec ? set_model_impl<double>(e, vp, rho, st) : set_model_impl<float>(e, vp, rho, st);
}

int swit_forward(swit_engine* e, const float* src, void* seis, int save_boundary, int on_device, void* stream) {
  if (!e || !src) return fail(SWIT_E_ARG, "null argument");
  if (!e->model_set) return fail(SWIT_E_STATE, "swit_set_model must be called before swit_forward");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = e->prec ? forward_impl<double>(e, src, seis, save_boundary != 0, on_device, st)
                   : forward_impl<float>(e, src, seis, save_boundary != 0, on_device, st);
  if (rc) return rc;
  if (!on_device) CK(cudaStreamSynchronize(st));
  return 0;
}

int swit_backward(swit_engine* e, const float* adj, void* grad, void* illum_fw, void* illum_bk, int on_device,
                  void* stream) {
  if (!e || !adj) return fail(SWIT_E_ARG, "null argument");
  if (e->exact) return fail(SWIT_E_STATE, "the engine was created for the exact adjoint: use swit_backward_exact");
  if (!e->fwd_ready) return fail(SWIT_E_STATE, "swit_backward needs a preceding swit_forward with save_boundary=1");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = e->prec ? backward_impl<double>(e, adj, grad, illum_fw, illum_bk, on_device, st)
                   : backward_impl<float>(e, adj, grad, illum_fw, illum_bk, on_device, st);
  if (rc) return rc;
  if (!on_device) CK(cudaStreamSynchronize(st));
  return 0;
}

int swit_gradient_l2(swit_engine* e, const float* src, const float* obs, void* grad, void* illum_fw, void* illum_bk,
                     void* seis, double* misfit, int on_device, void* stream) {
  if (!e || !src || !obs) return fail(SWIT_E_ARG, "null argument");
  if (e->exact && (illum_fw || illum_bk))
    return fail(SWIT_E_ARG, "the exact adjoint computes no illumination: pass null illum_fw and illum_bk");
  if (!e->model_set) return fail(SWIT_E_STATE, "swit_set_model must be called before swit_gradient_l2");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = e->prec ? gradient_impl<double>(e, src, obs, grad, illum_fw, illum_bk, seis, misfit, on_device, st)
                   : gradient_impl<float>(e, src, obs, grad, illum_fw, illum_bk, seis, misfit, on_device, st);
  if (rc) return rc;
  if (!on_device) CK(cudaStreamSynchronize(st));
  return 0;
}

int swit_backward_exact(swit_engine* e, const float* adj, void* grad, void* src_grad, int on_device, void* stream) {
  if (!e || !adj) return fail(SWIT_E_ARG, "null argument");
  if (!e->exact) return fail(SWIT_E_STATE, "the engine was created with adjoint_mode 0 (fd2dmpi's adjoint)");
  if (!e->fwd_ready)
    return fail(SWIT_E_STATE, "swit_backward_exact needs a preceding swit_forward with save_boundary=1");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = e->prec ? exact_impl<double>(e, adj, grad, src_grad, on_device, st)
                   : exact_impl<float>(e, adj, grad, src_grad, on_device, st);
  if (rc) return rc;
  if (!on_device) CK(cudaStreamSynchronize(st));
  return 0;
}

int swit_export_snapshot(swit_engine* e, void* boundary, void* p_end, void* u_end, void* w_end, int on_device,
                         void* stream) {
  if (!e) return fail(SWIT_E_ARG, "null argument");
  if (e->exact) return fail(SWIT_E_STATE, "an exact-adjoint engine keeps no boundary strips");
  if (!e->fwd_ready) return fail(SWIT_E_STATE, "no saved forward run (swit_forward with save_boundary=1)");
  cudaStream_t st = (cudaStream_t)stream;
  return e->prec ? export_impl<double>(e, boundary, p_end, u_end, w_end, on_device, st)
                 : export_impl<float>(e, boundary, p_end, u_end, w_end, on_device, st);
}

int swit_import_snapshot(swit_engine* e, const float* src, const float* boundary, const float* p_end,
                         const float* u_end, const float* w_end, int on_device, void* stream) {
  if (!e || !src || !boundary || !p_end || !u_end || !w_end) return fail(SWIT_E_ARG, "null argument");
  if (!e->model_set) return fail(SWIT_E_STATE, "swit_set_model must be called before swit_import_snapshot");
  if (e->exact) return fail(SWIT_E_STATE, "an exact-adjoint engine keeps no boundary strips");
  cudaStream_t st = (cudaStream_t)stream;
  return e->prec ? import_impl<double>(e, src, boundary, p_end, u_end, w_end, on_device, st)
                 : import_impl<float>(e, src, boundary, p_end, u_end, w_end, on_device, st);
}

namespace {
// Read-modify-write sweeps over a buffer, loads and stores through L2 only
// (ld.global.cg / st.global.cg): every thread touches the same 16-byte words on
// every sweep, so a buffer that fits the L2 is served from it.
__global__ void k_l2_rmw(float4* __restrict__ a, size_t n, int reps) {
  for (int r = 0; r < reps; ++r)
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
      float4 v = __ldcg(a + i);
      v.x += 1.f;
      __stcg(a + i, v);
    }
}
}  // namespace

int swit_l2_bandwidth(int64_t bytes, int32_t reps, double* gbs, void* stream) {
  if (!gbs || bytes < (1 << 20) || reps < 1) return fail(SWIT_E_ARG, "bytes >= 1 MiB, reps >= 1 and gbs required");
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const size_t n = (size_t)bytes / 16;
  float4* a = nullptr;
  CK(cudaMalloc(&a, n * 16));
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaMemsetAsync(a, 0, n * 16, st);
  const int grid = sms * 8;
  k_l2_rmw<<<grid, 256, 0, st>>>(a, n, 2);  // brings the buffer into the L2
  cudaEventRecord(t0, st);
  k_l2_rmw<<<grid, 256, 0, st>>>(a, n, reps);
  cudaEventRecord(t1, st);
  cudaError_t ce = cudaEventSynchronize(t1);
  float ms = 0.f;
  if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(a);
  if (ce != cudaSuccess) return fail(SWIT_E_CUDA, "swit_l2_bandwidth: %s", cudaGetErrorString(ce));
  *gbs = 2.0 * (double)n * 16 * reps / (ms * 1e-3) / 1e9;
  return 0;
}

int swit_profile_kernels(swit_engine* e, int32_t launches[4], double mean_ms[4], void* stream) {
  if (!e || !launches || !mean_ms) return fail(SWIT_E_ARG, "null argument");
  if (e->exact) return fail(SWIT_E_STATE, "swit_profile_kernels times fd2dmpi's adjoint (adjoint_mode 0)");
  if (!e->model_set) return fail(SWIT_E_STATE, "swit_set_model must be called first");
  cudaStream_t st = (cudaStream_t)stream;
  return e->prec ? profile_impl<double>(e, launches, mean_ms, st) : profile_impl<float>(e, launches, mean_ms, st);
}

int swit_query(const swit_engine* e, int64_t* device_bytes, int32_t* shots_per_batch, int32_t* block_x,
               int32_t* kernels_per_forward, int32_t* kernels_per_backward, int32_t* kernel_variant,
               int32_t* graph_branches) {
  if (!e) return fail(SWIT_E_ARG, "null argument");
  if (graph_branches) *graph_branches = e->path == 1 ? 1 : std::min(e->branches, (e->ns + e->batch - 1) / e->batch);
  if (device_bytes) *device_bytes = (int64_t)e->bytes;
  if (shots_per_batch) *shots_per_batch = e->path == 1 ? 1 : e->batch;
  if (block_x) *block_x = e->bx;
  if (kernels_per_forward) *kernels_per_forward = e->launches_fwd;
  if (kernels_per_backward) *kernels_per_backward = e->launches_bwd;
  if (kernel_variant) *kernel_variant = e->variant;
  return 0;
}

int swit_check(swit_engine* e, void* stream) {
  if (!e) return fail(SWIT_E_ARG, "null engine");
  CK(cudaStreamSynchronize((cudaStream_t)stream));
  int w = 0;
  CK(cudaMemcpy(&w, e->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (w) {
    CK(cudaMemset(e->d_err, 0, sizeof(int)));
    return fail(SWIT_E_TIMEOUT, "a kernel gave up waiting for its staged copies (error word %d); results are invalid", w);
  }
  return 0;
}

int swit_misfit_l2(swit_engine* e, const float* src, const float* obs, double* misfit, int32_t on_device,
                   void* stream) {
  if (!e || !src || !obs || !misfit) return fail(SWIT_E_ARG, "null argument");
  if (!e->model_set) return fail(SWIT_E_STATE, "swit_set_model has not been called");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = e->prec ? forward_impl<double>(e, src, nullptr, false, on_device, st)
                   : forward_impl<float>(e, src, nullptr, false, on_device, st);
  if (rc) return rc;
  rc = e->prec ? residual_l2<double>(e, obs, on_device, st) : residual_l2<float>(e, obs, on_device, st);
  if (rc) return rc;
  return misfit_sum(e, st, misfit);
}

int swit_multi_create(const swit_desc* descs, int32_t n, swit_multi** out) {
  if (!descs || !out || n < 1) return fail(SWIT_E_ARG, "null argument or no instance");
  if (n > 65535) return fail(SWIT_E_LIMIT, "at most 65535 instances");
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    const swit_desc& d = descs[i];
    if (d.nx + 2 * d.npml > 16384 || d.ns > 65535) return fail(SWIT_E_LIMIT, "instance %d: more than 16384 PML-grid columns", i);
    if (d.precision != 0 || d.path != 0 || (d.kernel_variant != 0 && d.kernel_variant != 3) || d.checkpoint_every ||
        d.adjoint_mode || d.receiver_component)
      return fail(SWIT_E_ARG,
                  "instance %d: a multi-instance engine runs FP32 vec kernels on the batched path with boundary saving",
                  i);
  }
  swit_multi* m = new swit_multi();
  for (int i = 0; i < n; ++i) {
    swit_engine* e = nullptr;
    int rc = swit_create(&descs[i], &e);
    if (rc) {
      std::string msg = g_err;
      multi_release(m);
      delete m;
      return fail(rc, "instance %d: %s", i, msg.c_str());
    }
    m->eng.push_back(e);
  }
  int rc = multi_build(m);
  if (rc) {
    multi_release(m);
    delete m;
    return rc;
  }
  *out = m;
  return 0;
}

int swit_multi_engine(swit_multi* m, int32_t i, swit_engine** e) {
  if (!m || !e || i < 0 || i >= (int32_t)m->eng.size()) return fail(SWIT_E_ARG, "bad multi-instance handle or index");
  *e = m->eng[i];
  return 0;
}

int swit_multi_gradient_l2(swit_multi* m, const float* const* src, const float* const* obs, void* const* grad,
                           void* const* illum_fw, void* const* illum_bk, double* misfit, int32_t on_device,
                           void* stream) {
  if (!m || !src || !obs) return fail(SWIT_E_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int n = (int)m->eng.size();
  for (int i = 0; i < n; ++i)
    if (!m->eng[i]->model_set) return fail(SWIT_E_STATE, "instance %d: swit_set_model has not been called", i);
  for (int i = 0; i < n; ++i) {
    int rc = forward_impl<float>(m->eng[i], src[i], nullptr, true, on_device, st, false);
    if (rc) return rc;
  }
  const std::vector<int> all(n, 1);
  int rc = multi_loop(m, 1, all, st);
  if (rc) return rc;
  for (int i = 0; i < n; ++i) {
    if ((rc = residual_l2<float>(m->eng[i], obs[i], on_device, st))) return rc;
    if ((rc = backward_begin<float>(m->eng[i], st))) return rc;
  }
  if ((rc = multi_loop(m, 2, all, st))) return rc;
  for (int i = 0; i < n; ++i) {
    rc = backward_end<float>(m->eng[i], grad ? grad[i] : nullptr, illum_fw ? illum_fw[i] : nullptr,
                             illum_bk ? illum_bk[i] : nullptr, on_device, st);
    if (rc) return rc;
  }
  if (misfit)
    for (int i = 0; i < n; ++i)
      if ((rc = misfit_sum(m->eng[i], st, &misfit[i]))) return rc;
  return 0;
}

int swit_multi_misfit_l2(swit_multi* m, const float* const* src, const float* const* obs, const int32_t* active,
                         double* misfit, int32_t on_device, void* stream) {
  if (!m || !src || !obs || !misfit) return fail(SWIT_E_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int n = (int)m->eng.size();
  std::vector<int> on(n, 1);
  if (active)
    for (int i = 0; i < n; ++i) on[i] = active[i] ? 1 : 0;
  for (int i = 0; i < n; ++i)
    if (on[i] && !m->eng[i]->model_set)
      return fail(SWIT_E_STATE, "instance %d: swit_set_model has not been called", i);
  for (int i = 0; i < n; ++i) {
    if (!on[i]) continue;
    int rc = forward_impl<float>(m->eng[i], src[i], nullptr, false, on_device, st, false);
    if (rc) return rc;
  }
  int rc = multi_loop(m, 0, on, st);
  if (rc) return rc;
  for (int i = 0; i < n; ++i)
    if (on[i] && (rc = residual_l2<float>(m->eng[i], obs[i], on_device, st))) return rc;
  for (int i = 0; i < n; ++i) {
    misfit[i] = 0.0;
    if (on[i] && (rc = misfit_sum(m->eng[i], st, &misfit[i]))) return rc;
  }
  return 0;
}

int swit_multi_destroy(swit_multi* m) {
  if (!m) return 0;
  multi_release(m);
  delete m;
  return 0;
}

int swit_destroy(swit_engine* e) {
  if (!e) return 0;
  release(e);
  delete e;
  return 0;
}

int swit_damp_profile(int32_t nx, int32_t nz, int32_t npml, float dx, float vmin, float* out) {
  if (nx < 1 || nz < 1 || npml < 2 || !(dx > 0.f) || !out) return fail(SWIT_E_ARG, "bad argument");
  const int NX = nx + 2 * npml, NZ = nz + 2 * npml, L = npml;
  std::vector<float> damp(L + 1, 0.f);
  const float a = (float)(L - 1) * dx;
  const float kappa = 3.0f * vmin * (float)std::log(1000.0) / (2.0f * a);
  for (int i = 1; i <= L; ++i) {
    const float xa = (float)(i - 1) * dx / a;
    damp[i] = kappa * xa * xa;
  }
  for (int ix = 1; ix <= NX; ++ix)
    for (int iz = 1; iz <= NZ; ++iz) out[(size_t)(ix - 1) * NZ + (iz - 1)] = damp_at(damp.data(), iz, ix, L, NX, NZ);
  return 0;
}

}  // extern "C"
