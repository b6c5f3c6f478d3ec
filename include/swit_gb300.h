/*
 * swit_gb300.h -- C ABI of the GB300 forward/adjoint wave-propagation engine.
 *
 * The engine is a drop-in for the computational core behind SWIT's
 * toolbox/solver.py forward() and adjoint() calls.  In the reference those calls
 * cross a process boundary (`mpirun fd2dmpi par=<parfile>`, toolbox/solver.py:54
 * and :79) and exchange files; here the same work is a library call with plain
 * pointers.  Each entry point below names the reference code it replaces.
 *
 * Conventions (identical to the reference's Python side and Fortran files):
 *   - every 2-D array is z-fastest: model and gradient (nx, nz), i.e. nx records
 *     of nz floats (toolbox/solver.py:116-119, fd2dmpi/io.f90:590-606);
 *   - sources (ns, nt); seismograms and adjoint sources (ns, ng_max, nt), one
 *     trace of nt samples per receiver (fd2dmpi/fdcore.f90:123-128, 181-188;
 *     toolbox/solver.py:112-113 with fd2dmpi/solver.f90:218);
 *   - coordinates are in metres, as in coord.txt (toolbox/solver.py:171-180);
 *     grid indices are npml + int(x/dx) + 1 in single precision
 *     (fd2dmpi/fdcore.f90:70-72, 124-126).
 *   - FP32 engines read and write float; FP64 engines (the FP64 build of the
 *     same kernels, used to state the error of FP32 results) read float inputs
 *     and write double outputs through the same void* parameters.
 *
 * Every call returns 0 on success or a negative SWIT_E_* code; the message of
 * the last failure on the calling thread is swit_last_error().  Buffers are
 * owned by the caller; the engine owns its device workspace (wavefields,
 * boundary strips, seismogram staging).  One engine must not be used from two
 * threads at once.  `on_device` = 1 means every array argument is a device
 * pointer and the call is stream-ordered on `stream` (no host synchronisation);
 * 0 means host arrays, copied inside the call, which returns when the outputs
 * are written.
 */
#ifndef SWIT_GB300_H
#define SWIT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWIT_OK 0
#define SWIT_E_ARG -1      /* invalid argument (null pointer, bad size)          */
#define SWIT_E_GEOM -2     /* source/receiver outside the model                  */
#define SWIT_E_CFL -3      /* dt violates dt < sqrt(3/8) dx / vmax               */
#define SWIT_E_MODEL -4    /* non-finite or non-positive vp / rho                */
#define SWIT_E_STATE -5    /* call out of order (e.g. backward before forward)   */
#define SWIT_E_CUDA -6     /* CUDA runtime error                                 */
#define SWIT_E_NOMEM -7    /* device allocation failed                           */
#define SWIT_E_LIMIT -8    /* problem larger than a fixed capacity               */
#define SWIT_E_TIMEOUT -9  /* a kernel stopped waiting on an in-kernel copy      */

typedef struct swit_engine swit_engine;

/* Problem description: the parfile keys NX, NZ, NPML, NT_WORK, DX, DT_WORK,
 * FREESURFACE (fd2dmpi/io.f90:74-96) and the coord.txt geometry
 * (fd2dmpi/io.f90:126-228). */
typedef struct swit_desc {
  int32_t nx, nz, npml, nt;
  float dx, dt;
  int32_t free_surface;     /* FREESURFACE, 1 = mirror conditions on           */
  int32_t ns;               /* number of shots                                  */
  int32_t ng_max;           /* receivers per shot, maximum                      */
  const int32_t* ng;        /* [ns] receivers of each shot                       */
  const float* src_x;       /* [ns]                                              */
  const float* src_z;       /* [ns]                                              */
  const float* rec_x;       /* [ns * ng_max]                                     */
  const float* rec_z;       /* [ns * ng_max]                                     */
  int32_t precision;        /* 0 = FP32 (default), 1 = FP64 build of the kernels */
  int32_t path;             /* 0 = batched shots + captured CUDA graph (default),
                               1 = plain: one shot per launch, one launch per
                               kernel and step, no graph                          */
  int32_t shots_per_batch;  /* batched path: shots per launch, 0 = automatic
                               (vec kernels: as many shots in flight as keep the
                               reverse loop's state in L2, spread evenly over
                               the graph branches; other kernels: all shots)    */
  int32_t block_x;          /* columns per CTA, 0 = automatic: split kernels
                               1, 2, 4 or 8 (x 32 rows); walk kernels: columns
                               per tile, 2..256 (default 8); vec kernels: task lists
                               ordered by tiles of block_x columns (a power of
                               two <= 64, default 4) x 256/block_x four-row
                               vectors;
                               cluster kernels: CTAs per cluster 1..16 (default
                               16; the reverse loop takes more CTAs when its six
                               wavefields need them)                            */
  int32_t kernel_variant;   /* 0 = automatic (vec), 1 = split: two kernels per step,
                               in place, one point per thread; 2 = walk: one
                               kernel per step, double-buffered, each warp
                               walking a tile of columns with the x-neighbours
                               in registers and the z-neighbours by shuffle;
                               3 = vec: split, four rows per thread;
                               4 = cluster: one launch per time loop, one
                               thread-block cluster per shot holding its
                               wavefields in distributed shared memory
                               (SWIT_E_LIMIT when they do not fit); 5 = hybrid:
                               cluster forward loop (all shots in one launch),
                               vec reverse loop (block_x = cluster size);
                               6 = band: the vec bodies on bands of block_x
                               columns (0 = as many as 256 threads cover) staged
                               through shared memory by bulk copies            */
  int32_t checkpoint_every; /* 0 = boundary saving (fd2dmpi's strategy: strips of
                               every step, ns*nt*(9nx+6nz) values); k > 0 =
                               checkpointed recomputation (vec and band kernels):
                               the forward keeps the full state every k steps, the
                               reverse loop re-runs each k-step segment from its
                               checkpoint to regenerate that segment's strips.
                               Same results bit for bit; about one more forward
                               pass of work; export/import of snapshots and
                               swit_profile_kernels need k = 0                 */
  int32_t graph_branches;   /* batched path: the shot batches' step chains form
                               this many concurrent branches of the captured
                               graphs (batch b on branch b mod graph_branches);
                               0 = automatic (3 with automatic shots_per_batch,
                               else 2), at most 4                               */
  int32_t adjoint_mode;     /* 0 = fd2dmpi's adjoint (boundary strips, reverse
                               reconstruction, continuous-adjoint imaging:
                               swit_backward); 1 = exact discrete adjoint of the
                               forward map (vec kernels; the forward stores the
                               divergence term of every step, NX*LD values per
                               step and shot, or regenerates them segment by
                               segment with checkpoint_every: swit_backward_exact) */
  int32_t receiver_component; /* 0 = pressure (fd2dmpi); 1 = vx, 2 = vz: the
                               receivers record u or w and the adjoint source
                               enters u or w (dev/solver/fdcore.f90:154-177,
                               465-485; vec kernels; with adjoint_mode 1 the
                               exact transpose of that recording)           */
} swit_desc;

/* Creates an engine and allocates its device workspace on the current device.
 * Replaces the setup half of fd2dmpi/solver.f90:36-91 and :120-192
 * (readparamfile, init_pml, readcoordfile, free_surface) -- the model itself is
 * given by swit_set_model. */
int swit_create(const swit_desc* desc, swit_engine** out);

/* Sets vp and rho, (nx, nz) each.  Pads them into the PML by edge replication
 * (fd2dmpi/io.f90:231-300), finds vmin below the free surface
 * (fd2dmpi/math.f90:342-361), builds the damping profile
 * (fd2dmpi/pml.f90:74-101) and the update coefficients of
 * fd2dmpi/fdcore.f90:79, 99, 312, 339.  Checks the CFL condition of
 * toolbox/base.py:42, 58-59. */
int swit_set_model(swit_engine* e, const float* vp, const float* rho, int on_device, void* stream);

/* Forward modeling of every shot: fd2dmpi/fdcore.f90:30-198 driven by
 * fd2dmpi/solver.f90:93-104 (jobtype=forward_modeling).  src is the already
 * integrated source (toolbox/solver.py:47), (ns, nt).  seis receives the
 * pressure seismograms (ns, ng_max, nt); traces beyond ng(is) are zero.
 * save_boundary = 1 keeps the boundary strips and final wavefields on the
 * device for swit_backward (STORE_SNAP=1, fdcore.f90:130-177). */
int swit_forward(swit_engine* e, const float* src, void* seis, int save_boundary, int on_device, void* stream);

/* Reverse-time loop of every shot: wavefield reconstruction from the saved
 * strips (fd2dmpi/fdcore.f90:202-289), adjoint propagation of the adjoint
 * sources adj (ns, ng_max, nt) (fdcore.f90:293-375), zero-lag imaging and
 * illumination (fd2dmpi/solver.f90:230-253), the shot sum and the -2/c scale
 * (solver.f90:263-270) -- jobtype=adjoint_modeling.  Writes the raw vp kernel
 * grad, illum_fw and illum_bk, (nx, nz) each: the contents of
 * src0_kernel_vp.bin, src0_illum_forw.bin, src0_illum_back.bin.  Needs a
 * preceding swit_forward with save_boundary = 1 on the same model. */
int swit_backward(swit_engine* e, const float* adj, void* grad, void* illum_fw, void* illum_bk, int on_device,
                  void* stream);

/* One Waveform-misfit (L2) shot-gradient of every shot in a single call:
 * forward with strips, the adjoint source syn - obs of every live trace
 * (toolbox/misfit.py:128-148), the misfit sum_traces sqrt(sum r^2 dt)
 * (toolbox/misfit.py:263-282), then the reverse loop as swit_backward.  obs is
 * (ns, ng_max, nt).  seis (optional, may be NULL) receives the synthetics.
 * misfit (optional) receives one double. */
int swit_gradient_l2(swit_engine* e, const float* src, const float* obs, void* grad, void* illum_fw,
                     void* illum_bk, void* seis, double* misfit, int on_device, void* stream);

/* Copies the boundary strips of the last forward run in the reference's
 * boundary.bin layout, (ns, nt, 9 nx + 6 nz) (fdcore.f90:130-159, 169-170), and
 * the final interior wavefields p_end, u_end, w_end, (ns, nx, nz) each
 * (fdcore.f90:162-176).  Any output may be NULL. */
int swit_export_snapshot(swit_engine* e, void* boundary, void* p_end, void* u_end, void* w_end, int on_device,
                         void* stream);

/* Loads a saved forward run instead of computing one: the forward source
 * (ns, nt), the boundary strips in boundary.bin layout (ns, nt, 9 nx + 6 nz) and
 * the final interior wavefields p_end, u_end, w_end (ns, nx, nz) -- the inputs
 * fd2dmpi's adjoint job reads from parfile/forward_source and
 * <DATA_OUT>N_snapshot/ (fd2dmpi/solver.f90:212-228).  A following
 * swit_backward then needs no swit_forward.  Inputs are float in both
 * precisions (the reference's file format). */
int swit_import_snapshot(swit_engine* e, const float* src, const float* boundary, const float* p_end,
                         const float* u_end, const float* w_end, int on_device, void* stream);

/* No counterpart in the reference: a measurement utility for the roofline of
 * the stencil kernels, whose per-step state stays in the L2.  Times `reps`
 * read-modify-write sweeps (16-byte words, loads and stores through L2 only)
 * over a device buffer of `bytes` bytes (allocated and freed here) on `stream`
 * and returns the bytes read plus written per second in GB/s; a buffer well
 * under the L2 size (e.g. 64 MiB of the GB300's 126 MB) gives the L2 bandwidth.
 * Synchronises the stream. */
int swit_l2_bandwidth(int64_t bytes, int32_t reps, double* gbs, void* stream);

/* Profiling hook (the reference has none; fd2dmpi only prints banners,
 * fd2dmpi/solver.f90:78-84).  For each stencil kernel -- [0] forward pressure
 * phase, [1] forward velocity phase, [2] backward velocity phase, [3] backward
 * pressure phase -- returns the number of launches timed and the mean time per
 * launch in milliseconds.  Batched vec engines time each kernel under the
 * conditions of the captured loop: one graph of that kernel alone, min(nt-1,
 * 256) steps of every batch on the graph branches, CUDA events around one
 * replay, so mean_ms x (batches per step) is the kernel's time per step and the
 * four add up to about the loop's.  Other engines launch every kernel of a
 * forward and reverse loop with an event pair around it.  With the walk
 * variant, [0] is the forward step kernel, [2] the reverse step kernel and [1],
 * [3] are unused (0 launches).  Leaves the wavefields undefined until the next
 * forward run; synchronises the stream. */
int swit_profile_kernels(swit_engine* e, int32_t launches[4], double mean_ms[4], void* stream);

/* Capacity of swit_forward_shot_static's fixed scratch (about 2.7 MB per GPU). */
#define SWIT_STATIC_MAX_POINTS 131072 /* (nx + 2 npml) x round_up(nz + 2 npml, 32) */
#define SWIT_STATIC_MAX_COLUMNS 4096  /* nx + 2 npml                             */
#define SWIT_STATIC_MAX_RECEIVERS 4096
#define SWIT_STATIC_MAX_NPML 256

/* No counterpart in the reference.  Forward modeling of ONE shot that
 * allocates no device memory, for callers that cannot call cudaMalloc: a host
 * framework or plugin host that owns all device memory through its own pool, or
 * a loop that cannot afford the device-wide synchronisation of cudaMalloc and
 * cudaFree.  Its wavefields, coefficients and receiver table live in one
 * file-scope static device array of fixed size (SWIT_STATIC_*; every GPU that
 * loads this library holds it until the process exits); larger problems are
 * rejected with SWIT_E_LIMIT before any GPU work.  vp, rho (nx, nz), src (nt)
 * and seis (ng, nt) are DEVICE arrays; rec_x, rec_z (ng) are host arrays.
 * Results equal swit_forward's for the same shot, bit for bit.  The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress)
 * -- make it before any stream capture.  The wavefields are cleared on every
 * call; all calls on a device share the array, so calls that overlap on the GPU
 * race.  The call is ordered on `stream` and returns once the launches are
 * queued: receiver and source indices reach the device as kernel arguments, and
 * the call never waits on the stream.  Because the model stays on the device,
 * the call cannot report a bad one: a vp or rho value that is not finite and
 * positive makes the whole seismogram NaN (swit_forward returns SWIT_E_MODEL
 * instead), and dt is not checked against the CFL limit. */
int swit_forward_shot_static(int32_t nx, int32_t nz, int32_t npml, int32_t nt, float dx, float dt,
                             int32_t free_surface, float src_x, float src_z, int32_t ng, const float* rec_x,
                             const float* rec_z, const float* vp, const float* rho, const float* src, float* seis,
                             void* stream);

/* Sizes and launch configuration the engine has chosen (graph_branches: the
 * concurrent branches its graphs use); any pointer may be NULL. */
int swit_query(const swit_engine* e, int64_t* device_bytes, int32_t* shots_per_batch, int32_t* block_x,
               int32_t* kernels_per_forward, int32_t* kernels_per_backward, int32_t* kernel_variant,
               int32_t* graph_branches);

/* Exact discrete adjoint (engines created with adjoint_mode = 1) after a
 * swit_forward with save_boundary = 1: the transpose of the forward map applied
 * to adjoint sources adj (ns, ng_max, nt) = dJ/dseis.
 *   grad     (nx, nz): dJ/dvp, the damping profile held fixed (it depends on vp
 *            only through vmin, pml.f90:80); exact for perturbations that keep
 *            vmin, e.g. <J dvp, adj> = <dvp, grad> to rounding.
 *   src_grad (ns, nt): dJ/dsrc for the source functions given to swit_forward.
 * Either output may be NULL; types and placement as swit_backward's.  Not a
 * reference algorithm: fd2dmpi's own gradient is swit_backward's. */
int swit_backward_exact(swit_engine* e, const float* adj, void* grad, void* src_grad, int32_t on_device,
                        void* stream);

/* Waits for `stream` and reports whether any kernel of the engine gave up
 * waiting for the copies it stages into shared memory (band variant: every such
 * wait is bounded, and a block that times out skips its update).  Returns
 * SWIT_E_TIMEOUT once for such an event, then clears it.  No counterpart in the
 * reference, whose CPU loops have no asynchronous copies. */
int swit_check(swit_engine* e, void* stream);

/* The Waveform misfit of swit_gradient_l2 alone: a forward run without strips,
 * then the same per-trace sums (misfit.py:128-148), for line-search trials
 * (inversion.py:274-350 evaluates misfits only).  Waits for the stream. */
int swit_misfit_l2(swit_engine* e, const float* src, const float* obs, double* misfit, int32_t on_device,
                   void* stream);

/* ---- Many independent problems in one set of launches --------------------
 * A multi-instance engine holds n regular engines (one swit_desc each: FP32,
 * batched path, vec kernels, boundary saving; grids, shot counts and nt may all
 * differ) and steps them together: the (instance, shot) pairs are grouped
 * into L2-sized waves (an instance's own shots, or several small instances),
 * and per wave each time step launches the phase kernels once over every pair
 * still running; the waves run on concurrent branches, and a call runs only
 * the waves holding a switched-on instance (swit_multi_misfit_l2's `active`).
 * Waves beyond a graph node budget are launched step by step, so a call with
 * many of them returns only once most of their launches are queued (the host
 * waits for room in the launch queues).  The reference runs one
 * fd2dmpi job per problem; this has no counterpart there.  Models are set per
 * instance through the handles of swit_multi_engine, which stay owned by the
 * multi-instance engine. */
typedef struct swit_multi swit_multi;

int swit_multi_create(const swit_desc* descs, int32_t n, swit_multi** out);

/* Borrowed handle of instance i (caller order) for swit_set_model, swit_query,
 * or single-instance calls. */
int swit_multi_engine(swit_multi* m, int32_t i, swit_engine** e);

/* swit_gradient_l2 for every instance: src[i] (ns_i, nt_i), obs[i]
 * (ns_i, ng_max_i, nt_i) float; grad[i], illum_fw[i], illum_bk[i] (nx_i, nz_i),
 * any array or entry may be NULL; misfit[i] on the host (waits), or misfit
 * NULL.  Every instance gets the bits its own engine's swit_gradient_l2 gives. */
int swit_multi_gradient_l2(swit_multi* m, const float* const* src, const float* const* obs, void* const* grad,
                           void* const* illum_fw, void* const* illum_bk, double* misfit, int32_t on_device,
                           void* stream);

/* Waveform misfit of the instances with active[i] != 0 (all if active is NULL;
 * the others do no work and get 0): forward runs only, no strips; misfit[n] on
 * the host (waits).  src[i], obs[i] of inactive instances are not read. */
int swit_multi_misfit_l2(swit_multi* m, const float* const* src, const float* const* obs, const int32_t* active,
                         double* misfit, int32_t on_device, void* stream);

int swit_multi_destroy(swit_multi* m);

/* Releases the engine and its device memory. */
int swit_destroy(swit_engine* e);

/* Message of the last failed call on this thread ("" if none). */
const char* swit_last_error(void);

/* Host-only helper (no GPU needed): writes the damping profile damp_global
 * (NZ, NX) that the kernels evaluate in closed form, z-fastest [NX][NZ], for a
 * given vmin.  Lets tests compare it with fd2dmpi/pml.f90:74-101. */
int swit_damp_profile(int32_t nx, int32_t nz, int32_t npml, float dx, float vmin, float* out);

#ifdef __cplusplus
}
#endif

#endif /* SWIT_GB300_H */
