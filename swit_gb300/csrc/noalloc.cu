// noalloc.cu -- single-shot forward modeling that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host application or plugin framework
// that owns all device memory through its own pool and forbids allocation once
// it runs, or a real-time loop that cannot afford the device-wide
// synchronisation cudaMalloc and cudaFree imply.  swit_forward_shot_static
// gives them the forward run of one shot with every intermediate array -- the
// three wavefields, the two update-coefficient arrays, the damping table and
// the receiver table -- in one file-scope static device array of fixed size
// (SWIT_STATIC_* in include/swit_gb300.h).  Every GPU that loads this library
// holds that array until the process exits.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress (in host code the array's name is only a host-side
// stand-in, not a device address) and caches it per device; make that first
// call before any stream capture.  All calls on a device share the array, which
// keeps the last call's contents: the wavefields are cleared at the start of
// every call, and calls that overlap on the GPU (different streams, or host
// threads) race on it.  No call waits on its stream: the receiver and source
// indices travel as kernel arguments, and the model check runs on the device
// (a model that fails it gives an all-NaN seismogram).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/swit_gb300.h"
#include "kernels.cuh"

namespace swit {
void set_last_error(const char* msg);  // engine.cu
}
using namespace swit;

namespace {

// Sizes of the static scratch (see SWIT_STATIC_* in the header).
constexpr int kMaxPoints = SWIT_STATIC_MAX_POINTS;        // NX x round_up(NZ, 32) per field
constexpr int kMaxColumns = SWIT_STATIC_MAX_COLUMNS;      // NX
constexpr int kMaxReceivers = SWIT_STATIC_MAX_RECEIVERS;  // ng
constexpr int kMaxPml = SWIT_STATIC_MAX_NPML;             // npml

// Layout of the scratch, in 4-byte words.
constexpr size_t kOffP = 0;
constexpr size_t kOffU = kOffP + kMaxPoints;
constexpr size_t kOffW = kOffU + kMaxPoints;
constexpr size_t kOffA = kOffW + kMaxPoints;
constexpr size_t kOffB = kOffA + kMaxPoints;
constexpr size_t kOffDamp = kOffB + kMaxPoints;               // damp(0..npml)
constexpr size_t kOffColptr = kOffDamp + kMaxPml + 1;         // colptr(0..NX+1)
constexpr size_t kOffIg = kOffColptr + kMaxColumns + 2;       // receiver number per entry
constexpr size_t kOffZr = kOffIg + kMaxReceivers;             // recording row per entry
constexpr size_t kOffGx = kOffZr + kMaxReceivers;             // receiver columns (set-up input)
constexpr size_t kOffGz = kOffGx + kMaxReceivers;             // receiver rows (set-up input)
constexpr size_t kOffSrc = kOffGz + kMaxReceivers;            // isx, isz, 0, 0
constexpr size_t kOffBad = kOffSrc + 4;                       // 1 if vp or rho is not finite and positive
constexpr size_t kWords = kOffBad + 4;

static __device__ __align__(256) float g_scratch[kWords];

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  set_last_error(buf);
  return code;
}

// Device address of g_scratch, looked up once per device.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
float* g_addr[kMaxDevices] = {};

int scratch_address(float** out) {
  int dev = 0;
  cudaError_t rc = cudaGetDevice(&dev);
  if (rc != cudaSuccess) return fail(SWIT_E_CUDA, "cudaGetDevice: %s", cudaGetErrorString(rc));
  if (dev < 0 || dev >= kMaxDevices) return fail(SWIT_E_LIMIT, "device %d beyond %d devices", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    rc = cudaGetSymbolAddress(&p, g_scratch);
    if (rc != cudaSuccess) return fail(SWIT_E_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(rc));
    g_addr[dev] = static_cast<float*>(p);
  }
  *out = g_addr[dev];
  return 0;
}

// Model set-up on the device: edge-replicated padding (fd2dmpi/io.f90:243-258,
// 280-292, which equals clamping the index to the interior), the update
// coefficients of fdcore.f90:79 and :99 in the reference's order, and zeroed
// wavefields.
__global__ void k_static_model(const float* __restrict__ vp, const float* __restrict__ rho, float* S, int nx, int nz,
                               int L, int NX, int NZ, int LD, float dt, float dx) {
  const int n = NX * LD;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int ix = t / LD + 1, iz = t - (ix - 1) * LD + 1;
    S[kOffP + t] = 0.f;
    S[kOffU + t] = 0.f;
    S[kOffW + t] = 0.f;
    float a = 0.f, b = 0.f;
    if (iz <= NZ) {
      const int jx = min(max(ix - L, 1), nx), jz = min(max(iz - L, 1), nz);
      const float c = vp[(size_t)(jx - 1) * nz + (jz - 1)];
      const float d = rho[(size_t)(jx - 1) * nz + (jz - 1)];
      a = d * c * c * dt / dx;
      b = dt / (d * dx);
    }
    S[kOffA + t] = a;
    S[kOffB + t] = b;
  }
}

// vmin below the free surface (fd2dmpi/math.f90:342-361 as called at
// solver.f90:73: interior rows 2..nz), the damping table (pml.f90:80-87) and
// the receiver table: receivers grouped by column in receiver order, the same
// table the batched engine builds on the host.
__global__ void k_static_tables(const float* __restrict__ vp, const float* __restrict__ rho, float* S, int nx,
                                int nz, int L, int NX, int ng, float dx, float l1000, int isx, int isz) {
  __shared__ float red[1024];
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  float m = 10000000000.0f;
  int mine = 0;
  for (int t = threadIdx.x; t < nx * nz; t += blockDim.x) {
    const float v = vp[t], d = rho[t];
    // finite and positive, as the engine's model set-up requires (NaN fails both)
    if (!(v > 0.f && v <= 3.402823466e38f) || !(d > 0.f && d <= 3.402823466e38f)) mine = 1;
    const int jz = t % nz + 1;
    if (jz > 1) m = fminf(m, v);
  }
  if (mine) bad = 1;  // benign race: every writer stores 1
  red[threadIdx.x] = m;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] = fminf(red[threadIdx.x], red[threadIdx.x + h]);
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  reinterpret_cast<int*>(S + kOffSrc)[0] = isx;
  reinterpret_cast<int*>(S + kOffSrc)[1] = isz;
  reinterpret_cast<int*>(S + kOffSrc)[2] = 0;
  reinterpret_cast<int*>(S + kOffSrc)[3] = 0;
  reinterpret_cast<int*>(S + kOffBad)[0] = bad;
  const float vmin = red[0];
  const float a = (float)(L - 1) * dx;
  const float kappa = 3.0f * vmin * l1000 / (2.0f * a);
  float* damp = S + kOffDamp;
  damp[0] = 0.f;
  for (int i = 1; i <= L; ++i) {
    const float xa = (float)(i - 1) * dx / a;
    damp[i] = kappa * xa * xa;
  }
  int* colptr = reinterpret_cast<int*>(S + kOffColptr);
  int* ig = reinterpret_cast<int*>(S + kOffIg);
  int* zr = reinterpret_cast<int*>(S + kOffZr);
  const int* gx = reinterpret_cast<const int*>(S + kOffGx);
  const int* gz = reinterpret_cast<const int*>(S + kOffGz);
  for (int c = 0; c <= NX + 1; ++c) colptr[c] = 0;
  for (int r = 0; r < ng; ++r) colptr[gx[r] + 1] += 1;  // counts shifted by one column
  for (int c = 1; c <= NX + 1; ++c) colptr[c] += colptr[c - 1];
  // colptr[c] now holds the first entry of column c; fill in receiver order
  for (int r = 0; r < ng; ++r) {
    const int e = colptr[gx[r]]++;
    ig[e] = r;
    zr[e] = gz[r];
  }
  for (int c = NX + 1; c >= 1; --c) colptr[c] = colptr[c - 1];  // undo the advance
  colptr[0] = 0;
}

// The velocity phase of the forward step (k_fwd_uw in kernels.cuh) for one
// shot, writing the seismogram straight into the caller's (ng, nt) array and
// keeping no boundary strips.
__global__ void __launch_bounds__(256) k_static_uw(Grid<float> g, Receivers rec, const float* __restrict__ P,
                                                   float* U, float* W, float* __restrict__ seis, int it) {
  const int iz = blockIdx.x * 32 + threadIdx.x + 1;
  const int ix = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (iz > g.NZ || ix > g.NX) return;
  const int LD = g.LD, L = g.L, NX = g.NX, NZ = g.NZ, fs = g.fs;
  const size_t k = (size_t)(ix - 1) * LD + (iz - 1);
  float uv = U[k], wv = W[k];
  if (ix >= 2 && ix <= NX - 2 && iz >= fs && iz <= NZ - 1) {
    const float alpha = g.B[k];
    const float kappa =
        0.5f * (damp_at(g.damp, iz, ix, L, NX, NZ) + damp_at(g.damp, iz, ix + 1, L, NX, NZ)) * g.dt;
    uv = (1.0f - kappa) * uv - alpha * (g.c1 * (P[k + LD] - P[k]) + g.c2 * (P[k + 2 * LD] - P[k - LD]));
    U[k] = uv;
  }
  if (ix >= 2 && ix <= NX - 1 && iz >= fs && iz <= NZ - 2) {
    const float alpha = g.B[k];
    const float kappa =
        0.5f * (damp_at(g.damp, iz, ix, L, NX, NZ) + damp_at(g.damp, iz + 1, ix, L, NX, NZ)) * g.dt;
    wv = (1.0f - kappa) * wv - alpha * (g.c1 * (P[k + 1] - P[k]) + g.c2 * (P[k + 2] - P[k - 1]));
    W[k] = wv;
  }
  if (g.fs_flag == 1 && iz == fs) W[k - 1] = wv;
  for (int e = rec.colptr[ix]; e < rec.colptr[ix + 1]; ++e)
    if (rec.zrow[e] == iz) seis[(size_t)rec.ig[e] * g.nt + (it - 1)] = P[k];
}

// Receiver grid indices of receivers [r0, r0 + n), n <= kChunk, passed by value
// so that the call stages nothing through host memory.
constexpr int kChunk = 256;
struct IndexChunk {
  int gx[kChunk];
  int gz[kChunk];
};
__global__ void k_static_put_indices(float* S, int r0, int n, IndexChunk c) {
  const int r = threadIdx.x;
  if (r >= n) return;
  reinterpret_cast<int*>(S + kOffGx)[r0 + r] = c.gx[r];
  reinterpret_cast<int*>(S + kOffGz)[r0 + r] = c.gz[r];
}

// A model that failed the finite-and-positive check gives an all-NaN
// seismogram: the check runs on the device, so the call itself cannot report it.
__global__ void k_static_poison(const float* S, float* seis, size_t n) {
  if (reinterpret_cast<const int*>(S + kOffBad)[0] == 0) return;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    seis[t] = __int_as_float(0x7fc00000);
}

__global__ void k_static_zero_first(float* seis, int ng, int nt) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < ng; r += gridDim.x * blockDim.x) seis[(size_t)r * nt] = 0.f;
}

inline int round_up(int a, int m) { return (a + m - 1) / m * m; }

}  // namespace

extern "C" int swit_forward_shot_static(int32_t nx, int32_t nz, int32_t npml, int32_t nt, float dx, float dt,
                                        int32_t free_surface, float src_x, float src_z, int32_t ng,
                                        const float* rec_x, const float* rec_z, const float* vp, const float* rho,
                                        const float* src, float* seis, void* stream) {
  // sizes first: nothing touches the GPU for a request that cannot fit
  if (nx < 8 || nz < 8 || npml < 2 || nt < 2 || ng < 1 || !(dx > 0.f) || !(dt > 0.f))
    return fail(SWIT_E_ARG, "bad size (nx=%d nz=%d npml=%d nt=%d ng=%d)", nx, nz, npml, nt, ng);
  if (!rec_x || !rec_z || !vp || !rho || !src || !seis) return fail(SWIT_E_ARG, "null argument");
  const int NX = nx + 2 * npml, NZ = nz + 2 * npml, LD = round_up(NZ, 32);
  if ((long long)NX * LD > kMaxPoints || NX > kMaxColumns || ng > kMaxReceivers || npml > kMaxPml)
    return fail(SWIT_E_LIMIT,
                "swit_forward_shot_static holds at most %d padded grid points, %d columns, %d receivers and "
                "npml %d (got %lld points, %d columns, %d receivers, npml %d)",
                kMaxPoints, kMaxColumns, kMaxReceivers, kMaxPml, (long long)NX * LD, NX, ng, npml);
  // geometry, exactly as the batched engine (fdcore.f90:70-72, 124-126)
  auto inside = [&](float x, int n) { return x >= -0.0f && (int)(x / dx) <= n - 1; };
  if (!inside(src_x, nx) || !inside(src_z, nz))
    return fail(SWIT_E_GEOM, "source at (%g, %g) m is outside the model", src_x, src_z);
  for (int r = 0; r < ng; ++r)
    if (!inside(rec_x[r], nx) || !inside(rec_z[r], nz))
      return fail(SWIT_E_GEOM, "receiver %d at (%g, %g) m is outside the model", r + 1, rec_x[r], rec_z[r]);
  float* S = nullptr;
  int rc = scratch_address(&S);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int fs = npml + 1;
  // receiver and source grid indices: computed here, handed to the device as
  // kernel arguments (no host staging buffer, no wait on the stream)
  for (int r0 = 0; r0 < ng; r0 += kChunk) {
    const int n = ng - r0 < kChunk ? ng - r0 : kChunk;
    IndexChunk c;
    for (int r = 0; r < n; ++r) {
      c.gx[r] = npml + (int)(rec_x[r0 + r] / dx) + 1;
      const int igz = npml + (int)(rec_z[r0 + r] / dx) + 1;
      c.gz[r] = igz == fs ? igz + 1 : igz;
    }
    k_static_put_indices<<<1, kChunk, 0, st>>>(S, r0, n, c);
  }
  const int isx = npml + (int)(src_x / dx) + 1;
  int isz = npml + (int)(src_z / dx) + 1;
  if (isz == fs) isz += 1;

  k_static_model<<<152 * 4, 256, 0, st>>>(vp, rho, S, nx, nz, npml, NX, NZ, LD, dt, dx);
  k_static_tables<<<1, 1024, 0, st>>>(vp, rho, S, nx, nz, npml, NX, ng, dx, (float)std::log(1000.0), isx, isz);
  k_static_zero_first<<<(ng + 255) / 256, 256, 0, st>>>(seis, ng, nt);

  Grid<float> g;
  g.nx = nx;
  g.nz = nz;
  g.L = npml;
  g.NX = NX;
  g.NZ = NZ;
  g.LD = LD;
  g.LDI = 0;
  g.fs = fs;
  g.fs_flag = free_surface == 1 ? 1 : 0;
  g.nt = nt;
  g.ngmax = ng;
  g.SL = 0;
  g.snt = nt;
  g.sit0 = 1;
  g.FSZ = 0;  // one shot
  g.FSI = 0;
  g.IL = 0;
  g.dt = dt;
  g.c1 = 9.0f / 8.0f;
  g.c2 = -1.0f / 24.0f;
  g.A = S + kOffA;
  g.B = S + kOffB;
  g.damp = S + kOffDamp;
  const int* si = reinterpret_cast<const int*>(S + kOffSrc);
  Sources sr{si, si + 1, si + 2, si + 3};
  Receivers rec{reinterpret_cast<const int*>(S + kOffColptr), reinterpret_cast<const int*>(S + kOffIg),
                reinterpret_cast<const int*>(S + kOffZr)};
  // the forward source as the pressure phase reads it: s(it) at src[it-1]
  // with a stride of nt+1 per shot; one shot, so the stride is never used
  const dim3 block(32, 4), grid((NZ + 31) / 32, (NX + 3) / 4, 1);
  for (int it = 2; it <= nt; ++it) {
    k_fwd_p<float><<<grid, block, 0, st>>>(g, sr, src, S + kOffP, S + kOffU, S + kOffW, it, 0);
    k_static_uw<<<grid, block, 0, st>>>(g, rec, S + kOffP, S + kOffU, S + kOffW, seis, it);
  }
  k_static_poison<<<152, 256, 0, st>>>(S, seis, (size_t)ng * nt);
  const cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return fail(SWIT_E_CUDA, "launch: %s", cudaGetErrorString(ce));
  return 0;
}
