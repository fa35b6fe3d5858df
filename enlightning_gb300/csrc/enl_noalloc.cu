// Stable time step of one patch without any device allocation.
//
// enl_cfl_dt_static computes, for one patch in SAMRAI CellData layout, the
// same time step as the engine's device CFL reduction (speed_kernel +
// dt_kernel in enl_engine.cu):
//   dt = min(dt_max, cfl * dx_min / max over the interior of max(|u|,|v|) + c)
// The engine keeps its reduction word in memory it allocates with
// cudaMalloc.  Some callers cannot allocate device memory at the point where
// they need a time step: a host framework whose device memory is owned by a
// pool allocator (SAMRAI patch data behind an Umpire pool, for instance) or
// that runs under a fixed memory budget during a time step, and code that
// must not call cudaMalloc/cudaFree because those calls can synchronise the
// whole device.  This entry point therefore uses a file-scope static device
// array for its per-block partial maxima; the caller passes only the patch
// and the output.
//
// Limits and sharing:
//   * the scratch holds kScratchBlocks partial maxima, one per 32x8 tile, so
//     a patch may have at most kScratchBlocks tiles (kScratchBlocks * 256 =
//     1,048,576 interior cells); larger patches are rejected with
//     ENL_ERR_ARG and a message on stderr;
//   * every GPU that loads the library holds the array (32 KB) until the
//     process exits;
//   * all calls share the array: every call writes the partials it reads, so
//     nothing needs clearing between calls, but calls that overlap on the GPU
//     (different streams, or two host threads) race on it;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current); make that first call
//     before any stream capture.  The address is cached per device together
//     with the id of the context it belongs to; a new context on the device
//     (after cudaDeviceReset) makes the next call look it up again, and so
//     does a failed launch.
//
// A non-finite or non-positive density anywhere in the interior is not
// turned into a speed: the partial of that tile is -1, and the final kernel
// then writes a quiet NaN to dt_out (never a small finite step), which the
// caller sees wherever it uses the step.  The engine reports the same state
// as ENL_ERR_NONFINITE through its health word.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdio>

#include "enl_common.cuh"

namespace enl {

constexpr int kScratchBlocks = 4096;
constexpr int kMaxDevices = 64;

// Per-block partial maxima of the speed.  Host code must not use this name
// as a device address (in host code it is a host-side stand-in); the address
// comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_cfl_partials[kScratchBlocks];

static double* g_partials_addr[kMaxDevices] = {nullptr};
static unsigned long long g_partials_ctx[kMaxDevices] = {0};

__global__ void cfl_partial_kernel(const double* __restrict__ w, long pitch, long fstride, int g0, int g1, int nx,
                                   int ny, double c, double* partials) {
  __shared__ double s_w[8];
  const int tiles_x = (nx + 31) / 32;
  const int tx0 = (blockIdx.x % tiles_x) * 32, ty0 = (blockIdx.x / tiles_x) * 8;
  const int ci = tx0 + (threadIdx.x & 31), cj = ty0 + (threadIdx.x >> 5);
  __shared__ int s_bad;
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  double m = 0.0;
  if (ci < nx && cj < ny) {
    long g = (long)(cj + g1) * pitch + (ci + g0);
    double r = w[g];
    m = fmax(fabs(w[fstride + g] / r), fabs(w[2 * fstride + g] / r)) + c;
    // fmax drops NaN operands, so a bad cell is flagged on its own
    if (!(r > 0.0) || !isfinite(r) || !isfinite(m)) s_bad = 1;
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < 8 ? s_w[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) partials[blockIdx.x] = s_bad ? -1.0 : m;
  }
}

__global__ void cfl_final_kernel(const double* partials, int n, double cfl_dxmin, double dt_max, double* dt_out) {
  __shared__ double s_w[8];
  double m = 0.0;
  int bad = 0;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const double v = partials[q];
    bad |= v < 0.0;
    m = fmax(m, v);
  }
  bad = __syncthreads_or(bad);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < 8 ? s_w[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) {
      double d = m > 0.0 ? cfl_dxmin / m : dt_max;
      *dt_out = bad ? __longlong_as_double(0x7ff8000000000000LL) : fmin(d, dt_max);
    }
  }
}

// Unique id of the current CUDA context (0 when it cannot be read): a new
// context on the same device (after cudaDeviceReset) has a new id.
static unsigned long long current_context_id() {
  static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Device address of the scratch on the current device, looked up again
// whenever the device's context is not the one of the cached address.
static double* partials_on_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  unsigned long long id = current_context_id();
  if (!g_partials_addr[dev] || id == 0 || id != g_partials_ctx[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_cfl_partials) != cudaSuccess) return nullptr;
    g_partials_addr[dev] = static_cast<double*>(ptr);
    g_partials_ctx[dev] = current_context_id();
  }
  return g_partials_addr[dev];
}

}  // namespace enl

using namespace enl;

extern "C" {

int enl_cfl_dt_static(int ifirst0, int ilast0, int ifirst1, int ilast1, int gcw0, int gcw1, const double* w_n,
                      const double* dx, double c, double cfl, double dt_max, double* dt_out) {
  const int nx = ilast0 - ifirst0 + 1, ny = ilast1 - ifirst1 + 1;
  if (nx <= 0 || ny <= 0 || gcw0 < 0 || gcw1 < 0 || !w_n || !dx || !dt_out || cfl <= 0.0 || dt_max <= 0.0) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  const long tiles = (long)((nx + 31) / 32) * ((ny + 7) / 8);
  if (tiles > kScratchBlocks) {
    fprintf(stderr,
            "enl_cfl_dt_static: patch of %d x %d cells needs %ld tiles of 32x8, the static scratch holds %d "
            "(at most %d cells)\n",
            nx, ny, tiles, kScratchBlocks, kScratchBlocks * 256);
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  double* partials = partials_on_current_device();
  if (!partials) {
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  const long pitch = nx + 2 * gcw0, fstride = pitch * (ny + 2 * gcw1);
  const double dxmin = dx[0] < dx[1] ? dx[0] : dx[1];
  cudaStream_t s = stream();
  cfl_partial_kernel<<<(unsigned)tiles, 256, 0, s>>>(w_n, pitch, fstride, gcw0, gcw1, nx, ny, c, partials);
  cfl_final_kernel<<<1, 256, 0, s>>>(partials, (int)tiles, cfl * dxmin, dt_max, dt_out);
  const int rc = check_launch("cfl_dt_static");
  if (rc != ENL_OK) {
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < kMaxDevices) g_partials_addr[dev] = nullptr;
  }
  return rc;
}

}  // extern "C"
