// kb_noalloc.cu -- CFL time-step reduction that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host that hands all of its device
// memory to its own pool (a Julia session whose CUDA arrays live in the
// CUDA.jl pool, a server whose admission control has already accounted every
// byte), or code that must not add allocations in the middle of a time loop.
// kb_timestep keeps its partial result in memory owned by a solver handle;
// this variant takes the primitive state and the output as the caller's own
// device pointers and keeps its per-block partial maxima in one fixed,
// file-scope device array instead.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/kitgpu.h"
#include "kb_kernels.cuh"

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_CELLS_PER_THREAD = 8;
constexpr int NA_MAX_BLOCKS = KB_NOALLOC_MAX_CELLS / (NA_THREADS * NA_CELLS_PER_THREAD);
constexpr int NA_MAX_DEVICES = 64;

// Per-block partial maxima of every call on this device (8 KB).  Each call
// rewrites entries [0, nblocks) before reading them back, so nothing has to
// start at zero; calls that overlap on the GPU share it and race.
static __device__ __align__(256) double g_na_partial[NA_MAX_BLOCKS];

// Device address of g_na_partial per device, looked up by the first call on
// that device.  A device reset (cudaDeviceReset, or a Julia session's
// device_reset!) unloads the module and releases the array, so the cached
// address is stale afterwards: the entry point must not be used again in a
// process after a reset of its device.
double* g_na_addr[NA_MAX_DEVICES] = {nullptr};
std::mutex g_na_mutex;

// Maximum over this block's physical cells of the CFL rate
// (max(umax, |U|) + c) / dx (+ the y term in 2D) of timestep
// (src/Solver/solver_main.jl:240-342), c = sqrt(gamma / (2 lambda)).
__global__ void k_na_partial(const double* __restrict__ prim, double* __restrict__ part, int dim,
                             int nx, int ny, int ngx, int ngy, double dx, double dy, double umax,
                             double vmax, double gamma) {
  __shared__ double red[NA_THREADS];
  const int nw = dim + 2, nxt = nx + 2 * ngx;
  const long ncell = (long)nx * ny;
  const long base = (long)blockIdx.x * NA_THREADS * NA_CELLS_PER_THREAD;
  double m = 0.0;
  for (int k = 0; k < NA_CELLS_PER_THREAD; ++k) {
    long t = base + (long)k * NA_THREADS + threadIdx.x;
    if (t >= ncell) break;
    int i = (int)(t % nx), j = (int)(t / nx);
    const double* p = prim + ((long)(j + ngy) * nxt + (i + ngx)) * nw;
    double sos = pow(0.5 * gamma / p[nw - 1], 0.5);
    double r = dim == 1 ? (fmax(umax, fabs(p[1])) + sos) / dx
                        : (fmax(umax, fabs(p[1])) + sos) / dx + (fmax(vmax, fabs(p[2])) + sos) / dy;
    m = fmax(m, r);
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = NA_THREADS / 2; s >= 1; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_na_final(const double* __restrict__ part, int nblocks, double* __restrict__ out) {
  __shared__ double red[NA_THREADS];
  double m = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += NA_THREADS) m = fmax(m, part[b]);
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = NA_THREADS / 2; s >= 1; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

int na_fail(int code, const std::string& msg) {
  kb::set_error(msg);
  return code;
}

}  // namespace

extern "C" int kb_timestep_noalloc(const kb_config_t* cfg, const double* d_prim, double* d_tmax,
                                   void* stream) {
  if (!cfg || !d_prim || !d_tmax) return na_fail(KB_ERR_ARG, "kb_timestep_noalloc: null argument");
  if (cfg->dim != 1 && cfg->dim != 2) return na_fail(KB_ERR_CONFIG, "kb_timestep_noalloc: dim must be 1 or 2");
  const int ny = cfg->dim == 2 ? cfg->ny : 1;
  const int ngy = cfg->dim == 2 ? cfg->ngy : 0;
  if (cfg->nx < 1 || ny < 1 || cfg->ngx < 0 || ngy < 0 || !(cfg->x1 > cfg->x0) ||
      (cfg->dim == 2 && !(cfg->y1 > cfg->y0)) || !(cfg->gamma > 1.0))
    return na_fail(KB_ERR_CONFIG, "kb_timestep_noalloc: invalid geometry or gas");
  const long ncell = (long)cfg->nx * ny;
  if (ncell > KB_NOALLOC_MAX_CELLS)
    return na_fail(KB_ERR_ARG, "kb_timestep_noalloc: " + std::to_string(ncell) +
                                   " physical cells exceed the fixed scratch limit of " +
                                   std::to_string((long)KB_NOALLOC_MAX_CELLS) +
                                   " (KB_NOALLOC_MAX_CELLS); use kb_timestep");
  // An error already pending on this thread belongs to the caller's earlier
  // work: report it without taking it (it stays for the caller to read), so
  // that it is neither lost nor mistaken for a failure of these launches.
  {
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess)
      return na_fail(KB_ERR_CUDA, std::string("kb_timestep_noalloc: an earlier CUDA error is "
                                              "pending on this thread (left in place): ") +
                                      cudaGetErrorString(pending));
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) {
    cudaGetLastError();
    return na_fail(KB_ERR_CUDA, "kb_timestep_noalloc: no usable current CUDA device");
  }
  double* part = nullptr;
  {
    // first call on a device: look up the scratch array's device address
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_addr[dev]) {
      cudaError_t e = cudaGetSymbolAddress((void**)&g_na_addr[dev], g_na_partial);
      if (e != cudaSuccess) {
        g_na_addr[dev] = nullptr;
        return na_fail(KB_ERR_CUDA, std::string("kb_timestep_noalloc: cudaGetSymbolAddress: ") +
                                        cudaGetErrorString(e));
      }
    }
    part = g_na_addr[dev];
  }
  const int nblocks = (int)((ncell + NA_THREADS * NA_CELLS_PER_THREAD - 1) /
                            (NA_THREADS * NA_CELLS_PER_THREAD));
  const double dx = (cfg->x1 - cfg->x0) / cfg->nx;
  const double dy = cfg->dim == 2 ? (cfg->y1 - cfg->y0) / ny : 1.0;
  cudaStream_t st = (cudaStream_t)stream;
  k_na_partial<<<nblocks, NA_THREADS, 0, st>>>(d_prim, part, cfg->dim, cfg->nx, ny, cfg->ngx, ngy,
                                               dx, dy, cfg->umax, cfg->vmax, cfg->gamma);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return na_fail(KB_ERR_CUDA, std::string("kb_timestep_noalloc: launch of the per-block "
                                            "partial maxima: ") + cudaGetErrorString(e));
  k_na_final<<<1, NA_THREADS, 0, st>>>(part, nblocks, d_tmax);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return na_fail(KB_ERR_CUDA, std::string("kb_timestep_noalloc: launch of the final maximum: ") +
                                    cudaGetErrorString(e));
  return KB_OK;
}
