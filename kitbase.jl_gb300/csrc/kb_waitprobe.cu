// kb_waitprobe.cu -- exercises the bounded device wait on a GPU without a fault.
//
// Every staging kernel (pass A, pass B, the batch segments) waits on
// mbarriers through mbar_wait_ns; a wait that gives up records status bit 1
// and the host reports KB_ERR_TIMEOUT.  This probe makes that wait run out on
// purpose, in the way a lost copy would leave it: phase 0 of an mbarrier
// completes by its one arrival, then the probe waits on phase 1, on which
// nothing ever arrives.  The wait gives up after the given limit, the status
// bit is set, the kernel returns, and the context stays usable.
#include <cuda_runtime.h>

#include <string>

#include "../../include/kitgpu.h"
#include "kb_kernels.cuh"
#include "kb_tma.cuh"

namespace {

// out[0]: status bits (bit 1 = a wait gave up, bit 2 = the completed phase
// was not seen); out[1]: nanoseconds the second wait took
__global__ void k_wait_probe(unsigned long long limit_ns, unsigned long long* out) {
  __shared__ unsigned long long bar;
  if (threadIdx.x != 0) return;
  kb::mbar_init(&bar, 1);
  kb::mbar_arrive(&bar);  // phase 0 completes
  unsigned long long st = 0;
  if (!kb::mbar_wait_ns(&bar, 0, limit_ns)) st |= 4;
  const unsigned long long t0 = kb::gtimer();
  if (!kb::mbar_wait_ns(&bar, 1, limit_ns)) st |= 2;  // phase 1: no arrival
  out[1] = kb::gtimer() - t0;
  out[0] = st;
}

int wp_fail(int code, const std::string& msg) {
  kb::set_error(msg);
  return code;
}

}  // namespace

extern "C" int kb_wait_probe(double limit_s, int32_t* status_out, double* waited_s) {
  if (!(limit_s > 0.0) || limit_s > 2.0)
    return wp_fail(KB_ERR_ARG, "kb_wait_probe: limit_s must be in (0, 2] seconds");
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) {
    cudaGetLastError();
    return wp_fail(KB_ERR_NOMEM, "kb_wait_probe: device allocation failed");
  }
  unsigned long long r[2] = {0, 0};
  int rc = KB_OK;
  k_wait_probe<<<1, 32>>>((unsigned long long)(limit_s * 1e9), d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(r, d, sizeof(r), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess)
    rc = wp_fail(KB_ERR_CUDA, std::string("kb_wait_probe: ") + cudaGetErrorString(e));
  cudaFree(d);
  if (rc != KB_OK) return rc;
  if (status_out) *status_out = (int32_t)r[0];
  if (waited_s) *waited_s = (double)r[1] * 1e-9;
  if (r[0] & 4) return wp_fail(KB_ERR_STATE, "kb_wait_probe: a completed mbarrier phase was not seen");
  if (r[0] & 2) return wp_fail(KB_ERR_TIMEOUT, "kb_wait_probe: the wait gave up after its limit (expected)");
  return KB_OK;
}
