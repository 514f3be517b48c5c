// Self-test of the library's bounded device waits.
//
// Every spin-wait of the library (the Lanczos team kernel's cooperative
// barrier, and the bounded mbarrier wait of common.cuh) gives up after a time
// limit, records ST_BARRIER_TIMEOUT in the caller's status word and returns, so
// the context stays usable.  usbs_selftest_wait_limits runs exactly those two
// waits on a condition that nothing ever satisfies (a team barrier that expects
// one CTA more than the launch has; an mbarrier that no thread or copy arrives
// at), with a caller-chosen limit, so a test can see the timeout path end in
// the status word instead of a hang.  The reference has no device code and no
// counterpart.
#include "../../include/usbs_gb300.h"
#include "common.cuh"
#include "internal.h"

namespace usbs {

__global__ void selftest_wait_kernel(int which, int expected, unsigned long long limit_ns,
                                     unsigned int* ctr, int* status) {
  if (which == 0) {
    TeamBarrier bar{ctr, expected, status};
    bar.sync(limit_ns);
    return;
  }
  __shared__ __align__(8) uint64_t mb;
  if (threadIdx.x == 0) {
    mbar_init(&mb, 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (threadIdx.x == 0 && !mbar_wait(&mb, 0u, limit_ns)) atomicOr(status, ST_BARRIER_TIMEOUT);
  __syncthreads();
}

}  // namespace usbs

using namespace usbs;

extern "C" int usbs_selftest_wait_limits(int which, int nctas, long long limit_ns,
                                         unsigned int* counters, int* status, void* stream) {
  if ((which != 0 && which != 1) || nctas < 1 || nctas > 8 || limit_ns < 1000 ||
      limit_ns > 2000000000LL || !status || (which == 0 && !counters)) {
    set_error("selftest_wait_limits: which=%d nctas=%d limit_ns=%lld (1 us .. 2 s)", which, nctas,
              limit_ns);
    return -2;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (which == 0 && cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned int), st) != cudaSuccess) {
    set_error("selftest_wait_limits: memset failed");
    return -5;
  }
  // the team barrier expects one CTA more than are launched; the launch is
  // cooperative so that the CTAs that do exist are co-resident
  int expected = nctas + 1;
  unsigned long long lim = (unsigned long long)limit_ns;
  void* args[] = {(void*)&which, (void*)&expected, (void*)&lim, (void*)&counters, (void*)&status};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)selftest_wait_kernel, dim3(nctas),
                                              dim3(64), args, 0, st);
  if (e != cudaSuccess) {
    set_error("selftest_wait_limits: launch failed: %s", cudaGetErrorString(e));
    return -5;
  }
  return 0;
}
