// Shared device helpers for the USBS GB300 kernels: error/status codes, bounded
// team barriers, warp/block reductions and the counter-based normal generator.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace usbs {

// Status bits written by kernels into a per-instance status word.
enum : int {
  ST_OK = 0,
  ST_BARRIER_TIMEOUT = 1,   // a team barrier wait ran past its limit
  ST_NONFINITE = 2,         // NaN/Inf met in a reduction
  ST_BREAKDOWN = 4,         // Lanczos breakdown path taken (informational)
  ST_SMALL_DENSE_FAIL = 8,  // singular k x k system / eigensolver did not converge
};

constexpr int WARP = 32;
constexpr int MAXM = 32;        // largest Lanczos inner dimension supported
constexpr int MAXK = 16;        // largest bundle rank k = k_curr + k_past
constexpr int MAXS = MAXK * (MAXK + 1) / 2;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Reduce-scatter of 32 per-lane columns across a warp: on return lane l holds
// the warp-wide sum of column l.  Butterfly with halving payload: 16+8+4+2+1
// shuffle-adds per lane instead of 32 x 5 for 32 separate warp sums.  x is
// consumed.  All 32 lanes must call it.
template <typename T>
__device__ __forceinline__ T warp_reduce_scatter32(T* x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const bool up = (lane & h) != 0;
#pragma unroll
    for (int j = 0; j < h; ++j) {
      const T send = up ? x[j] : x[j + h];
      const T keep = up ? x[j + h] : x[j];
      x[j] = keep + __shfl_xor_sync(0xffffffffu, send, h);
    }
  }
  return x[0];
}

// Sum of one double per thread over the block; result returned to every thread.
// `red` needs blockDim.x/32 doubles of shared memory.
__device__ __forceinline__ double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < nw; ++w) s += red[w];  // fixed order: identical in every CTA
  return s;
}

__device__ __forceinline__ double block_max(double v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = red[0];
  for (int w = 1; w < nw; ++w) s = fmax(s, red[w]);
  return s;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Team barrier over `nctas` CTAs that are co-resident (cooperative launch).
// `ctr[0]` counts arrivals, `ctr[1]` is the generation.  Every wait is bounded:
// after `limit_ns` of spinning the barrier records ST_BARRIER_TIMEOUT in
// *status and returns false; callers then leave the kernel.
struct TeamBarrier {
  unsigned int* ctr;
  int nctas;
  int* status;
  __device__ __forceinline__ bool sync(uint64_t limit_ns = 4000000000ull) {
    __syncthreads();
    bool ok = true;
    if (threadIdx.x == 0) {
      volatile unsigned int* vgen = ctr + 1;
      unsigned int gen = *vgen;
      __threadfence();
      unsigned int arrived = atomicAdd(ctr, 1u) + 1u;
      if (arrived == (unsigned)nctas) {
        atomicExch(ctr, 0u);
        __threadfence();
        atomicAdd(ctr + 1, 1u);
      } else {
        uint64_t t0 = globaltimer_ns();
        unsigned int spins = 0;
        while (*vgen == gen) {
          if (++spins > 64) __nanosleep(64);
          if ((spins & 255u) == 0 && globaltimer_ns() - t0 > limit_ns) {
            atomicOr(status, ST_BARRIER_TIMEOUT);
            ok = false;
            break;
          }
        }
      }
      __threadfence();
    }
    __syncthreads();
    // every CTA leaves if any CTA of the team timed out
    if (*(volatile int*)status & ST_BARRIER_TIMEOUT) ok = false;
    return ok;
  }
};

// ---- mbarrier in shared memory with a wait bounded by a globaltimer limit
// (run by the wait self-test).
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// wait for the phase with parity `parity` to complete; false after limit_ns
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  for (unsigned it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 63u) == 0 && globaltimer_ns() - t0 > limit_ns) return false;
  }
}

// splitmix64 (Vigna) and Box-Muller: the counter-based normal generator that the
// host side and the tests restate bit-for-bit in their integer part.
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double hash_normal(uint64_t key, uint64_t j) {
  const uint64_t base = key << 32;
  const uint64_t h1 = splitmix64(base + 2ull * j);
  const uint64_t h2 = splitmix64(base + 2ull * j + 1ull);
  const double u1 = ((double)(h1 >> 11) + 1.0) * 0x1.0p-53;
  const double u2 = (double)(h2 >> 11) * 0x1.0p-53;
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

template <typename T> struct Acc;            // per-thread accumulation type
template <> struct Acc<double> { typedef double type; };
template <> struct Acc<float> { typedef float type; };

}  // namespace usbs
