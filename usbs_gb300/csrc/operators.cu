// Problem-data callbacks on the device (reference: solver/utils.py:11-37 and the
// Lanczos operator of solver/lanczos.py:86-87).
//
// Triples (constraint c, row i, column j, value a) are kept in two sorted
// copies prepared once on the host: by constraint (for A(.), a segmented
// reduction per constraint) and by row (for A*(.), a segmented reduction per
// output row).  Neither kernel needs atomics, so every sum has a fixed order.
// The Lanczos operator C + A*(w) is assembled once per eigsh call onto the
// union of C's pattern and the triples' (i, j) positions; the solver's SpMV then
// reads one CSR matrix.
#include "common.cuh"
#include "internal.h"

namespace usbs {

template <typename OT>
__global__ void assemble_kernel(int nnz, const double* __restrict__ c_val, double alpha_c,
                                const int* __restrict__ slot_ptr, const int* __restrict__ slot_tid,
                                const int* __restrict__ con, const double* __restrict__ a,
                                const double* __restrict__ w, OT* __restrict__ out) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x) {
    double v = (alpha_c != 0.0 && c_val) ? alpha_c * c_val[p] : 0.0;
    if (w) {
      const int e = slot_ptr[p + 1];
      for (int q = slot_ptr[p]; q < e; ++q) {
        const int t = slot_tid[q];
        v += a[t] * w[con[t]];
      }
    }
    out[p] = (OT)v;
  }
}

int assemble_operator(int nnz, const double* c_val, double alpha_c, const int* slot_ptr,
                      const int* slot_tid, const int* con, const double* a, const double* w,
                      void* op_val, int prec, cudaStream_t stream) {
  if (nnz <= 0) return 0;
  const int threads = 256;
  int blocks = (nnz + threads - 1) / threads;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (prec == 64)
    assemble_kernel<double><<<blocks, threads, 0, stream>>>(nnz, c_val, alpha_c, slot_ptr,
                                                            slot_tid, con, a, w, (double*)op_val);
  else
    assemble_kernel<float><<<blocks, threads, 0, stream>>>(nnz, c_val, alpha_c, slot_ptr,
                                                           slot_tid, con, a, w, (float*)op_val);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_error("assemble_operator: %s", cudaGetErrorString(e)); return -5; }
  return 0;
}

// y[row] = sum_p val[p] x[col[p]], L lanes per row (vector CSR)
template <typename VT, int L>
__global__ void csr_spmv_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                const VT* __restrict__ val, const VT* __restrict__ x,
                                VT* __restrict__ y) {
  const int lanes_total = gridDim.x * blockDim.x;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int lig = gid % L;
  const int lane = threadIdx.x & 31;
  const unsigned gmask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << (lane & ~(L - 1)));
  for (int row = gid / L; row < n; row += lanes_total / L) {
    VT s = (VT)0;
    const int e = rowptr[row + 1];
    for (int p = rowptr[row] + lig; p < e; p += L) s += val[p] * x[col[p]];
#pragma unroll
    for (int o = L >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(gmask, s, o, L);
    if (lig == 0) y[row] = s;
  }
}

template <typename VT>
static void spmv_dispatch(int L, int blocks, int threads, cudaStream_t st, int n, const int* rp,
                          const int* c, const VT* v, const VT* x, VT* y) {
  switch (L) {
    case 1: csr_spmv_kernel<VT, 1><<<blocks, threads, 0, st>>>(n, rp, c, v, x, y); break;
    case 2: csr_spmv_kernel<VT, 2><<<blocks, threads, 0, st>>>(n, rp, c, v, x, y); break;
    case 4: csr_spmv_kernel<VT, 4><<<blocks, threads, 0, st>>>(n, rp, c, v, x, y); break;
    case 8: csr_spmv_kernel<VT, 8><<<blocks, threads, 0, st>>>(n, rp, c, v, x, y); break;
    case 16: csr_spmv_kernel<VT, 16><<<blocks, threads, 0, st>>>(n, rp, c, v, x, y); break;
    default: csr_spmv_kernel<VT, 32><<<blocks, threads, 0, st>>>(n, rp, c, v, x, y); break;
  }
}

int csr_spmv(int n, long long nnz, const int* rowptr, const int* col, const void* val,
             const void* x, void* y, int prec, int sm_count, cudaStream_t stream) {
  if (n <= 0) return 0;
  const int L = lanczos_lanes(n, nnz);
  const int threads = 256;
  long long need = ((long long)n * L + threads - 1) / threads;
  int blocks = (int)(need < (long long)sm_count * 8 ? need : (long long)sm_count * 8);
  if (blocks < 1) blocks = 1;
  if (prec == 64)
    spmv_dispatch<double>(L, blocks, threads, stream, n, rowptr, col, (const double*)val,
                          (const double*)x, (double*)y);
  else
    spmv_dispatch<float>(L, blocks, threads, stream, n, rowptr, col, (const float*)val,
                         (const float*)x, (float*)y);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_error("csr_spmv: %s", cudaGetErrorString(e)); return -5; }
  return 0;
}

// ------------------------------------------------------------------------
// Sliced-ELL operator apply.  Rows are grouped in windows of SELL_WIN = 256
// rows; inside a window they are sorted by length (longest first) and cut into
// 8 slices of 32 rows.  A slice stores its entries column-major (entry k of
// the slice's row r at sl_ptr[s] + 32 k + r), padded to the slice's longest
// row with column 0 and value 0.  One block per window, one warp per slice,
// lane = row: every load of col / val is a coalesced 128-byte line, and all of
// a row's loads are independent (no rowptr -> col -> x chain).  sl_row[32 s + r]
// is the row's position inside its window; results pass through shared memory
// so y is written in the original order, coalesced.
constexpr int SELL_WIN = 256;

template <typename VT>
__global__ void __launch_bounds__(SELL_WIN) sell_spmv_kernel(int n, const int* __restrict__ sl_ptr,
                                                           const int* __restrict__ col,
                                                           const VT* __restrict__ val,
                                                           const unsigned char* __restrict__ sl_row,
                                                           const VT* __restrict__ x,
                                                           VT* __restrict__ y) {
  __shared__ VT ys[SELL_WIN];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int s = blockIdx.x * (SELL_WIN / 32) + warp;
  const int w0 = blockIdx.x * SELL_WIN;
  const int nslices = (n + 31) / 32;
  VT acc = (VT)0;
  if (s < nslices) {
    const int base = sl_ptr[s], width = (sl_ptr[s + 1] - base) >> 5;
    const int* cp = col + base + lane;
    const VT* vp = val + base + lane;
    // the first SELL_PF entries of the row: every col / val load, then every
    // x gather, in flight at once; longer rows finish in a plain loop
    constexpr int SELL_PF = 16;
    int c[SELL_PF];
    VT v[SELL_PF], xv[SELL_PF];
#pragma unroll
    for (int u = 0; u < SELL_PF; ++u) {
      c[u] = (u < width) ? __ldg(cp + 32 * u) : 0;
      v[u] = (u < width) ? __ldg(vp + 32 * u) : (VT)0;
    }
#pragma unroll
    for (int u = 0; u < SELL_PF; ++u) xv[u] = (u < width) ? __ldg(x + c[u]) : (VT)0;
#pragma unroll
    for (int u = 0; u < SELL_PF; ++u) acc += v[u] * xv[u];
    for (int k = SELL_PF; k < width; ++k) acc += __ldg(vp + 32 * k) * __ldg(x + __ldg(cp + 32 * k));
    ys[sl_row[32 * s + lane]] = acc;
  }
  __syncthreads();
  const int r = w0 + threadIdx.x;
  if (r < n) y[r] = ys[threadIdx.x];
}

int sell_spmv(int n, const int* sl_ptr, const int* col, const void* val,
              const unsigned char* sl_row, const void* x, void* y, int prec, cudaStream_t stream) {
  if (n <= 0) return 0;
  const int blocks = (n + SELL_WIN - 1) / SELL_WIN;
  if (prec == 64)
    sell_spmv_kernel<double><<<blocks, SELL_WIN, 0, stream>>>(n, sl_ptr, col, (const double*)val,
                                                            sl_row, (const double*)x, (double*)y);
  else
    sell_spmv_kernel<float><<<blocks, SELL_WIN, 0, stream>>>(n, sl_ptr, col, (const float*)val,
                                                           sl_row, (const float*)x, (float*)y);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_error("sell_spmv: %s", cudaGetErrorString(e)); return -5; }
  return 0;
}

// Streaming reference for the SpMV's bandwidth: one pass over a (int4 words)
// and b (float4 words) with 16-byte loads, grid-stride, no gathers; block k
// writes the sum of the floats it read to out_sum[k] and the XOR of the words
// it read to out_xor[k].  Timed like the SpMV (one launch after an L2 flush),
// it shows what a kernel moving the same bytes can reach at that size.
__global__ void __launch_bounds__(256) stream_probe_kernel(long long na, const int4* __restrict__ a,
                                                           long long nb, const float4* __restrict__ b,
                                                           float* __restrict__ out_sum,
                                                           unsigned* __restrict__ out_xor) {
  __shared__ float ssum[8];
  __shared__ unsigned sxor[8];
  float acc = 0.f;
  unsigned x = 0u;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long nmax = na > nb ? na : nb;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nmax; i += stride) {
    if (i < na) {
      const int4 u = __ldg(a + i);
      x ^= (unsigned)u.x ^ (unsigned)u.y ^ (unsigned)u.z ^ (unsigned)u.w;
    }
    if (i < nb) {
      const float4 v = __ldg(b + i);
      acc += (v.x + v.y) + (v.z + v.w);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_xor_sync(0xffffffffu, acc, o);
    x ^= __shfl_xor_sync(0xffffffffu, x, o);
  }
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { ssum[warp] = acc; sxor[warp] = x; }
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    unsigned u = 0u;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { t += ssum[w]; u ^= sxor[w]; }
    out_sum[blockIdx.x] = t;
    out_xor[blockIdx.x] = u;
  }
}

int stream_probe(long long a_words, const void* a, long long b_words, const void* b, int blocks,
                 float* out_sum, unsigned* out_xor, cudaStream_t stream) {
  if (blocks < 1) return 0;
  stream_probe_kernel<<<blocks, 256, 0, stream>>>(a_words, (const int4*)a, b_words,
                                                  (const float4*)b, out_sum, out_xor);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_error("stream_probe: %s", cudaGetErrorString(e)); return -5; }
  return 0;
}

// dst[e] = src[map[e]] (0 where map[e] < 0): operator values from CSR to sliced-ELL order
template <typename VT>
__global__ void gather_values_kernel(long long total, const int* __restrict__ map,
                                     const VT* __restrict__ src, VT* __restrict__ dst) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int m = map[e];
    dst[e] = (m >= 0) ? src[m] : (VT)0;
  }
}

int gather_values(long long total, const int* map, const void* src, void* dst, int prec,
                  cudaStream_t stream) {
  if (total <= 0) return 0;
  long long b = (total + 255) / 256;
  const int blocks = (int)(b < 152 * 16 ? b : 152 * 16);
  if (prec == 64)
    gather_values_kernel<double><<<blocks, 256, 0, stream>>>(total, map, (const double*)src, (double*)dst);
  else
    gather_values_kernel<float><<<blocks, 256, 0, stream>>>(total, map, (const float*)src, (float*)dst);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_error("gather_values: %s", cudaGetErrorString(e)); return -5; }
  return 0;
}

// out[c] = sum_{t in constraint c} a_t * U[i_t, :] . U[j_t, :]    (one warp per constraint)
__global__ void A_operator_kernel(int m, const int* __restrict__ con_ptr,
                                  const int* __restrict__ t_row, const int* __restrict__ t_col,
                                  const double* __restrict__ a, const double* __restrict__ U,
                                  int ldu, int k, double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < m; c += warps) {
    double s = 0.0;
    const int e = con_ptr[c + 1];
    for (int t = con_ptr[c] + lane; t < e; t += 32) {
      const int i = t_row[t], j = t_col[t];
      double d = 0.0;
      for (int q = 0; q < k; ++q) d += U[(size_t)q * ldu + i] * U[(size_t)q * ldu + j];
      s += a[t] * d;
    }
    s = warp_sum(s);
    if (lane == 0) out[c] = s;
  }
}

int apply_A_operator(int m, const int* con_ptr, const int* t_row, const int* t_col,
                     const double* a, const double* U, int ldu, int k, double* out,
                     cudaStream_t stream) {
  if (m <= 0) return 0;
  const int threads = 256;
  long long need = ((long long)m * 32 + threads - 1) / threads;
  int blocks = (int)(need < 152 * 16 ? need : 152 * 16);
  A_operator_kernel<<<blocks, threads, 0, stream>>>(m, con_ptr, t_row, t_col, a, U, ldu, k, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_error("apply_A_operator: %s", cudaGetErrorString(e)); return -5; }
  return 0;
}

// out[i, q] = sum_{t with row i} a_t z[c_t] U[j_t, q]    (one warp per row, lanes over triples)
__global__ void A_adjoint_kernel(int n, const int* __restrict__ row_ptr,
                                 const int* __restrict__ r_con, const int* __restrict__ r_col,
                                 const double* __restrict__ r_a, const double* __restrict__ z,
                                 const double* __restrict__ U, int ldu, int k,
                                 double* __restrict__ out, int ldo) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const int b = row_ptr[i], e = row_ptr[i + 1];
    for (int q = 0; q < k; ++q) {
      double s = 0.0;
      for (int t = b + lane; t < e; t += 32)
        s += r_a[t] * z[r_con[t]] * U[(size_t)q * ldu + r_col[t]];
      s = warp_sum(s);
      if (lane == 0) out[(size_t)q * ldo + i] = s;
    }
  }
}

int apply_A_adjoint(int n, const int* row_ptr, const int* r_con, const int* r_col,
                    const double* r_a, const double* z, const double* U, int ldu, int k,
                    double* out, int ldo, cudaStream_t stream) {
  if (n <= 0) return 0;
  const int threads = 256;
  long long need = ((long long)n * 32 + threads - 1) / threads;
  int blocks = (int)(need < 152 * 16 ? need : 152 * 16);
  A_adjoint_kernel<<<blocks, threads, 0, stream>>>(n, row_ptr, r_con, r_col, r_a, z, U, ldu, k,
                                                   out, ldo);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_error("apply_A_adjoint: %s", cudaGetErrorString(e)); return -5; }
  return 0;
}

}  // namespace usbs
