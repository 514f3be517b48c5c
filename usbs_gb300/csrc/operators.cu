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
