// Host-side declarations shared by the translation units of libusbs_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace usbs {

// Device properties cached per device.
struct DeviceInfo {
  int device = -1;
  int sm_count = 0;
  int lanczos_occ64 = 0;   // co-resident Lanczos CTAs per SM (FP64)
  int lanczos_occ32 = 0;   // co-resident Lanczos CTAs per SM (FP32)
  int stream_occ64 = 0;    // co-resident CTAs per SM of the stream-path kernels (FP64)
  int stream_occ32 = 0;    // ... (FP32)
};
int get_device_info(DeviceInfo* out);

void set_error(const char* fmt, ...);

// ---------------------------------------------------------------- Lanczos
// One eigsh_smallest problem on the device.  Q[:, 0] must hold the unit start
// vector.  `prec` 64 (double storage/arithmetic) or 32 (float storage, FP32
// dot products, FP64 team reductions and FP64 projected eigensolve).
struct LanczosProblem {
  int n, ld, m, num_desired, max_restarts;
  long long nnz;
  double tol;
  const int* rowptr;
  const int* col;
  const void* val;      // assembled operator values (double or float)
  void* Q;              // ld x (m+1), column-major
  double* alpha;        // m: Ritz values (alpha_hat) after the last restart
  double* beta;         // m
  int* ctl;             // 16 ints: k_next, nconv, restarts, breakdowns, steps, -, cycle counters
  int* status;
  void* work;           // workspace of lanczos_workspace_bytes()
  int rows_per_cta = 0; // cluster path: rows per CTA (0: measured class choice or default)
  int no_coop = 0;      // 1: never the cooperative team kernel (the stream path instead)
};
// `stream`: size for the stream path even where the team kernel would fit
size_t lanczos_workspace_bytes(int n, long long nnz, int ld, int m, int prec, int nctas,
                               bool stream = false);
int lanczos_team_size(const DeviceInfo& di, int n, int prec, bool stream = false);
int lanczos_lanes(int n, long long nnz);
int lanczos_occupancy(int prec);
int lanczos_stream_occupancy(int prec);
// 1 if a problem of n rows and m inner vectors runs as a thread-block cluster
// (shared-memory resident), 0 if it runs as a cooperative team.
int lanczos_kernel_kind(int n, int m, int prec);
// Runs `count` independent problems in one launch: one cluster each when they
// fit, else one cooperative team each.
int lanczos_run(const DeviceInfo& di, const LanczosProblem* probs, int count, int prec,
                cudaStream_t stream);
// kernels the calling thread's last lanczos_run launched
int lanczos_last_launches();
// cluster-size policy (rows per CTA by precision, batch and size class) and
// the autotuner's hooks
int lanczos_tune_candidates(int i);          // i-th candidate rows per CTA, 0 past the end
void lanczos_force_target(int target);       // this thread's launches use it (0: policy)
int lanczos_cluster_size(int nmax, int target);
void lanczos_tune_record(int prec, int count, int nmax, int target);   // target 0 erases
int lanczos_tune_entries(long long* keys, int* targets, int cap);
void lanczos_tune_clear();

// ---------------------------------------------------------------- operators
// op_val[p] = alpha_c * c_val[p] + sum_{t in slot p} a[t] * w[con[t]]
int assemble_operator(int nnz, const double* c_val, double alpha_c, const int* slot_ptr,
                      const int* slot_tid, const int* con, const double* a, const double* w,
                      void* op_val, int prec, cudaStream_t stream);
// y = M x  for CSR M (values double or float), optional per-row partial dots
int csr_spmv(int n, long long nnz, const int* rowptr, const int* col, const void* val,
             const void* x, void* y, int prec, int sm_count, cudaStream_t stream);
// y = M x for M in the sliced-ELL layout (windows of 256 rows, 32-row slices)
int sell_spmv(int n, const int* sl_ptr, const int* col, const void* val,
              const unsigned char* sl_row, const void* x, void* y, int prec, cudaStream_t stream);
// one pass over a (int4 words) and b (float4 words); per-block sum / XOR
int stream_probe(long long a_words, const void* a, long long b_words, const void* b, int blocks,
                 float* out_sum, unsigned* out_xor, cudaStream_t stream);
// dst[e] = src[map[e]], 0 where map[e] < 0
int gather_values(long long total, const int* map, const void* src, void* dst, int prec,
                  cudaStream_t stream);
// out[c] += sum over triples of constraint c: a * u[i] . u[j]   (k columns, ld)
int apply_A_operator(int m, const int* con_ptr, const int* t_row, const int* t_col,
                     const double* a, const double* U, int ldu, int k, double* out,
                     cudaStream_t stream);
// out[i, :] = sum over triples with row i: a * z[con] * U[j, :]
int apply_A_adjoint(int n, const int* row_ptr, const int* r_con, const int* r_col,
                    const double* r_a, const double* z, const double* U, int ldu, int k,
                    double* out, int ldo, cudaStream_t stream);

}  // namespace usbs
