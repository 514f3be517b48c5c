// extern "C" entry points of libusbs_gb300 (declared in include/usbs_gb300.h).
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <mutex>
#include "../../include/usbs_gb300.h"
#include "common.cuh"
#include "internal.h"

namespace usbs {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

static DeviceInfo g_info[64];
static std::mutex g_info_mu;

int get_device_info(DeviceInfo* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) { set_error("cudaGetDevice: %s", cudaGetErrorString(e)); return -5; }
  if (dev < 0 || dev >= 64) { set_error("device index %d out of range", dev); return -2; }
  std::lock_guard<std::mutex> lk(g_info_mu);
  DeviceInfo& di = g_info[dev];
  if (di.device != dev) {
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) { set_error("device attribute: %s", cudaGetErrorString(e)); return -5; }
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) { set_error("device %d does not support cooperative launches", dev); return -5; }
    di.sm_count = sms;
    di.lanczos_occ64 = lanczos_occupancy(64);
    di.lanczos_occ32 = lanczos_occupancy(32);
    di.stream_occ64 = lanczos_stream_occupancy(64);
    di.stream_occ32 = lanczos_stream_occupancy(32);
    di.device = dev;
  }
  *out = di;
  return 0;
}

static size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

// Fixed device scratch of usbs_eigsh_smallest_noalloc: part of the module
// image, so it exists on every device that loads the library and is never
// allocated or freed at run time.  Its address belongs to a CUDA context (the
// module is loaded once per context), so it is looked up once per device and
// looked up again when the current context of that device has changed (a
// device reset, or a caller that made another context current through the
// driver API).
static __device__ __align__(256) unsigned char g_eigsh_scratch[USBS_EIGSH_STATIC_SCRATCH_BYTES];
struct ScratchAddr {
  void* ctx;
  void* ptr;
};
static ScratchAddr g_eigsh_scratch_addr[64];
static std::mutex g_eigsh_scratch_mu;

// the calling thread's current CUDA context (driver handle), or null
static void* current_context() {
  typedef int (*CtxGetCurrent)(void**);
  static const CtxGetCurrent fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      f = nullptr;
    }
    return (CtxGetCurrent)f;
  }();
  void* ctx = nullptr;
  if (fn && fn(&ctx) == 0) return ctx;
  return nullptr;
}

static int eigsh_static_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) { set_error("cudaGetDevice: %s", cudaGetErrorString(e)); return -5; }
  if (dev < 0 || dev >= 64) { set_error("device index %d out of range", dev); return -2; }
  void* ctx = current_context();
  std::lock_guard<std::mutex> lk(g_eigsh_scratch_mu);
  ScratchAddr& a = g_eigsh_scratch_addr[dev];
  if (!a.ptr || a.ctx != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_eigsh_scratch);
    if (e != cudaSuccess || !p) {
      set_error("eigsh_noalloc: cudaGetSymbolAddress of the static scratch on device %d: %s", dev,
                cudaGetErrorString(e));
      return -5;
    }
    a.ptr = p;
    a.ctx = current_context();   // the lookup made the device's context current if none was
  }
  *out = a.ptr;
  return 0;
}

}  // namespace usbs

using namespace usbs;

extern "C" {

int usbs_abi_version(void) { return USBS_GB300_ABI_VERSION; }

const char* usbs_last_error(void) { return g_err; }

int usbs_device_info(int device, int* sm_count, int* occ64, int* occ32) {
  int prev = 0;
  cudaGetDevice(&prev);
  if (cudaSetDevice(device) != cudaSuccess) { set_error("cudaSetDevice(%d) failed", device); return -5; }
  DeviceInfo di;
  int rc = get_device_info(&di);
  cudaSetDevice(prev);
  if (rc) return rc;
  if (sm_count) *sm_count = di.sm_count;
  if (occ64) *occ64 = di.lanczos_occ64;
  if (occ32) *occ32 = di.lanczos_occ32;
  return 0;
}

int usbs_assemble_operator(long long nnz, const double* c_val, double c_scale,
                           const int* slot_ptr, const int* slot_tid, const int* t_con,
                           const double* t_a, const double* w, void* op_val, int precision,
                           void* stream) {
  if (precision != 32 && precision != 64) { set_error("precision must be 32 or 64"); return -2; }
  if (nnz < 0 || nnz > 0x7fffffffLL) { set_error("nnz %lld out of range", nnz); return -2; }
  if (w && (!slot_ptr || !slot_tid || !t_con || !t_a)) {
    set_error("assemble: w given without the slot map / triples");
    return -2;
  }
  return assemble_operator((int)nnz, c_val, c_scale, slot_ptr, slot_tid, t_con, t_a, w, op_val,
                           precision, (cudaStream_t)stream);
}

int usbs_operator_apply(int n, long long nnz, const int* rowptr, const int* col,
                        const void* op_val, const void* x, void* y, int precision,
                        void* stream) {
  if (precision != 32 && precision != 64) { set_error("precision must be 32 or 64"); return -2; }
  if (n < 0) { set_error("n < 0"); return -2; }
  DeviceInfo di;
  int rc = get_device_info(&di);
  if (rc) return rc;
  return csr_spmv(n, nnz, rowptr, col, op_val, x, y, precision, di.sm_count,
                  (cudaStream_t)stream);
}

int usbs_operator_apply_sell(int n, const int* sl_ptr, const int* sl_col, const void* sl_val,
                             const unsigned char* sl_row, const void* x, void* y, int precision,
                             void* stream) {
  if (precision != 32 && precision != 64) { set_error("precision must be 32 or 64"); return -2; }
  if (n < 0) { set_error("n < 0"); return -2; }
  return sell_spmv(n, sl_ptr, sl_col, sl_val, sl_row, x, y, precision, (cudaStream_t)stream);
}

int usbs_stream_probe(const void* a, long long a_bytes, const void* b, long long b_bytes,
                      int blocks, float* out_sum, unsigned* out_xor, void* stream) {
  if (a_bytes < 0 || b_bytes < 0 || (a_bytes & 15) || (b_bytes & 15)) {
    set_error("usbs_stream_probe: byte counts must be non-negative multiples of 16");
    return -2;
  }
  if ((a_bytes && ((uintptr_t)a & 15)) || (b_bytes && ((uintptr_t)b & 15))) {
    set_error("usbs_stream_probe: buffers must be 16-byte aligned");
    return -2;
  }
  if (blocks < 1 || !out_sum || !out_xor) {
    set_error("usbs_stream_probe: blocks >= 1 and both outputs are required");
    return -2;
  }
  return stream_probe(a_bytes / 16, a, b_bytes / 16, b, blocks, out_sum, out_xor,
                      (cudaStream_t)stream);
}

int usbs_gather_values(long long total, const int* map, const void* src, void* dst,
                       int precision, void* stream) {
  if (precision != 32 && precision != 64) { set_error("precision must be 32 or 64"); return -2; }
  if (total < 0) { set_error("total < 0"); return -2; }
  return gather_values(total, map, src, dst, precision, (cudaStream_t)stream);
}

int usbs_apply_A_operator(int m, int k, const int* con_ptr, const int* t_row, const int* t_col,
                          const double* t_a, const double* U, int ldu, double* out,
                          void* stream) {
  if (m < 0 || k < 1 || ldu < 1) { set_error("apply_A_operator: bad sizes m=%d k=%d ldu=%d", m, k, ldu); return -2; }
  return apply_A_operator(m, con_ptr, t_row, t_col, t_a, U, ldu, k, out, (cudaStream_t)stream);
}

int usbs_apply_A_adjoint(int n, int k, const int* row_ptr, const int* r_con, const int* r_col,
                         const double* r_a, const double* z, const double* U, int ldu,
                         double* out, int ldo, void* stream) {
  if (n < 0 || k < 1 || ldu < n || ldo < n) {
    set_error("apply_A_adjoint: bad sizes n=%d k=%d ldu=%d ldo=%d", n, k, ldu, ldo);
    return -2;
  }
  return apply_A_adjoint(n, row_ptr, r_con, r_col, r_a, z, U, ldu, k, out, ldo,
                         (cudaStream_t)stream);
}

int usbs_lanczos_kernel(int n, int inner_iterations, int precision) {
  if (precision != 32 && precision != 64) { set_error("precision must be 32 or 64"); return -2; }
  return lanczos_kernel_kind(n, inner_iterations, precision);
}

size_t usbs_eigsh_workspace_bytes(int n, long long nnz, int inner_iterations, int precision) {
  DeviceInfo di;
  if (get_device_info(&di)) {
    // no device: size for the largest GB300 team (152 SMs x 4 CTAs)
    di.sm_count = 152;
    di.lanczos_occ64 = di.lanczos_occ32 = 4;
    di.stream_occ64 = di.stream_occ32 = 8;
  }
  const int vt = (precision == 64) ? 8 : 4;
  const int ld = (n + 31) & ~31;
  const int nctas = lanczos_team_size(di, n, precision);
  size_t b = a256((size_t)(nnz > 0 ? nnz : 1) * vt);
  b += a256(2 * MAXM * sizeof(double));
  b += lanczos_workspace_bytes(n, nnz, ld, inner_iterations, precision, nctas);
  return b;
}

int usbs_eigsh_smallest(int n, long long nnz, const int* rowptr, const int* col,
                        const double* c_val, double c_scale, const int* slot_ptr, const int* slot_tid,
                        const int* t_con, const double* t_a, const double* adjoint_left_vec,
                        const void* q0, int num_desired, int inner_iterations, int max_restarts,
                        double tolerance, int precision, void* Q, int ldq, double* eigenvalues,
                        int* info, void* workspace, size_t workspace_bytes, void* stream) {
  if (precision != 32 && precision != 64) { set_error("precision must be 32 or 64"); return -2; }
  if (n < 1 || ldq < n || inner_iterations < 1 || inner_iterations > MAXM ||
      num_desired < 1 || num_desired > inner_iterations || max_restarts < 0) {
    set_error("eigsh: bad sizes n=%d ldq=%d inner_iterations=%d (<= %d) num_desired=%d "
              "max_restarts=%d", n, ldq, inner_iterations, MAXM, num_desired, max_restarts);
    return -2;
  }
  if (nnz < 0 || nnz > 0x7fffffffLL) { set_error("nnz %lld out of range", nnz); return -2; }
  const size_t need = usbs_eigsh_workspace_bytes(n, nnz, inner_iterations, precision);
  if (!workspace || workspace_bytes < need) {
    set_error("eigsh: workspace of %zu bytes given, %zu needed", workspace_bytes, need);
    return -2;
  }
  DeviceInfo di;
  int rc = get_device_info(&di);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int vt = (precision == 64) ? 8 : 4;
  char* w = (char*)workspace;
  void* op_val = w; w += a256((size_t)(nnz > 0 ? nnz : 1) * vt);
  double* alpha = (double*)w;
  double* beta = alpha + MAXM;
  w += a256(2 * MAXM * sizeof(double));
  rc = assemble_operator((int)nnz, c_val, c_scale, slot_ptr, slot_tid, t_con, t_a, adjoint_left_vec,
                         op_val, precision, st);
  if (rc) return rc;
  if (cudaMemcpyAsync(Q, q0, (size_t)n * vt, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
      cudaMemsetAsync(alpha, 0, 2 * MAXM * sizeof(double), st) != cudaSuccess) {
    set_error("eigsh: staging copy failed");
    return -5;
  }
  LanczosProblem p;
  p.n = n; p.ld = ldq; p.m = inner_iterations; p.num_desired = num_desired;
  p.max_restarts = max_restarts; p.nnz = nnz; p.tol = tolerance;
  p.rowptr = rowptr; p.col = col; p.val = op_val; p.Q = Q;
  p.alpha = alpha; p.beta = beta; p.ctl = info; p.status = info + 5; p.work = w;
  rc = lanczos_run(di, &p, 1, precision, st);
  if (rc) return rc;
  if (cudaMemcpyAsync(eigenvalues, alpha, (size_t)num_desired * sizeof(double),
                      cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
    set_error("eigsh: result copy failed");
    return -5;
  }
  return 0;
}

int usbs_eigsh_smallest_batched(int count, const usbs_eigsh_problem* problems,
                                int inner_iterations, int max_restarts, double tolerance,
                                int precision, void* stream) {
  if (precision != 32 && precision != 64) { set_error("precision must be 32 or 64"); return -2; }
  if (count < 0 || (count > 0 && !problems) || inner_iterations < 1 ||
      inner_iterations > MAXM || max_restarts < 0) {
    set_error("eigsh_batched: bad arguments count=%d inner_iterations=%d (<= %d) max_restarts=%d",
              count, inner_iterations, MAXM, max_restarts);
    return -2;
  }
  for (int i = 0; i < count; ++i) {
    const usbs_eigsh_problem& q = problems[i];
    if (q.n < 1 || q.ldq < q.n || q.num_desired < 1 || q.num_desired > inner_iterations ||
        q.nnz < 0 || q.nnz > 0x7fffffffLL) {
      set_error("eigsh_batched: problem %d: bad sizes n=%d ldq=%d num_desired=%d nnz=%lld", i,
                q.n, q.ldq, q.num_desired, q.nnz);
      return -2;
    }
    const size_t need = usbs_eigsh_workspace_bytes(q.n, q.nnz, inner_iterations, precision);
    if (!q.workspace || q.workspace_bytes < need) {
      set_error("eigsh_batched: problem %d: workspace of %zu bytes given, %zu needed", i,
                q.workspace_bytes, need);
      return -2;
    }
  }
  if (count == 0) return 0;
  DeviceInfo di;
  int rc = get_device_info(&di);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int vt = (precision == 64) ? 8 : 4;
  constexpr int CHUNK = 48;                 // problems per launch (the kernels' batch limit)
  LanczosProblem lp[CHUNK];
  for (int c0 = 0; c0 < count; c0 += CHUNK) {
    const int cnt = (count - c0) < CHUNK ? (count - c0) : CHUNK;
    for (int j = 0; j < cnt; ++j) {
      const usbs_eigsh_problem& q = problems[c0 + j];
      char* w = (char*)q.workspace;
      void* op_val = w; w += a256((size_t)(q.nnz > 0 ? q.nnz : 1) * vt);
      double* alpha = (double*)w;
      w += a256(2 * MAXM * sizeof(double));
      rc = assemble_operator((int)q.nnz, q.c_val, q.c_scale, q.slot_ptr, q.slot_tid, q.t_con,
                             q.t_a, q.adjoint_left_vec, op_val, precision, st);
      if (rc) return rc;
      if (cudaMemcpyAsync(q.Q, q.q0, (size_t)q.n * vt, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
          cudaMemsetAsync(alpha, 0, 2 * MAXM * sizeof(double), st) != cudaSuccess) {
        set_error("eigsh_batched: staging copy failed");
        return -5;
      }
      LanczosProblem& p = lp[j];
      p.n = q.n; p.ld = q.ldq; p.m = inner_iterations; p.num_desired = q.num_desired;
      p.max_restarts = max_restarts; p.nnz = q.nnz; p.tol = tolerance;
      p.rowptr = q.rowptr; p.col = q.col; p.val = op_val; p.Q = q.Q;
      p.alpha = alpha; p.beta = alpha + MAXM; p.ctl = q.info; p.status = q.info + 5; p.work = w;
    }
    rc = lanczos_run(di, lp, cnt, precision, st);
    if (rc) return rc;
    for (int j = 0; j < cnt; ++j) {
      if (cudaMemcpyAsync(problems[c0 + j].eigenvalues, lp[j].alpha,
                          (size_t)lp[j].num_desired * sizeof(double), cudaMemcpyDeviceToDevice,
                          st) != cudaSuccess) {
        set_error("eigsh_batched: result copy failed");
        return -5;
      }
    }
  }
  return 0;
}

int usbs_lanczos_autotune(int count, const usbs_eigsh_problem* problems, int inner_iterations,
                          int max_restarts, double tolerance, int precision, void* stream,
                          int* best_rows_per_cta, float* candidate_ms) {
  if (count < 1 || count > 48 || !problems || !best_rows_per_cta) {
    set_error("lanczos_autotune: count=%d must be in [1, 48] with problems and an output", count);
    return -2;
  }
  int nmax = 1;
  for (int i = 0; i < count; ++i) nmax = problems[i].n > nmax ? problems[i].n : nmax;
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    set_error("lanczos_autotune: event create failed");
    return -5;
  }
  int best = 0, prev_csize = -1, rc = 0;
  float best_ms = 0.f;
  for (int i = 0; lanczos_tune_candidates(i) > 0; ++i) {
    const int target = lanczos_tune_candidates(i);
    if (candidate_ms) candidate_ms[i] = -1.f;
    const int cs = lanczos_cluster_size(nmax, target);
    if (cs == prev_csize) continue;               // the same launch as the previous candidate
    prev_csize = cs;
    lanczos_force_target(target);
    rc = usbs_eigsh_smallest_batched(count, problems, inner_iterations, max_restarts, tolerance,
                                     precision, stream);           // warm-up
    if (!rc && cudaEventRecord(e0, st) != cudaSuccess) rc = -5;
    if (!rc) rc = usbs_eigsh_smallest_batched(count, problems, inner_iterations, max_restarts,
                                              tolerance, precision, stream);
    if (!rc && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess))
      rc = -5;
    lanczos_force_target(0);
    float ms = 0.f;
    if (!rc && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = -5;
    if (rc) break;
    if (candidate_ms) candidate_ms[i] = ms;
    if (!best || ms < best_ms) { best = target; best_ms = ms; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) {
    if (rc == -5) set_error("lanczos_autotune: timing failed");
    return rc;
  }
  lanczos_tune_record(precision, count, nmax, best);
  *best_rows_per_cta = best;
  // leave the outputs of the chosen configuration
  return usbs_eigsh_smallest_batched(count, problems, inner_iterations, max_restarts, tolerance,
                                     precision, stream);
}

int usbs_lanczos_tuning_get(long long* keys, int* rows_per_cta, int capacity) {
  if (capacity < 0 || (capacity > 0 && (!keys || !rows_per_cta))) {
    set_error("lanczos_tuning_get: bad capacity %d or null arrays", capacity);
    return -2;
  }
  return lanczos_tune_entries(keys, rows_per_cta, capacity);
}

int usbs_lanczos_tuning_put(int precision, int count, int max_n, int rows_per_cta) {
  if ((precision != 32 && precision != 64) || count < 1 || max_n < 1 ||
      (rows_per_cta != 0 && rows_per_cta < 16)) {
    set_error("lanczos_tuning_put: precision=%d count=%d max_n=%d rows_per_cta=%d", precision,
              count, max_n, rows_per_cta);
    return -2;
  }
  lanczos_tune_record(precision, count, max_n, rows_per_cta);
  return 0;
}

void usbs_lanczos_tuning_clear(void) { lanczos_tune_clear(); }

int usbs_eigsh_smallest_noalloc(int n, long long nnz, const int* rowptr, const int* col,
                                const double* c_val, double c_scale, const int* slot_ptr,
                                const int* slot_tid, const int* t_con, const double* t_a,
                                const double* adjoint_left_vec, const void* q0, int num_desired,
                                int inner_iterations, int max_restarts, double tolerance,
                                int precision, void* Q, int ldq, double* eigenvalues, int* info,
                                void* stream) {
  if (precision != 32 && precision != 64) { set_error("precision must be 32 or 64"); return -2; }
  if (n < 1 || inner_iterations < 1 || inner_iterations > MAXM || nnz < 0 || nnz > 0x7fffffffLL) {
    set_error("eigsh_noalloc: bad sizes n=%d nnz=%lld inner_iterations=%d (<= %d)", n, nnz,
              inner_iterations, MAXM);
    return -2;
  }
  const size_t need = usbs_eigsh_workspace_bytes(n, nnz, inner_iterations, precision);
  if (need > (size_t)USBS_EIGSH_STATIC_SCRATCH_BYTES) {
    set_error("eigsh_noalloc: n=%d nnz=%lld inner_iterations=%d precision=%d needs %zu bytes of "
              "scratch, the static scratch holds %zu; call usbs_eigsh_smallest with a workspace",
              n, nnz, inner_iterations, precision, need, (size_t)USBS_EIGSH_STATIC_SCRATCH_BYTES);
    return -2;
  }
  void* scratch = nullptr;
  int rc = eigsh_static_scratch(&scratch);
  if (rc) return rc;
  return usbs_eigsh_smallest(n, nnz, rowptr, col, c_val, c_scale, slot_ptr, slot_tid, t_con, t_a,
                             adjoint_left_vec, q0, num_desired, inner_iterations, max_restarts,
                             tolerance, precision, Q, ldq, eigenvalues, info, scratch,
                             (size_t)USBS_EIGSH_STATIC_SCRATCH_BYTES, stream);
}

}  // extern "C"
