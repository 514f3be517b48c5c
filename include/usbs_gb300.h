/*
 * usbs_gb300 — C ABI of the GB300 (sm_103a) USBS hot path.
 *
 * Conventions
 *  - Every pointer argument is a DEVICE pointer unless its comment says
 *    otherwise; the library never frees or reallocates caller memory.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *    Calls are stream-ordered and asynchronous unless stated otherwise.
 *  - Return value: 0 on success, negative on a host-side error (bad sizes,
 *    launch failure); usbs_last_error() then holds a thread-local message.
 *    Numerical/device conditions are reported through the `info`/`status`
 *    words the caller passes (device memory, read after synchronising).
 *  - `precision` selects the storage/arithmetic type of the n-sized vectors:
 *    64 = FP64 throughout (the parity path; the projected eigensolve is FP32
 *    Jacobi refined to FP64 by two Ogita-Aishima steps), 32 = FP32 vectors,
 *    dot products and projected eigensolve, with FP64 reductions over CTAs.
 *  - Triples: the reference's constraint tensor A is a list of (c, i, j, a)
 *    (A_indices rows and A_data, utils/maxcut_helpers.py:26-33,
 *    utils/qap_helpers.py:175-318).  The device keeps them sorted by
 *    constraint (con_ptr / t_row / t_col / t_a) and by row (row_ptr / r_con /
 *    r_col / r_a).  The Lanczos operator lives on the union pattern of C and
 *    the triples' (i, j) positions (rowptr / col); slot_ptr / slot_tid list,
 *    for every position of that pattern, the triples that land on it.
 */
#ifndef USBS_GB300_H
#define USBS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define USBS_GB300_ABI_VERSION 5

/* ABI version of the loaded library (USBS_GB300_ABI_VERSION). */
int usbs_abi_version(void);

/* Last host-side error message of the calling thread ("" if none). */
const char* usbs_last_error(void);

/* Multiprocessor count and the number of co-resident Lanczos CTAs per SM for
 * FP64 and FP32 on `device` (host pointers). */
int usbs_device_info(int device, int* sm_count, int* lanczos_ctas_per_sm64,
                     int* lanczos_ctas_per_sm32);

/* Lanczos operator values on the union pattern:
 *   op_val[p] = c_scale * c_val[p] + sum_{q in [slot_ptr[p], slot_ptr[p+1])}
 *               t_a[slot_tid[q]] * w[t_con[slot_tid[q]]]
 * i.e. the CSR of c_scale*C + A*(w).  Replaces the per-step
 * `C @ q + apply_A_adjoint_slim(n, A_data, A_indices, w, q)` of
 * solver/lanczos.py:86-87 by one assembled matrix per eigsh call.
 * c_val or w may be NULL (term omitted).  op_val is double (precision 64) or
 * float (precision 32). */
int usbs_assemble_operator(long long nnz, const double* c_val, double c_scale,
                           const int* slot_ptr, const int* slot_tid, const int* t_con,
                           const double* t_a, const double* w, void* op_val, int precision,
                           void* stream);

/* y = Op x for the assembled CSR operator (the "C matvec" callback,
 * solver/lanczos.py:86).  x, y, op_val in the type chosen by `precision`. */
int usbs_operator_apply(int n, long long nnz, const int* rowptr, const int* col,
                        const void* op_val, const void* x, void* y, int precision,
                        void* stream);

/* y = Op x with the operator in the sliced-ELL layout built by
 * usbs_gb300.problem.sell_layout: rows in windows of 256, sorted by length
 * inside a window and cut into 32-row slices; slice s holds its entries
 * column-major from sl_ptr[s] (sl_ptr has ceil(n/32)+1 ints, slices padded
 * with column 0 / value 0); sl_row[32 s + r] is row r's position inside its
 * window.  Same result as usbs_operator_apply on the CSR it was built from (up
 * to summation order).  No counterpart in the reference (its operator is a
 * BCOO matvec). */
int usbs_operator_apply_sell(int n, const int* sl_ptr, const int* sl_col, const void* sl_val,
                             const unsigned char* sl_row, const void* x, void* y, int precision,
                             void* stream);

/* Bandwidth reference for the operator apply, no counterpart in the
 * reference: one pass over a (a_bytes, read as 16-byte integer words) and b
 * (b_bytes, read as groups of four floats) with coalesced 16-byte loads and
 * no gathers, on `blocks` blocks of 256 threads.  Block k writes the sum of
 * the floats it read to out_sum[k] and the XOR of the 32-bit words of a it
 * read to out_xor[k].  Timed like usbs_operator_apply_sell over the same
 * bytes, it gives the bandwidth a kernel of that size reaches on this GPU.
 * Byte counts must be multiples of 16 and both buffers 16-byte aligned. */
int usbs_stream_probe(const void* a, long long a_bytes, const void* b, long long b_bytes,
                      int blocks, float* out_sum, unsigned* out_xor, void* stream);

/* dst[e] = src[map[e]] (0 where map[e] < 0), `total` entries of the
 * `precision` type: the CSR operator values moved into sliced-ELL order. */
int usbs_gather_values(long long total, const int* map, const void* src, void* dst,
                       int precision, void* stream);

/* out[c] = sum_j sum_{t in c} t_a[t] U[t_row[t], j] U[t_col[t], j], c < m:
 * apply_A_operator_slim (k = 1) / apply_A_operator_batched (k columns),
 * solver/utils.py:11-16 and 27-31.  U column-major n x k with leading
 * dimension ldu; out has m doubles. */
int usbs_apply_A_operator(int m, int k, const int* con_ptr, const int* t_row, const int* t_col,
                          const double* t_a, const double* U, int ldu, double* out,
                          void* stream);

/* out[i, q] = sum_{t with row i} r_a[t] z[r_con[t]] U[r_col[t], q], i < n:
 * apply_A_adjoint_slim (k = 1) / apply_A_adjoint_batched, solver/utils.py:19-24
 * and 34-37.  U and out column-major (ldu, ldo). */
int usbs_apply_A_adjoint(int n, int k, const int* row_ptr, const int* r_con, const int* r_col,
                         const double* r_a, const double* z, const double* U, int ldu,
                         double* out, int ldo, void* stream);

/* Which Lanczos path usbs_eigsh_smallest takes for n rows (host call):
 *   1 = one thread-block cluster with the basis in shared memory;
 *   0 = one cooperative launch (a team of CTAs, x staged in shared memory,
 *       n * sizeof(value) <= 160 KB); it needs the whole GPU co-resident;
 *   2 = the stream path (larger n): every Lanczos phase is an ordinary
 *       full-GPU launch, and the loop state is read back once per restart,
 *       so such a call synchronises `stream` at each restart and cannot be
 *       captured into a CUDA graph;
 * negative on error.  No counterpart in the reference. */
int usbs_lanczos_kernel(int n, int inner_iterations, int precision);

/* Workspace bytes needed by usbs_eigsh_smallest (host call, no GPU work). */
size_t usbs_eigsh_workspace_bytes(int n, long long nnz, int inner_iterations, int precision);

/* eigsh_smallest (solver/lanczos.py:239-284): the num_desired smallest
 * eigenpairs of c_scale*C + A*(adjoint_left_vec) (the solvers pass c_scale = -1
 * for their -C, solver/usbs.py:590) by thick-restart Lanczos with
 * inner_iterations (<= 32) vectors, at most max_restarts cycles and absolute
 * residual tolerance `tolerance`.
 *   q0:   unit start vector, n entries of the `precision` type;
 *   Q:    ldq x (inner_iterations + 1) column-major (`precision` type, ldq >= n);
 *         on return Q[:, :num_desired] are the eigenvectors;
 *   eigenvalues: num_desired doubles (ascending);
 *   info: 16 ints: [0] saved vectors of the last restart, [1] converged count,
 *         [2] restarts run, [3] breakdown restarts, [4] operator applications,
 *         [5] status bits (1 barrier timeout, 2 non-finite projected matrix:
 *             the call ends at that restart, 8 projected eigensolver failure),
 *         [6] kilo-cycles in the restarts, [7] kilo-cycles in total,
 *         [8..12] kilo-cycles of CTA 0 in barrier waits, team reductions and
 *         the three step phases, [13] sum over steps of the active basis
 *         columns, [14] sum over restarts of the saved vectors (for byte counts),
 *         [15] kilo-cycles of CTA 0 in the projected eigensolver.
 * Runs as one kernel launch when the problem's rows fit in a thread-block
 * cluster's shared memory or its x in one CTA's (usbs_lanczos_kernel 1 or 0);
 * the call is then asynchronous.  Larger problems take the stream path
 * (usbs_lanczos_kernel 2): a sequence of launches, with `stream`
 * synchronised once per restart.  Kilo-cycle counters [7..12] stay 0 there. */
int usbs_eigsh_smallest(int n, long long nnz, const int* rowptr, const int* col,
                        const double* c_val, double c_scale, const int* slot_ptr, const int* slot_tid,
                        const int* t_con, const double* t_a, const double* adjoint_left_vec,
                        const void* q0, int num_desired, int inner_iterations, int max_restarts,
                        double tolerance, int precision, void* Q, int ldq, double* eigenvalues,
                        int* info, void* workspace, size_t workspace_bytes, void* stream);

/* Bytes of the library's fixed device scratch for usbs_eigsh_smallest_noalloc. */
#define USBS_EIGSH_STATIC_SCRATCH_BYTES (16u << 20)

/* usbs_eigsh_smallest without a workspace argument, for callers that cannot
 * allocate device memory (a JAX/XLA custom call, whose runtime has already
 * reserved most of HBM, or a serving process with a fixed memory budget).
 * No counterpart in the reference: its eigsh_smallest allocates through JAX.
 *  - Allocates nothing: no cudaMalloc/cudaFree, no allocating library call.
 *    Scratch is a 16 MiB static device array in the library image.
 *  - The first call on each device looks up that array's address
 *    (cudaGetSymbolAddress, with that device current) and caches it, keyed
 *    by the current CUDA context: a call under another context (after a
 *    device reset, or with a context the caller made current through the
 *    driver API) looks it up again.  Make the first call on a device, and
 *    the first after such a change, before any stream capture on it.
 *  - Problems whose usbs_eigsh_workspace_bytes() exceeds
 *    USBS_EIGSH_STATIC_SCRATCH_BYTES are rejected (-2, usbs_last_error()).
 *    The scratch holds the assembled operator (nnz values), three n-vectors
 *    and at most 0.5 MB of partial sums, so with 32 inner iterations problems
 *    up to about nnz + 3n = 2.0e6 (FP64) or 4.0e6 (FP32) fit.  Stream-path
 *    problems (n > 20,480 in FP64, 40,960 in FP32) also hold the operator's
 *    sliced-ELL copy, about 1.5 * average degree * n more entries.
 *  - The scratch need not start at zero: each call clears its barrier
 *    counters, info words and Lanczos coefficients on `stream` before use.
 *  - One scratch per device: calls whose work may overlap in time on the
 *    same device (different streams or host threads) race.  Calls issued in
 *    order on one stream are safe.
 * Arguments, results and asynchrony are those of usbs_eigsh_smallest. */
int usbs_eigsh_smallest_noalloc(int n, long long nnz, const int* rowptr, const int* col,
                                const double* c_val, double c_scale, const int* slot_ptr,
                                const int* slot_tid, const int* t_con, const double* t_a,
                                const double* adjoint_left_vec, const void* q0, int num_desired,
                                int inner_iterations, int max_restarts, double tolerance,
                                int precision, void* Q, int ldq, double* eigenvalues, int* info,
                                void* stream);

/* One problem of usbs_eigsh_smallest_batched: the arguments of
 * usbs_eigsh_smallest that differ between problems (device pointers; the
 * workspace is usbs_eigsh_workspace_bytes(n, nnz, inner_iterations,
 * precision) bytes, one per problem). */
typedef struct usbs_eigsh_problem {
  int n;
  long long nnz;
  const int* rowptr;
  const int* col;
  const double* c_val;
  double c_scale;
  const int* slot_ptr;
  const int* slot_tid;
  const int* t_con;
  const double* t_a;
  const double* adjoint_left_vec;
  const void* q0;
  int num_desired;
  void* Q;
  int ldq;
  double* eigenvalues;
  int* info;
  void* workspace;
  size_t workspace_bytes;
} usbs_eigsh_problem;

/* eigsh_smallest for `count` independent problems with shared settings, in
 * as few launches as the kernels allow: up to 48 problems per launch, one
 * thread-block cluster each when every problem fits one (cluster size of
 * the largest), otherwise one cooperative team each.  Results and info words
 * as usbs_eigsh_smallest's, per problem (host array of `count` problems).
 * No counterpart in the reference, which solves one instance per call. */
int usbs_eigsh_smallest_batched(int count, const usbs_eigsh_problem* problems,
                                int inner_iterations, int max_restarts, double tolerance,
                                int precision, void* stream);

/* Cluster-size autotuner for the Lanczos launches (no counterpart in the
 * reference).  A cluster-path launch spreads its problems over
 * ceil(n_max / rows_per_cta) CTAs per cluster (at most 16): one problem
 * alone runs fastest spread thin, a batch or concurrent solves fastest packed.
 * usbs_lanczos_autotune runs the batch (as usbs_eigsh_smallest_batched, at
 * most 48 problems) once per candidate rows per CTA (64, 128, 256, 640, 1280;
 * candidates giving the same cluster size are skipped, their time -1), times
 * each with CUDA events on `stream` after a warm-up run, records the fastest
 * for the batch's class -- (precision, floor(log2(count)), floor(log2(max n)))
 * -- in a process-wide table that later launches of that class use, and
 * returns with the batch's outputs from the chosen candidate.  Host call that
 * waits for the device. */
int usbs_lanczos_autotune(int count, const usbs_eigsh_problem* problems, int inner_iterations,
                          int max_restarts, double tolerance, int precision, void* stream,
                          int* best_rows_per_cta, float* candidate_ms /* [5] or NULL */);
/* The table: entries as keys (precision << 32 | log2 count << 16 | log2 max n)
 * and rows per CTA; returns the number of entries (writes at most capacity). */
int usbs_lanczos_tuning_get(long long* keys, int* rows_per_cta, int capacity);
/* Sets (rows_per_cta >= 16) or erases (0) the entry of a class. */
int usbs_lanczos_tuning_put(int precision, int count, int max_n, int rows_per_cta);
void usbs_lanczos_tuning_clear(void);

/* ------------------------------------------------------------------ usbs()
 * One SDP instance, resident in device memory.  Field meanings follow the
 * reference's SDPState (utils/common.py:11-26) after scale_sdp_state. */
typedef struct usbs_problem {
  int n;                    /* order of X (C is n x n) */
  int m;                    /* number of constraints (len(b)) */
  long long nnz;            /* entries of the union pattern */
  int num_triples;
  const int* rowptr;        /* [n+1] union pattern */
  const int* col;           /* [nnz] */
  const double* c_val;      /* [nnz] C on the union pattern */
  const int* slot_ptr;      /* [nnz+1] */
  const int* slot_tid;      /* [num_triples] */
  const int* t_con;         /* [num_triples] caller order */
  const double* t_a0;       /* [num_triples] caller order */
  const int* con_ptr;       /* [m+1] triples sorted by constraint */
  const int* t_row;
  const int* t_col;
  const double* t_a;
  const int* row_ptr;       /* [n+1] triples sorted by row */
  const int* r_con;
  const int* r_col;
  const double* r_a;
  const double* b;          /* [m] */
  const double* b_ineq_mask;/* [m] 1.0 for "<=" rows */
  const double* scale_a;    /* [m] SCALE_A */
  double scale_c, scale_x;  /* SCALE_C, SCALE_X */
  double b_norm;            /* || (b / SCALE_A) / SCALE_X ||_2 (host-computed) */
  int has_ineq;             /* any b_ineq_mask != 0 */
} usbs_problem;

/* Solver settings: the arguments of usbs() (solver/usbs.py:436-459). */
typedef struct usbs_params {
  double trace_ub, trace_factor, rho, beta;
  int k_curr, k_past;       /* k = k_curr + k_past <= 12 */
  int max_iters;
  double max_time;          /* seconds of wall clock */
  double obj_gap_eps, infeas_gap_eps, max_infeas_eps;
  int lanczos_inner_iterations;  /* <= 32 */
  int lanczos_max_restarts;
  double subprob_eps;
  int subprob_max_iters;
  double cond_exp_base;     /* in [1, 2] */
  int precision;            /* 64: FP64 everywhere; 32: FP32 Lanczos + FP64 rest */
  int sketch_mode;          /* 0: Nystrom sketch P = X Omega, 1: dense X, 2: diag(X) only */
  int sketch_dim;           /* columns of Omega (mode 0) */
  int lanczos_rows_per_cta; /* cluster Lanczos: rows per CTA (>= 16); 0: the class's tuned
                               choice (usbs_lanczos_autotune), else 64 */
  int lanczos_path;         /* 0: the library's choice (usbs_lanczos_kernel); 2: a problem too
                               large for one cluster always takes the stream path, never the
                               cooperative launch, so the solve never needs the GPU to itself
                               (a service running several solves at once sets this) */
} usbs_params;

/* Iterate state (device arrays, column-major with leading dimension ld) and
 * host-side scalars.  y, z, P, X are read as the starting point and hold the
 * result on return; V receives the final bundle basis. */
typedef struct usbs_state {
  int ld;                   /* n rounded up to a multiple of 32 */
  double* y;                /* [m] */
  double* z;                /* [m] */
  double* V;                /* [ld x (k_curr + k_past)] */
  double* P;                /* mode 0: [ld x sketch_dim]; mode 2: [n] */
  double* Omega;            /* mode 0: [ld x sketch_dim] */
  double* X;                /* mode 1: [n x n] row-major */
  const double* q0;         /* [n] unit Lanczos start vector (solver/usbs.py:691-692) */
  double* trace;            /* optional [trace_capacity x 20] per-iteration record */
  int trace_capacity;
  double* debug;            /* optional [8192]: IPM histories of iteration 0 and phase cycles */
  double tr_X, primal_obj;  /* in: starting values; out: final values */
  /* outputs */
  int iterations;
  double obj_gap, infeas_gap, max_infeas, obj_ub, pen_dual_obj, elapsed;
  int status;               /* device status bits (see usbs_eigsh_smallest) */
  /* measurement (outputs): Lanczos launches of the outer loop, their CUDA-event
   * time on `stream`, their algorithmic bytes, and all kernel launches */
  int lanczos_launches;
  double lanczos_ms, lanczos_bytes;
  long long kernel_launches;
  /* the state at the latest condition check, written before the callback
   * runs, in the trace-record layout (usbs_solve: t, primal_obj, obj_ub,
   * obj_gap, infeas_gap, max_infeas, pen_dual_obj, cand_pen_dual_obj,
   * lb_spec_est, eig0, descent, eta, trS, tr_X, IPM iterations x2,
   * bar_primal_obj, tr_X_bar, b.y; usbs_cgal_solve: its first 8 trace fields);
   * the scaled problem's values, as the reference's cond_func sees them */
  double cond[20];
  /* outer iterations that ran as one launch of the captured CUDA graph of the
   * iteration (usbs_solve: problems without inequality constraints whose
   * Lanczos runs as one cluster; the others run eagerly); negative: the
   * capture failed with that CUDA error and every iteration ran eagerly */
  long long graph_iterations;
} usbs_state;

/* Called on the host at every condition check (after the device has caught
 * up), before the stop decision: the place for the reference's callback_fn
 * (solver/usbs.py:505-512). */
typedef void (*usbs_cond_callback)(void* user, int t);

/* Workspace bytes for usbs_solve (host call). */
size_t usbs_solve_workspace_bytes(const usbs_problem* problem, const usbs_params* params);

/* usbs() (solver/usbs.py:436-789): initial eigsh for the bundle, then at most
 * max_iters outer iterations while the reference's stop condition holds
 * (obj_gap, infeas_gap, max_infeas above their eps and time < max_time),
 * checking it on the cond_exp_base schedule (utils/loop.py:80-115).
 * Synchronous: returns when the loop has stopped. */
int usbs_solve(const usbs_problem* problem, const usbs_params* params, usbs_state* state,
               void* workspace, size_t workspace_bytes, usbs_cond_callback callback,
               void* callback_user, void* stream);

/* ------------------------------------------------------------------ cgal()
 * Settings of cgal() (solver/cgal.py:21-39). */
typedef struct usbs_cgal_params {
  double trace_ub, beta0;
  int max_iters;
  double max_time;          /* seconds of wall clock */
  double obj_gap_eps, infeas_gap_eps, max_infeas_eps;
  int lanczos_inner_iterations;  /* <= 32 */
  int lanczos_max_restarts;
  double subprob_eps;       /* Lanczos tolerance */
  double cond_exp_base;     /* in [1, 2] */
  int precision;            /* 64: FP64 everywhere; 32: FP32 Lanczos + FP64 rest */
  int sketch_mode;          /* 0: Nystrom sketch P = X Omega, 1: dense X */
  int sketch_dim;           /* columns of Omega (mode 0) */
} usbs_cgal_params;

/* Workspace bytes for usbs_cgal_solve (host call). */
size_t usbs_cgal_workspace_bytes(const usbs_problem* problem, const usbs_cgal_params* params);

/* cgal() (solver/cgal.py:21-243): CGAL iterations (one smallest eigenpair of
 * -C + A*(adj) per iteration, rank-one sketch update, dual step) until the
 * reference's stop condition holds, checked on the cond_exp_base schedule.
 * Uses y, z, P/Omega (mode 0) or X (mode 1), q0, tr_X and primal_obj of
 * `state` (V and debug are ignored); trace, if given, receives per iteration
 * [t, smallest eigenvalue, obj_gap, infeas_gap, max_infeas, primal_obj, tr_X,
 * dual step] in the first 8 of 20 doubles.  Synchronous. */
int usbs_cgal_solve(const usbs_problem* problem, const usbs_cgal_params* params,
                    usbs_state* state, void* workspace, size_t workspace_bytes,
                    usbs_cond_callback callback, void* callback_user, void* stream);

/* ---------------------------------------------------------------- rounding */

/* Workspace bytes of usbs_reconstruct_from_sketch / usbs_maxcut_round for n
 * rows and a sketch of s <= 32 columns (0 for unsupported sizes). */
size_t usbs_round_workspace_bytes(int n, int s);

/* reconstruct_from_sketch (utils/common.py:99-116): the Nystrom factors of
 * the sketch P = X Omega.  Omega and P are n x s, column-major with leading
 * dimension ld.  E (n x s, lde; may be NULL) receives the left singular
 * vectors of P_rho L^-T, Lambda (s; may be NULL) max(Rho^2 - rho, 0), both in
 * the reference's order (Rho descending; each column of E up to its sign).
 * Where B = sym(Omega^T P_rho) is not positive definite, E and Lambda are NaN
 * as jnp.linalg.cholesky makes them.  Stream-ordered; device pointers. */
int usbs_reconstruct_from_sketch(int n, int s, const double* Omega, const double* P, int ld,
                                 double approx_eps, double* E, int lde, double* Lambda,
                                 void* workspace, size_t workspace_bytes, void* stream);

/* compute_max_cut (utils/maxcut_helpers.py:292-302): *value (device) =
 * max_j w_j^T C w_j with w_j = +1 where column j of the reconstructed E is
 * positive and -1 elsewhere, for the CSR matrix C (the unscaled objective,
 * both triangles).  column_values (s; may be NULL) receives every w_j^T C w_j,
 * signs (n; may be NULL) the sign words (bit j set: +1).  approx_eps is the
 * reference's 1e-6.  Stream-ordered; device pointers. */
int usbs_maxcut_round(int n, int s, const double* Omega, const double* P, int ld,
                      const int* rowptr, const int* col, const double* val, double approx_eps,
                      double* value, double* column_values, unsigned* signs, void* workspace,
                      size_t workspace_bytes, void* stream);

/* Workspace bytes of usbs_qap_round for l facilities (l <= 64) and a sketch
 * of s <= 32 columns (0 for unsupported sizes). */
size_t usbs_qap_round_workspace_bytes(int l, int s);

/* qap_round (utils/qap_helpers.py:624-653): the QAP rounding callback.  Omega
 * and P are (l^2 + 1) x s, column-major with leading dimension ld; W (flow)
 * and D (distance) are l x l row-major.  For each of the first min(l, s)
 * columns of the reconstructed E and for its negative, an optimal assignment
 * of the cost max(c) - c (c = +-E[1:, i] as an l x l row-major matrix, row =
 * facility) and its objective trace(W P D P^T).  *value (device) = the
 * smaller of the minimum over the positive and over the negative candidates.
 * candidate_values (2 min(l, s) doubles, positive first) and candidate_perms
 * (2 min(l, s) x l ints: the location of each facility) may be NULL.
 * Stream-ordered; device pointers. */
int usbs_qap_round(int l, int s, const double* Omega, const double* P, int ld, const double* W,
                   const double* D, double approx_eps, double* value, double* candidate_values,
                   int* candidate_perms, void* workspace, size_t workspace_bytes, void* stream);

/* Self-test of the bounded device waits (no counterpart in the reference,
 * which has no device code).  Every spin-wait of the library's kernels gives
 * up after a time limit, ORs ST_BARRIER_TIMEOUT (1) into the caller's status
 * word and returns.  This call runs one such wait on a condition nothing
 * satisfies, for `limit_ns` (1 us .. 2 s):
 *   which 0: the cooperative team barrier, `nctas` (1..8) CTAs launched and
 *            nctas + 1 expected; `counters` = 2 device uints (cleared here);
 *   which 1: an mbarrier wait that no thread or copy completes (counters
 *            unused).
 * *status (device int) gains bit 1 once the launch ends.  Stream-ordered. */
int usbs_selftest_wait_limits(int which, int nctas, long long limit_ns, unsigned int* counters,
                              int* status, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* USBS_GB300_H */
