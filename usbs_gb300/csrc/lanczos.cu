// Thick-restart Lanczos (smallest eigenpairs) as one cooperative launch.
//
// Reference: solver/lanczos.py:80-236 (restart loop, CGS2 full
// reorthogonalisation, arrowhead projected matrix, gap-ratio restart choice).
//
// Layout and schedule.  The CTAs of the launch are split into teams, one team
// per problem.  A team owns a contiguous range of 256-row tiles of its problem;
// every phase below walks the same tiles, so a CTA only ever reads and writes
// its own rows of Q and of the work vectors, except for the SpMV gathers of x
// (read through L2 with ld.global.cg after a team barrier).  One Lanczos step i
// is three phases separated by team barriers:
//   A  y = Op x  (CSR, `lanes` threads per row) fused with h1 = Q[:, :i+1]^T y
//   B  q1 = y - Q h1, fused with h2 = Q^T q1
//   C  q2 = q1 - Q h2, fused with ||q2||^2
// The normalisation q2 / beta is folded into the next phase A (x = v * 1/beta),
// which also stores Q[:, i+1] for its rows.  Partial sums go to a per-team
// [pass][cta][column] buffer and every CTA reduces them in the same fixed order,
// so all CTAs hold bit-identical alpha/beta and take identical branches.
// At a restart CTA 0 builds the arrowhead matrix and runs the FP64 warp
// eigensolver; after a barrier every CTA rotates its rows of Q by the saved
// Ritz vectors.
#include <stdlib.h>
#include <map>
#include <mutex>
#include "common.cuh"
#include "dense.cuh"
#include "internal.h"

namespace usbs {

constexpr int LZ_BLOCK = 256;
constexpr int LZ_NW = LZ_BLOCK / 32;
constexpr int MAX_TEAMS = 48;
constexpr int MP1 = MAXM + 1;

constexpr int LZ_XS_BYTES = 160 * 1024;   // dynamic shared memory for a staged x

template <typename VT>
struct TeamDesc {
  int n, ld, m, num_desired, max_restarts, lanes, first_cta, nctas, xsmem;
  long long nnz;
  double tol;
  const int* rowptr;
  const int* col;
  const VT* val;
  VT* Q;                 // the caller's basis, ld x (m+1) column-major
  // working basis: element (c, row) at Qw[qix(c, row)] (here always Q:
  // tile stride LZ_BLOCK, column stride ld)
  VT* Qw;
  long long qts, qcs;    // tile and column strides (elements)
  // stream path: the operator in a sliced-ELL layout built on the device (rows
  // of each 256-row window sorted by length, 32-row slices, each slice
  // holding at most wcap entries per row; longer rows finish from the CSR)
  int wcap;
  int* sl_ptr;           // slice s: entries [sl_ptr[s], sl_ptr[s + 1]), column-major
  unsigned char* sl_row; // sorted position -> row offset inside its window
  int* sl_col;
  VT* sl_val;
  VT* vbuf;              // 3 flat vectors: two work vectors, then Q[:, k] of the cycle
  double* part;
  double* Ybuf;
  double* alpha;
  double* beta;
  int* ctl;
  unsigned int* bar;
  int* status;
};

template <typename VT>
__device__ __forceinline__ size_t qix(const TeamDesc<VT>& P, int c, int row) {
  return (size_t)(row / LZ_BLOCK) * (size_t)P.qts + (size_t)c * (size_t)P.qcs +
         (size_t)(row % LZ_BLOCK);
}

template <typename VT>
struct TeamBatch {
  int count;
  TeamDesc<VT> t[MAX_TEAMS];
};

template <typename VT>
struct LzShared {
  union {
    struct {                     // Lanczos step phases
      double ys[LZ_BLOCK];
      double wred[LZ_NW][MP1];
    } st;
    VT cys[LZ_BLOCK];            // cluster kernel: row results of the SpMV, in the vector type
    struct {                     // restart on CTA 0 (T, X, R, S, W row-major, ld MP1)
      double T[MAXM * MP1];
      double X[MAXM * MP1];
      double R[MAXM * MP1];      // float copy of T during the Jacobi sweeps
      double S[MAXM * MP1];      // float eigenvectors during the Jacobi sweeps
      double W[MAXM * MP1];
    } rs;
    VT Ys[MAXM * MAXM];          // saved Ritz vectors, every CTA, after the restart barrier
    double red4[4][MP1];         // cluster reduction: the four level-two sums
  } u;
  double h[MP1];
  VT hv[MP1];                    // h in the vector type, converted once per reduction
  double bnorm;                  // cluster kernel: sqrt(h[0]) of a norm reduction ...
  VT binv;                       // ... and 1 / bnorm in the vector type
  double alpha[MAXM];
  double beta[MAXM];
  double ritz[MAXM];
  double red[LZ_NW];
  float wf[MAXM], redf[32];
  int order[MAXM];
  int k_next, nconv;
  long long eig_cycles;          // cycles in the projected eigensolver (thread 0)
};

// acc[c] (c < nv) summed over the CTA, written to out[c * R] (column-major
// [column][cta] partial layout, so the team reduction reads each column in one
// coalesced load).  Columns 0..31 are reduced across each warp by one
// butterfly reduce-scatter (lane c ends with column c), column 32 by a warp sum.
template <typename SH, typename AT>
__device__ __forceinline__ void block_reduce_cols(AT* acc, int nv, SH& sh, double* out,
                                                  int R) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (nv == 1) {
    const AT v = warp_sum(acc[0]);
    if (lane == 0) sh.u.st.wred[wid][0] = (double)v;
  } else {
    const AT extra = (nv > 32) ? warp_sum(acc[32]) : (AT)0;
    const AT v = warp_reduce_scatter32(acc);
    sh.u.st.wred[wid][lane] = (double)v;
    if (lane == 0 && nv > 32) sh.u.st.wred[wid][32] = (double)extra;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nv; c += LZ_BLOCK) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < LZ_NW; ++w) s += sh.u.st.wred[w][c];
    out[(size_t)c * R] = s;
  }
}

// h[c] = sum over the team's CTAs of part_pass[c][r], identical order in every
// CTA.  Warp 0 issues all loads (lane l takes CTAs l, l+32, ...), then one
// butterfly reduce-scatter leaves column c in lane c.
template <typename VT>
__device__ __forceinline__ void reduce_part(const double* part_pass, int R, int nv,
                                            LzShared<VT>& sh) {
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < 32) {
    if (nv == 1) {
      double a = 0.0;
      for (int r = lane; r < R; r += 32) a += __ldcg(part_pass + r);
      a = warp_sum(a);
      if (lane == 0) { sh.h[0] = a; sh.hv[0] = (VT)a; }
    } else {
      double acc[32];
#pragma unroll
      for (int c = 0; c < 32; ++c) acc[c] = 0.0;
      double extra = 0.0;
      for (int r = lane; r < R; r += 32) {
#pragma unroll
        for (int c = 0; c < 32; ++c)
          if (c < nv) acc[c] += __ldcg(part_pass + (size_t)c * R + r);
        if (nv > 32) extra += __ldcg(part_pass + (size_t)32 * R + r);
      }
      extra = warp_sum(extra);
      const double v = warp_reduce_scatter32(acc);
      if (lane < nv) { sh.h[lane] = v; sh.hv[lane] = (VT)v; }
      if (lane == 0 && nv > 32) { sh.h[32] = extra; sh.hv[32] = (VT)extra; }
    }
  }
  __syncthreads();
}

// SpMV of one 256-row tile, L lanes per row: sh.u.st.ys[r] = (Op x)[base + r].
// Groups of up to 4 passes issue their rowptr loads, then their first col/val
// loads, before any result is used: two dependent L2 round trips per group
// instead of two per pass.
template <typename VT, int L, typename SH>
__device__ __forceinline__ void spmv_tile(const TeamDesc<VT>& P, SH& sh, int base,
                                          const VT* xsrc, const VT* xs, bool use_xs) {
  typedef typename Acc<VT>::type AT;
  constexpr int GPP = LZ_BLOCK / L;
  constexpr int CH = L < 4 ? L : 4;          // passes whose loads are issued together
  const int tid = threadIdx.x, g = tid / L, lig = tid - (tid / L) * L;
#pragma unroll 1
  for (int q0 = 0; q0 < L; q0 += CH) {
    int pb[CH], pe[CH];
#pragma unroll
    for (int q = 0; q < CH; ++q) {
      const int row = base + (q0 + q) * GPP + g;
      pb[q] = 0; pe[q] = 0;
      if (row < P.n) { pb[q] = P.rowptr[row] + lig; pe[q] = P.rowptr[row + 1]; }
    }
    int c0[CH];
    VT v0[CH];
#pragma unroll
    for (int q = 0; q < CH; ++q) {
      c0[q] = 0; v0[q] = (VT)0;
      if (pb[q] < pe[q]) { c0[q] = P.col[pb[q]]; v0[q] = P.val[pb[q]]; }
    }
#pragma unroll
    for (int q = 0; q < CH; ++q) {
      AT s = (AT)v0[q] * (AT)(use_xs ? xs[c0[q]] : __ldcg(xsrc + c0[q]));
      for (int p = pb[q] + L; p < pe[q]; p += L)
        s += (AT)P.val[p] * (AT)(use_xs ? xs[P.col[p]] : __ldcg(xsrc + P.col[p]));
#pragma unroll
      for (int o = L >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lig == 0) sh.u.st.ys[(q0 + q) * GPP + g] = (double)s;
    }
  }
}

// Phase A: y = Op (xsrc * xscale) for own rows -> vout, acc[c] = Q[:, c] . y (c <= i).
// If wq, also stores Q[:, i] = xsrc * xscale for own rows.
template <typename VT>
__device__ void phase_spmv(const TeamDesc<VT>& P, LzShared<VT>& sh, int t0, int t1, int i,
                           const VT* xsrc, VT xscale, bool wq, VT* vout, double* part_out) {
  typedef typename Acc<VT>::type AT;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  const int tid = threadIdx.x, L = P.lanes, gpp = LZ_BLOCK / L;
  const int g = tid / L, lig = tid - g * L;
  const size_t ld = (size_t)P.ld;
  // small vectors: stage x once in shared memory so the gathers skip L2
  extern __shared__ __align__(16) unsigned char lz_dyn[];
  VT* xs = (VT*)lz_dyn;
  const bool use_xs = P.xsmem != 0;
  if (use_xs) {
    // 16-byte loads, several in flight per thread (xsrc is a 256-byte aligned
    // vector buffer or a column of Q with ld a multiple of 32)
    constexpr int VE = 16 / (int)sizeof(VT);
    const int n16 = P.n / VE;
    const uint4* src = (const uint4*)xsrc;
    uint4* dst = (uint4*)xs;
    int j = tid;
    for (; j + 3 * LZ_BLOCK < n16; j += 4 * LZ_BLOCK) {
      const uint4 a = __ldcg(src + j), b = __ldcg(src + j + LZ_BLOCK),
                  c = __ldcg(src + j + 2 * LZ_BLOCK), d = __ldcg(src + j + 3 * LZ_BLOCK);
      dst[j] = a; dst[j + LZ_BLOCK] = b; dst[j + 2 * LZ_BLOCK] = c; dst[j + 3 * LZ_BLOCK] = d;
    }
    for (; j < n16; j += LZ_BLOCK) dst[j] = __ldcg(src + j);
    for (int r = n16 * VE + tid; r < P.n; r += LZ_BLOCK) xs[r] = __ldcg(xsrc + r);
    __syncthreads();
  }
  (void)gpp; (void)g; (void)lig;
  for (int tile = t0; tile < t1; ++tile) {
    const int base = tile * LZ_BLOCK;
    switch (L) {
      case 1: spmv_tile<VT, 1>(P, sh, base, xsrc, xs, use_xs); break;
      case 2: spmv_tile<VT, 2>(P, sh, base, xsrc, xs, use_xs); break;
      case 4: spmv_tile<VT, 4>(P, sh, base, xsrc, xs, use_xs); break;
      case 8: spmv_tile<VT, 8>(P, sh, base, xsrc, xs, use_xs); break;
      case 16: spmv_tile<VT, 16>(P, sh, base, xsrc, xs, use_xs); break;
      default: spmv_tile<VT, 32>(P, sh, base, xsrc, xs, use_xs); break;
    }
    __syncthreads();
    const int row = base + tid;
    if (row < P.n) {
      const VT y = (VT)sh.u.st.ys[tid] * xscale;
      vout[row] = y;
      VT xn = (VT)0;
      if (wq) {
        xn = __ldcg(xsrc + row) * xscale;
        P.Qw[qix(P, i, row)] = xn;
      }
#pragma unroll
      for (int c = 0; c < MP1; ++c) {
        if (c <= i) {
          const VT qc = (wq && c == i) ? xn : P.Qw[qix(P, c, row)];
          acc[c] += (AT)qc * (AT)y;
        }
      }
    }
    __syncthreads();
  }
  block_reduce_cols(acc, i + 1, sh, part_out, P.nctas);
}

// Breakdown pass a: buf = hash_normal(key) for own rows, acc[c] = Q[:, c] . buf (c < nv)
template <typename VT, typename SH>
__device__ void phase_random(const TeamDesc<VT>& P, SH& sh, int t0, int t1, int nv,
                             uint64_t key, VT* buf, double* part_out) {
  typedef typename Acc<VT>::type AT;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  const size_t ld = (size_t)P.ld;
  for (int tile = t0; tile < t1; ++tile) {
    const int row = tile * LZ_BLOCK + threadIdx.x;
    if (row < P.n) {
      const VT r = (VT)hash_normal(key, (uint64_t)row);
      buf[row] = r;
#pragma unroll
      for (int c = 0; c < MP1; ++c)
        if (c < nv) acc[c] += (AT)P.Qw[qix(P, c, row)] * (AT)r;
    }
  }
  block_reduce_cols(acc, nv, sh, part_out, P.nctas);
}

// Phase B: buf -= Q h (c < nv); acc[c] = Q[:, c] . buf
template <typename VT, typename SH>
__device__ void phase_update_dot(const TeamDesc<VT>& P, SH& sh, int t0, int t1, int nv,
                                 VT* buf, double* part_out) {
  typedef typename Acc<VT>::type AT;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  const size_t ld = (size_t)P.ld;
  for (int tile = t0; tile < t1; ++tile) {
    const int row = tile * LZ_BLOCK + threadIdx.x;
    if (row < P.n) {
      VT qr[MP1];
      VT s = (VT)0;
#pragma unroll
      for (int c = 0; c < MP1; ++c) {
        if (c < nv) {
          qr[c] = P.Qw[qix(P, c, row)];
          s += qr[c] * sh.hv[c];
        }
      }
      const VT q1 = buf[row] - s;
      buf[row] = q1;
#pragma unroll
      for (int c = 0; c < MP1; ++c)
        if (c < nv) acc[c] += (AT)qr[c] * (AT)q1;
    }
  }
  block_reduce_cols(acc, nv, sh, part_out, P.nctas);
}

// Phase C: buf -= Q h (c < nv); part_out[0] = sum buf^2 over own rows
template <typename VT, typename SH>
__device__ void phase_update_norm(const TeamDesc<VT>& P, SH& sh, int t0, int t1, int nv,
                                  VT* buf, double* part_out) {
  typedef typename Acc<VT>::type AT;
  AT nrm = (AT)0;
  const size_t ld = (size_t)P.ld;
  for (int tile = t0; tile < t1; ++tile) {
    const int row = tile * LZ_BLOCK + threadIdx.x;
    if (row < P.n) {
      VT s = (VT)0;
#pragma unroll
      for (int c = 0; c < MP1; ++c)
        if (c < nv) s += P.Qw[qix(P, c, row)] * sh.hv[c];
      const VT q2 = buf[row] - s;
      buf[row] = q2;
      nrm += (AT)q2 * (AT)q2;
    }
  }
  AT one[MP1];
  one[0] = nrm;
  block_reduce_cols(one, 1, sh, part_out, P.nctas);
}

// CTA 0 of a team: projected eigenproblem and thick-restart selection
// (solver/lanczos.py:128-168, 202-221).  k = number of saved vectors of the
// finished cycle, beta_last = beta[m-1].
// LOCAL_YS: every CTA of a cluster runs this redundantly (identical inputs give
// identical results) and keeps the saved Ritz vectors in sh.u.Ys; only the CTA
// with write_out set stores alpha/beta/ctl.  Otherwise (team kernel) the Ritz
// vectors go through P.Ybuf.
template <bool LOCAL_YS, typename VT, typename D>
__device__ void restart_select(const D& P, LzShared<VT>& sh, int k, bool write_out = true) {
  const int m = P.m, tid = threadIdx.x;
  double* T = sh.u.rs.T;
  double* X = sh.u.rs.X;
  float* Tf = (float*)sh.u.rs.R;
  float* Zf = (float*)sh.u.rs.S;
  for (int e = tid; e < m * m; e += LZ_BLOCK) {
    const int r = e / m, c = e - r * m;
    double v = 0.0;
    if (r == c) v = sh.alpha[r];
    else if (c == k && r < k) v = sh.beta[r];
    else if (r == k && c < k) v = sh.beta[c];
    else if (c == r + 1 && r >= k) v = sh.beta[r];
    else if (r == c + 1 && c >= k) v = sh.beta[c];
    T[r * MP1 + c] = v;
    Tf[r * MP1 + c] = (float)v;
  }
  __syncthreads();
  // eigh(T) (solver/lanczos.py:203): FP32 parallel Jacobi by the CTA ...
  {
    const long long c0 = clock64();
    const bool ok = cta_jacobi_f32<32>(Tf, (float*)sh.u.rs.W, MP1, m, sh.wf, Zf, MP1, sh.redf);
    if (tid == 0) sh.eig_cycles += clock64() - c0;
    if (!ok && tid == 0) atomicOr(P.status, ST_SMALL_DENSE_FAIL);
  }
  for (int e = tid; e < m * m; e += LZ_BLOCK) {
    const int r = e / m, c = e - r * m;
    X[r * MP1 + c] = (double)Zf[r * MP1 + c];
  }
  if (tid < m) sh.ritz[tid] = (double)sh.wf[tid];
  __syncthreads();
  if (sizeof(VT) == 8) {
    // ... refined to FP64 accuracy by two Ogita-Aishima steps, then re-sorted
    cta_refine_eig(T, X, sh.u.rs.R, sh.u.rs.S, sh.u.rs.W, sh.ritz, sh.red, m, MP1);
    cta_refine_eig(T, X, sh.u.rs.R, sh.u.rs.S, sh.u.rs.W, sh.ritz, sh.red, m, MP1);
    if (tid == 0) {
      for (int i = 0; i < m; ++i) sh.order[i] = i;
      for (int i = 0; i < m - 1; ++i) {
        int kmin = i;
        for (int j = i + 1; j < m; ++j)
          if (sh.ritz[sh.order[j]] < sh.ritz[sh.order[kmin]]) kmin = j;
        const int t = sh.order[i]; sh.order[i] = sh.order[kmin]; sh.order[kmin] = t;
      }
    }
    __syncthreads();
    double* Sx = sh.u.rs.S;
    for (int e = tid; e < m * m; e += LZ_BLOCK) {
      const int r = e / m, c = e - r * m;
      Sx[r * MP1 + c] = X[r * MP1 + sh.order[c]];
    }
    double rv = (tid < m) ? sh.ritz[sh.order[tid]] : 0.0;
    __syncthreads();
    for (int e = tid; e < m * m; e += LZ_BLOCK) {
      const int r = e / m, c = e - r * m;
      X[r * MP1 + c] = Sx[r * MP1 + c];
    }
    if (tid < m) sh.ritz[tid] = rv;
    __syncthreads();
  }
  const double* Z = X;
  if (tid == 0) {
    // a NaN / Inf in the projected matrix (e.g. from a non-finite operator)
    // ends the call after this restart with ST_NONFINITE
    bool fin = true;
    for (int c = 0; c < m; ++c) fin = fin && isfinite(sh.alpha[c]) && isfinite(sh.beta[c]);
    if (!fin) atomicOr(P.status, ST_NONFINITE);
    const double bl = sh.beta[m - 1];
    int nconv = m;
    for (int c = 0; c < m; ++c) {
      if (!(bl * fabs(Z[(m - 1) * MP1 + c]) < P.tol)) { nconv = c; break; }
    }
    const int delta = min(m - P.num_desired, 2 * (m - nconv) / 5);
    const double lt = sh.ritz[min(nconv, m - 1)];
    int kl = 0;
    double bv = 0.0;
    for (int c = 0; c < m; ++c) {
      const int kr = c + delta;
      double g = 0.0;
      if (kr <= m) g = (sh.ritz[c] - lt) / (sh.ritz[min(kr, m - 1)] - lt);
      if (c == 0) { bv = g; kl = 0; if (isnan(g)) break; continue; }
      if (isnan(g)) { kl = c; break; }
      if (g > bv) { bv = g; kl = c; }
    }
    const int kright = kl + delta;
    int kn = 0;
    for (int c = 0; c < m; ++c)
      if (kl >= c || kright < c) sh.order[kn++] = c;
    int pos = kn;
    for (int c = 0; c < m; ++c)
      if (!(kl >= c || kright < c)) sh.order[pos++] = c;
    sh.k_next = kn;
    sh.nconv = nconv;
  }
  __syncthreads();
  const int kn = sh.k_next;
  const double bl = sh.beta[m - 1];
  if constexpr (LOCAL_YS) {
    // sh.u.Ys overlays sh.u.rs.T only (T is no longer needed; Z lives in X)
    for (int e = tid; e < m * MAXM; e += LZ_BLOCK) {
      const int j = e / MAXM, c = e - j * MAXM;
      sh.u.Ys[e] = (c < kn) ? (VT)Z[j * MP1 + sh.order[c]] : (VT)0;
    }
  } else {
    for (int e = tid; e < m * m; e += LZ_BLOCK) {
      const int j = e / m, c = e - j * m;
      P.Ybuf[j * m + c] = Z[j * MP1 + sh.order[c]];
    }
  }
  __syncthreads();
  if (tid < m) {
    const int c = tid;
    const double a = (c < kn) ? sh.ritz[sh.order[c]] : 0.0;
    const double b = (c < kn) ? bl * Z[(m - 1) * MP1 + sh.order[c]] : 0.0;
    sh.alpha[c] = a;
    sh.beta[c] = b;
    if (write_out) {
      P.alpha[c] = a;
      P.beta[c] = b;
    }
  }
  if (tid == 0 && write_out) {
    P.ctl[0] = kn;
    P.ctl[1] = sh.nconv;
  }
  __syncthreads();
}

template <typename VT>
__global__ void __launch_bounds__(LZ_BLOCK, 1)
lanczos_team_kernel(const __grid_constant__ TeamBatch<VT> batch) {
  __shared__ LzShared<VT> sh;
  int team = 0;
  for (int t = 1; t < batch.count; ++t)
    if ((int)blockIdx.x >= batch.t[t].first_cta) team = t;
  const TeamDesc<VT>& P = batch.t[team];
  const int rank = (int)blockIdx.x - P.first_cta, R = P.nctas;
  const int tid = threadIdx.x;
  TeamBarrier bar{P.bar, R, P.status};
  auto team_sync = [&]() -> bool { return bar.sync(); };
  const int n = P.n, m = P.m;
  const size_t ld = (size_t)P.ld;
  const int ntiles = (n + LZ_BLOCK - 1) / LZ_BLOCK;
  const int t0 = (int)((long long)ntiles * rank / R);
  const int t1 = (int)((long long)ntiles * (rank + 1) / R);
  // [pass][column][cta] partial sums
  double* part0 = P.part;
  double* part1 = P.part + (size_t)R * MP1;
  double* part2 = P.part + (size_t)2 * R * MP1;

  int k = 0, nconv = 0, restart = 0, breakdowns = 0, steps = 0, sum_nv = 0, sum_kn = 0;
  long long clk_start = clock64(), clk_restart = 0;
  // rank-0 phase accounting: [0] barrier waits, [1] team reductions, [2..4] phases A..C
  long long tp[5] = {0, 0, 0, 0, 0}, tmark = clock64();
  const bool timing = (rank == 0 && tid == 0);
#define LZ_MARK(slot)                                   \
  do {                                                  \
    if (timing) {                                       \
      const long long _c = clock64();                   \
      tp[slot] += _c - tmark;                           \
      tmark = _c;                                       \
    }                                                   \
  } while (0)
  if (rank == 0 && tid < MAXM) { sh.alpha[tid] = 0.0; sh.beta[tid] = 0.0; }
  if (tid == 0) sh.eig_cycles = 0;
  // the start vector Q[:, 0]: flat copy for the first cycle's gathers
  VT* xk = P.vbuf + 2 * ld;
  for (int tile = t0; tile < t1; ++tile) {
    const int row = tile * LZ_BLOCK + tid;
    if (row < n) xk[row] = P.Q[row];
  }
  __syncthreads();
  if (!team_sync()) return;
  int prev = 0;          // vbuf slot holding the latest unnormalised vector
  VT invb = (VT)1;       // its normalisation
  while (nconv < P.num_desired && restart < P.max_restarts) {
    int cur = 0;
    for (int i = k; i < m; ++i) {
      const VT* xsrc;
      bool wq;
      if (i == k) {
        xsrc = xk;       // = Q[:, k]
        invb = (VT)1;
        wq = false;
      } else {
        reduce_part(part2, R, 1, sh);
        const double b = sqrt(sh.h[0]);
        if (rank == 0 && tid == 0) sh.beta[i - 1] = b;
        if (b < 1e-15) {
          // Krylov space exhausted: random vector orthogonalised twice
          // against Q[:, :i] (solver/lanczos.py:107-117)
          ++breakdowns;
          VT* buf = P.vbuf + (size_t)prev * ld;
          phase_random(P, sh, t0, t1, i, (uint64_t)i, buf, part0 + rank);
          if (!team_sync()) return;
          reduce_part(part0, R, i, sh);
          phase_update_dot(P, sh, t0, t1, i, buf, part1 + rank);
          if (!team_sync()) return;
          reduce_part(part1, R, i, sh);
          phase_update_norm(P, sh, t0, t1, i, buf, part2 + rank);
          if (!team_sync()) return;
          reduce_part(part2, R, 1, sh);
          invb = (VT)(1.0 / sqrt(sh.h[0]));
        } else {
          invb = (VT)(1.0 / b);
        }
        xsrc = P.vbuf + (size_t)prev * ld;
        wq = true;
      }
      VT* vout = P.vbuf + (size_t)cur * ld;
      LZ_MARK(1);
      phase_spmv(P, sh, t0, t1, i, xsrc, invb, wq, vout, part0 + rank);
      LZ_MARK(2);
      if (!team_sync()) return;
      LZ_MARK(0);
      reduce_part(part0, R, i + 1, sh);
      LZ_MARK(1);
      const double h1i = sh.h[i];
      phase_update_dot(P, sh, t0, t1, i + 1, vout, part1 + rank);
      LZ_MARK(3);
      if (!team_sync()) return;
      LZ_MARK(0);
      reduce_part(part1, R, i + 1, sh);
      LZ_MARK(1);
      if (rank == 0 && tid == 0) sh.alpha[i] = h1i + sh.h[i];
      phase_update_norm(P, sh, t0, t1, i + 1, vout, part2 + rank);
      LZ_MARK(4);
      if (!team_sync()) return;
      LZ_MARK(0);
      prev = cur;
      cur ^= 1;
      ++steps;
      sum_nv += i + 1;
    }
    // ---- restart ----
    const bool stepped = (k < m);
    if (stepped) {
      reduce_part(part2, R, 1, sh);
      const double b = sqrt(sh.h[0]);
      if (rank == 0 && tid == 0) sh.beta[m - 1] = b;
      if (b < 1e-15) {
        ++breakdowns;
        VT* buf = P.vbuf + (size_t)prev * ld;
        phase_random(P, sh, t0, t1, m, (uint64_t)m, buf, part0 + rank);
        if (!team_sync()) return;
        reduce_part(part0, R, m, sh);
        phase_update_dot(P, sh, t0, t1, m, buf, part1 + rank);
        if (!team_sync()) return;
        reduce_part(part1, R, m, sh);
        phase_update_norm(P, sh, t0, t1, m, buf, part2 + rank);
        if (!team_sync()) return;
        reduce_part(part2, R, 1, sh);
        invb = (VT)(1.0 / sqrt(sh.h[0]));
      } else {
        invb = (VT)(1.0 / b);
      }
    }
    __syncthreads();
    if (rank == 0) {
      const long long c0 = clock64();
      restart_select<false>(P, sh, k);
      clk_restart += clock64() - c0;
    }
    if (!team_sync()) return;
    if (__ldcg(P.status) & ST_NONFINITE) { ++restart; break; }
    const int kn = __ldcg(P.ctl + 0);
    nconv = __ldcg(P.ctl + 1);
    for (int e = tid; e < m * MAXM; e += LZ_BLOCK) {
      const int j = e / MAXM, c = e - j * MAXM;
      sh.u.Ys[e] = (c < kn) ? (VT)__ldcg(P.Ybuf + j * m + c) : (VT)0;
    }
    __syncthreads();
    const VT* lastv = P.vbuf + (size_t)prev * ld;
    for (int tile = t0; tile < t1; ++tile) {
      const int row = tile * LZ_BLOCK + tid;
      if (row < n) {
        VT qr[MAXM];
#pragma unroll
        for (int j = 0; j < MAXM; ++j) qr[j] = (j < m) ? P.Qw[qix(P, j, row)] : (VT)0;
        const VT xl = stepped ? lastv[row] * invb : P.Qw[qix(P, m, row)];
        for (int c = 0; c < kn; ++c) {
          if (c >= m) break;
          VT s = (VT)0;
#pragma unroll
          for (int j = 0; j < MAXM; ++j)
            if (j < m) s += qr[j] * sh.u.Ys[j * MAXM + c];
          P.Qw[qix(P, c, row)] = s;
        }
        P.Qw[qix(P, kn, row)] = xl;
        if (kn != m) P.Qw[qix(P, m, row)] = xl;
        xk[row] = xl;
      }
    }
    k = kn;
    sum_kn += kn;
    ++restart;
    if (!team_sync()) return;
    if (timing) tmark = clock64();   // restart time is reported separately (ctl[6])
  }
  if (rank == 0 && tid == 0) {
    P.ctl[2] = restart;
    P.ctl[3] = breakdowns;
    P.ctl[4] = steps;
    P.ctl[6] = (int)(clk_restart >> 10);
    P.ctl[7] = (int)((clock64() - clk_start) >> 10);
    for (int j = 0; j < 5; ++j) P.ctl[8 + j] = (int)(tp[j] >> 10);
    P.ctl[13] = sum_nv;
    P.ctl[14] = sum_kn;
    P.ctl[15] = (int)(sh.eig_cycles >> 10);
    if (restart == 0) P.ctl[0] = 0;
  }
}

// ---------------------------------------------------------------- stream path
// Problems whose x does not fit in shared memory (n * sizeof(VT) > 160 KB) run
// as a sequence of ordinary full-GPU launches instead of one cooperative
// launch: every Lanczos step is
//   A1  y = Op x for one 256-row window per CTA on a sliced-ELL copy of the
//       operator built at the call's start, x = v * 1/beta folded in; also
//       stores Q[:, i] = x                           (no partial sums)
//   A2  h1 = Q[:, :i+1]^T y                          (partials, last-CTA sum)
//   B   q1 = y - Q h1,  h2 = Q^T q1                  (partials, last-CTA sum)
//   C   q2 = q1 - Q h2, ||q2||^2                     (partials, last-CTA sum)
// and a restart is one CTA's projected eigensolve and selection followed by a
// full-GPU rotation of the basis.  A kernel boundary is the grid-wide
// barrier, so no CTA ever waits on another and the kernels may share the GPU
// with other work.  Each CTA writes its partial sums to [column][cta]; the
// last CTA to finish (an atomic ticket after a fence) sums them in CTA order,
// so the result does not depend on which CTA is last.  The loop state lives
// in a device control block (StreamCtl) that only those last CTAs and the
// restart kernel write: every kernel of a step reads the same state at its
// start and derives the same mode (step, breakdown replacement, or nothing
// to do), so the host enqueues a cycle's launches without reading anything
// back, and reads the block once per restart.
struct __align__(16) StreamCtl {
  int i, k, bd, cur;           // step, saved vectors, breakdown pending, work vector in use
  int stop, rot, stepped;      // loop ended; rotation pending; the finished cycle had steps
  int restarts, breakdowns, steps, sum_nv, sum_kn, nconv;
  unsigned ticket[4];          // last-CTA tickets of A2, B, C and the rotation
  double invb;                 // 1 / beta of the latest unnormalised vector
  double h1[MP1], h2[MP1];
  double alpha[MAXM], beta[MAXM];
};

template <typename VT>
struct StShared {
  union {
    struct {
      double ys[LZ_BLOCK];
      double wred[LZ_NW][MP1];
    } st;
    __align__(16) VT Ys[MAXM * MAXM];
  } u;
  double h[MP1];
  VT hv[MP1];
  int last;
};

enum { SM_SKIP = 0, SM_STEP = 1, SM_BREAKDOWN = 2 };

// the step's mode from the control block's first eight ints (i, k, bd, cur,
// stop, rot, ...; the same in every kernel of a step), read as two 16-byte
// loads in one round trip
__device__ __forceinline__ int st_mode_of(int4 a, int4 b, int m, int* i, int* nv, int* buf) {
  const int ii = a.x, bd = a.z, cur = a.w, stop = b.x, rot = b.y;
  *i = ii;
  if (stop || rot) return SM_SKIP;
  if (bd) { *nv = ii; *buf = cur ^ 1; return SM_BREAKDOWN; }
  if (ii < m) { *nv = ii + 1; *buf = cur; return SM_STEP; }
  return SM_SKIP;
}
// Reads of the control block go through the read-only (L1) path: within a
// kernel only its last CTA writes the block, after every other CTA has
// finished, and the L1 caches start empty at each launch.  (Through L2 alone,
// every warp of every CTA would queue on the same L2 line.)
__device__ __forceinline__ int st_mode(const StreamCtl* c, int m, int* i, int* nv, int* buf) {
  const int4* p = (const int4*)c;
  return st_mode_of(__ldg(p), __ldg(p + 1), m, i, nv, buf);
}

// Programmatic dependent launch: each stream kernel lets the next one in the
// stream launch as soon as all of its own CTAs have started, then waits until
// the previous kernel has finished and its writes are visible.  The next
// kernel's launch thus overlaps this one's tail; no data is read early.
__device__ __forceinline__ void st_pdl_prologue() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ticket of the last CTA: true in every thread of the CTA that finished last
// (its partial sums, fenced by their writers, are then visible to it)
template <typename SH>
__device__ __forceinline__ bool st_last_cta(unsigned* ticket, SH& sh) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) sh.last = (atomicAdd(ticket, 1u) == gridDim.x - 1) ? 1 : 0;
  __syncthreads();
  if (sh.last) __threadfence();
  return sh.last != 0;
}

// h[c] = sum over the R CTAs of part[c][r], c < nv: warp w takes columns
// w, w + 8, ...; lane l sums CTAs l, l + 32, ... in order, then a butterfly
template <typename VT, typename SH>
__device__ __forceinline__ void st_reduce(const double* part, int R, int nv, SH& sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int c = w; c < nv; c += LZ_NW) {
    const double* p = part + (size_t)c * R;
    double a0 = 0.0, a1 = 0.0;
    int r = lane;
    for (; r + 32 < R; r += 64) { a0 += __ldcg(p + r); a1 += __ldcg(p + r + 32); }
    if (r < R) a0 += __ldcg(p + r);
    const double a = warp_sum(a0 + a1);
    if (lane == 0) { sh.h[c] = a; sh.hv[c] = (VT)a; }
  }
  __syncthreads();
}

// ---- vector helpers of the Q-streaming kernels ----
// 4 consecutive rows of a column (16-byte aligned: ld is a multiple of 32 and
// the first row a multiple of 4); rows at or past n read as 0.  The basis is
// read through the read-only path (no stream kernel writes a column it
// reads); the work vectors, which B and C update, through L2.
template <typename VT> struct Row4 { VT v[4]; };
template <typename VT, bool RO = true>
__device__ __forceinline__ Row4<VT> ld4(const VT* p, int r4, int n) {
  Row4<VT> o;
  if (r4 + 4 <= n) {
    if constexpr (sizeof(VT) == 4) {
      const float4 a = RO ? __ldg((const float4*)(p + r4)) : __ldcg((const float4*)(p + r4));
      o.v[0] = a.x; o.v[1] = a.y; o.v[2] = a.z; o.v[3] = a.w;
    } else {
      const double2 a = RO ? __ldg((const double2*)(p + r4)) : __ldcg((const double2*)(p + r4));
      const double2 b =
          RO ? __ldg((const double2*)(p + r4 + 2)) : __ldcg((const double2*)(p + r4 + 2));
      o.v[0] = a.x; o.v[1] = a.y; o.v[2] = b.x; o.v[3] = b.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      o.v[j] = (r4 + j < n) ? (RO ? __ldg(p + r4 + j) : __ldcg(p + r4 + j)) : (VT)0;
  }
  return o;
}
template <typename VT>
__device__ __forceinline__ void st4(VT* p, int r4, int n, const Row4<VT>& o) {
  if (r4 + 4 <= n) {
    if constexpr (sizeof(VT) == 4) {
      *(float4*)(p + r4) = make_float4(o.v[0], o.v[1], o.v[2], o.v[3]);
    } else {
      *(double2*)(p + r4) = make_double2(o.v[0], o.v[1]);
      *(double2*)(p + r4 + 2) = make_double2(o.v[2], o.v[3]);
    }
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (r4 + j < n) p[r4 + j] = o.v[j];
  }
}

constexpr int ST_ROWS = 4 * LZ_BLOCK;   // rows of one chunk (4 per thread)
// column loads issued before any is used: 128 bytes per thread either way
template <typename VT> constexpr int st_batch() { return sizeof(VT) == 4 ? 8 : 4; }

// s = sum_{c < nv} Q[r4.., c] * hv[c] for a thread's 4 rows, in column
// order, st_batch() column loads in flight at a time
template <typename VT>
__device__ __forceinline__ Row4<VT> st_combine(const VT* Q, size_t ld, int r4, int n, int nv,
                                               const VT* hv) {
  constexpr int NB = st_batch<VT>();
  Row4<VT> s;
#pragma unroll
  for (int j = 0; j < 4; ++j) s.v[j] = (VT)0;
#pragma unroll 1
  for (int c0 = 0; c0 < nv; c0 += NB) {
    Row4<VT> q[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b)
      if (c0 + b < nv) q[b] = ld4(Q + (size_t)(c0 + b) * ld, r4, n);
#pragma unroll
    for (int b = 0; b < NB; ++b)
      if (c0 + b < nv) {
        const VT h = hv[c0 + b];
#pragma unroll
        for (int j = 0; j < 4; ++j) s.v[j] += q[b].v[j] * h;
      }
  }
  return s;
}

// sacc[c][tid] += sum_j Q[r4 + j, c] * x.v[j], c < nv (a per-thread column of
// shared memory), st_batch() loads in flight at a time
template <typename VT, typename AT>
__device__ __forceinline__ void st_dots(const VT* Q, size_t ld, int r4, int n, int nv,
                                        const Row4<VT>& x, AT* sacc) {
  constexpr int NB = st_batch<VT>();
#pragma unroll 1
  for (int c0 = 0; c0 < nv; c0 += NB) {
    Row4<VT> q[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b)
      if (c0 + b < nv) q[b] = ld4(Q + (size_t)(c0 + b) * ld, r4, n);
#pragma unroll
    for (int b = 0; b < NB; ++b)
      if (c0 + b < nv) {
        AT d = (AT)0;
#pragma unroll
        for (int j = 0; j < 4; ++j) d += (AT)q[b].v[j] * (AT)x.v[j];
        sacc[(c0 + b) * LZ_BLOCK + threadIdx.x] += d;
      }
  }
}

// out[c * R] = sum over the CTA's threads of sacc[c][t], c < nv: warp w takes
// columns w, w + 8, ...; lane l sums threads l, l + 32, ... in order
template <typename AT>
__device__ __forceinline__ void st_block_cols(const AT* sacc, int nv, double* out, int R) {
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int c = w; c < nv; c += LZ_NW) {
    AT a = (AT)0;
#pragma unroll
    for (int k = 0; k < LZ_BLOCK / 32; ++k) a += sacc[c * LZ_BLOCK + lane + 32 * k];
    a = warp_sum(a);
    if (lane == 0) out[(size_t)c * R] = (double)a;
  }
}

// the per-thread dot accumulators of A2 and B (dynamic shared memory)
template <typename VT>
constexpr size_t st_sacc_bytes() {
  return (size_t)MP1 * LZ_BLOCK * sizeof(typename Acc<VT>::type);
}

// chunk range [c0, c1) of ST_ROWS-row chunks of this CTA
__device__ __forceinline__ void st_chunks(int n, int* c0, int* c1) {
  const int nch = (n + ST_ROWS - 1) / ST_ROWS, R = gridDim.x;
  *c0 = (int)((long long)nch * blockIdx.x / R);
  *c1 = (int)((long long)nch * (blockIdx.x + 1) / R);
}

// ---- the stream path's operator layout (built once per call) ----
// Rows of each 256-row window are ordered by length (longest first, then by
// row) and cut into 32-row slices; slice s keeps entry k of its lane-th row at
// sl_ptr[s] + 32 k + lane for k below the slice's width (its longest row's
// length, at most wcap; shorter rows are padded with column 0, value 0; rows
// longer than wcap finish from the CSR).  Three launches: the order and the
// widths per window, a prefix sum of the slice sizes, the entries.
template <typename VT>
__global__ void __launch_bounds__(LZ_BLOCK) st_sell_order_kernel(
    const __grid_constant__ TeamDesc<VT> P) {
  __shared__ int len[LZ_BLOCK];
  __shared__ int order[LZ_BLOCK];
  const int w0 = blockIdx.x * LZ_BLOCK, tid = threadIdx.x, r = w0 + tid;
  const int rows = min(LZ_BLOCK, P.n - w0);
  len[tid] = (r < P.n) ? P.rowptr[r + 1] - P.rowptr[r] : -1;
  __syncthreads();
  if (tid < rows) {
    const int mine = len[tid];
    int rank = 0;
    for (int j = 0; j < rows; ++j) {
      const int lj = len[j];
      rank += (lj > mine || (lj == mine && j < tid)) ? 1 : 0;
    }
    order[rank] = tid;
  }
  __syncthreads();
  // thread p: sorted position p of the window (slice p / 32, lane p % 32).  A
  // slice that exists (s < ceil(n / 32)) has a real row at its first position.
  const int p = tid, s = blockIdx.x * (LZ_BLOCK / 32) + p / 32, lane = p & 31;
  if (s >= (P.n + 31) / 32) return;
  const int lr = (p < rows) ? order[p] : p;      // padding lanes: unused positions
  P.sl_row[32 * s + lane] = (unsigned char)lr;
  if (lane == 0) P.sl_ptr[s + 1] = 32 * min(len[order[p]], P.wcap);
}

// sl_ptr[1..ns] (slice sizes) -> offsets, sl_ptr[0] = 0; one CTA of 1024
__global__ void __launch_bounds__(1024) st_sell_scan_kernel(int ns, int* sl_ptr) {
  __shared__ int part[1024];
  const int tid = threadIdx.x, per = (ns + 1023) / 1024;
  const int t0 = min(tid * per, ns), t1 = min(t0 + per, ns);
  int sum = 0;
  for (int i = t0; i < t1; ++i) sum += sl_ptr[i + 1];
  part[tid] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int v = tid >= off ? part[tid - off] : 0;
    __syncthreads();
    part[tid] += v;
    __syncthreads();
  }
  int base = tid ? part[tid - 1] : 0;
  for (int i = t0; i < t1; ++i) {
    base += sl_ptr[i + 1];
    sl_ptr[i + 1] = base;
  }
  if (tid == 0) sl_ptr[0] = 0;
}

template <typename VT>
__global__ void __launch_bounds__(LZ_BLOCK) st_sell_fill_kernel(
    const __grid_constant__ TeamDesc<VT> P) {
  const int w0 = blockIdx.x * LZ_BLOCK, p = threadIdx.x;
  const int s = blockIdx.x * (LZ_BLOCK / 32) + p / 32, lane = p & 31;
  if (s >= (P.n + 31) / 32) return;
  const int base = P.sl_ptr[s], w = (P.sl_ptr[s + 1] - base) >> 5;
  const int r = w0 + P.sl_row[32 * s + lane];
  const int b = (r < P.n) ? P.rowptr[r] : 0;
  const int lenr = (r < P.n) ? P.rowptr[r + 1] - b : 0;
  int* cdst = P.sl_col + base + lane;
  VT* vdst = P.sl_val + base + lane;
  for (int k = 0; k < w; ++k) {
    const bool e = k < lenr;
    cdst[32 * k] = e ? P.col[b + k] : 0;
    vdst[32 * k] = e ? P.val[b + k] : (VT)0;
  }
}

// A1: y = Op x on the sliced-ELL layout, one CTA per window, one warp per
// slice, lane = row: the first 16 entries' column / value loads, then their x
// gathers, all in flight at once.  Step: vbuf[cur] = Op x with x = (i == k ?
// Q[:, k] : vbuf[cur ^ 1] / beta), and Q[:, i] = x when i > k.  Breakdown:
// vbuf[cur ^ 1] = a Gaussian vector keyed by i (the replacement of
// solver/lanczos.py:107-117).  x is not written here, so it is gathered
// through the read-only (L1) path.
template <typename VT>
__global__ void __launch_bounds__(LZ_BLOCK, 8) st_sell_spmv_kernel(
    const __grid_constant__ TeamDesc<VT> P, StreamCtl* ctl) {
  st_pdl_prologue();
  typedef typename Acc<VT>::type AT;
  __shared__ VT ys[LZ_BLOCK];
  // every load that depends on no other is issued first: the control block,
  // the slice's width and row map
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int s = blockIdx.x * (LZ_BLOCK / 32) + warp;
  const bool has = s < (P.n + 31) / 32;
  const int4 ca = __ldg((const int4*)ctl), cb = __ldg((const int4*)ctl + 1);
  const double invb_d = __ldg(&ctl->invb);
  const int sb = has ? __ldg(P.sl_ptr + s) : 0;
  const int width = has ? (__ldg(P.sl_ptr + s + 1) - sb) >> 5 : 0;
  const int lr = has ? (int)__ldg(P.sl_row + 32 * s + lane) : 0;
  int i, nv, buf;
  const int mode = st_mode_of(ca, cb, P.m, &i, &nv, &buf);
  if (mode == SM_SKIP) return;
  const size_t ld = (size_t)P.ld;
  const int w0 = blockIdx.x * LZ_BLOCK, row = w0 + threadIdx.x;
  if (mode == SM_BREAKDOWN) {
    if (row < P.n) P.vbuf[(size_t)buf * ld + row] = (VT)hash_normal((uint64_t)i, (uint64_t)row);
    return;
  }
  const int k = ca.y;
  const bool wq = i > k;
  const VT xscale = wq ? (VT)invb_d : (VT)1;
  const VT* __restrict__ x = wq ? P.vbuf + (size_t)(buf ^ 1) * ld : P.Q + (size_t)k * ld;
  const VT xrow = (wq && row < P.n) ? __ldg(x + row) : (VT)0;
  if (has) {
    const int* cp = P.sl_col + sb + lane;
    const VT* vp = P.sl_val + sb + lane;
    constexpr int PF = 16;
    int c[PF];
    VT v[PF], xv[PF];
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      c[u] = (u < width) ? __ldg(cp + 32 * u) : 0;
      v[u] = (u < width) ? __ldg(vp + 32 * u) : (VT)0;
    }
#pragma unroll
    for (int u = 0; u < PF; ++u) xv[u] = (u < width) ? __ldg(x + c[u]) : (VT)0;
    AT acc = (AT)0;
#pragma unroll
    for (int u = 0; u < PF; ++u) acc += (AT)v[u] * (AT)xv[u];
    for (int u = PF; u < width; ++u) acc += (AT)__ldg(vp + 32 * u) * (AT)__ldg(x + __ldg(cp + 32 * u));
    const int r = w0 + lr;
    if (r < P.n && width == P.wcap) {
      // the rest of a row longer than the slice capacity
      const int e = P.rowptr[r + 1];
      for (int q = P.rowptr[r] + P.wcap; q < e; ++q)
        acc += (AT)__ldg(P.val + q) * (AT)__ldg(x + __ldg(P.col + q));
    }
    ys[lr] = (VT)acc;
  }
  __syncthreads();
  if (row < P.n) {
    P.vbuf[(size_t)buf * ld + row] = ys[threadIdx.x] * xscale;
    if (wq) P.Q[(size_t)i * ld + row] = xrow * xscale;
  }
}

// A2: h1[c] = Q[:, c] . v for c < nv (v = the step's y, or the breakdown vector)
template <typename VT>
__global__ void __launch_bounds__(LZ_BLOCK) st_dot_kernel(const __grid_constant__ TeamDesc<VT> P,
                                                           StreamCtl* ctl) {
  st_pdl_prologue();
  typedef typename Acc<VT>::type AT;
  __shared__ StShared<VT> sh;
  int i, nv, buf;
  if (st_mode(ctl, P.m, &i, &nv, &buf) == SM_SKIP) return;
  const int R = gridDim.x;
  const size_t ld = (size_t)P.ld;
  int c0, c1;
  st_chunks(P.n, &c0, &c1);
  const VT* v = P.vbuf + (size_t)buf * ld;
  extern __shared__ __align__(16) unsigned char st_dyn[];
  AT* sacc = (AT*)st_dyn;
  for (int c = 0; c < nv; ++c) sacc[c * LZ_BLOCK + threadIdx.x] = (AT)0;
  for (int ch = c0; ch < c1; ++ch) {
    const int r4 = ch * ST_ROWS + 4 * threadIdx.x;
    if (r4 < P.n) st_dots(P.Q, ld, r4, P.n, nv, ld4<VT, false>(v, r4, P.n), sacc);
  }
  st_block_cols(sacc, nv, P.part + blockIdx.x, R);
  if (!st_last_cta(&ctl->ticket[0], sh)) return;
  st_reduce<VT>(P.part, R, nv, sh);
  for (int c = threadIdx.x; c < nv; c += LZ_BLOCK) ctl->h1[c] = sh.h[c];
  if (threadIdx.x == 0) ctl->ticket[0] = 0u;
}

// B, one pass over Q: each thread keeps its rows of the nv basis columns in
// registers (8-byte loads: two FP32 rows or one FP64 row), forms
// v -= Q h1, then h2 = Q^T v from the same registers.
template <typename VT>
__global__ void __launch_bounds__(LZ_BLOCK, 2) st_update_dot1_kernel(
    const __grid_constant__ TeamDesc<VT> P, StreamCtl* ctl) {
  st_pdl_prologue();
  typedef typename Acc<VT>::type AT;
  constexpr int RW = 8 / (int)sizeof(VT);           // rows per thread
  constexpr int CROWS = RW * LZ_BLOCK;              // rows per chunk
  __shared__ StShared<VT> sh;
  int i, nv, buf;
  const int mode = st_mode(ctl, P.m, &i, &nv, &buf);
  if (mode == SM_SKIP) return;
  const int R = gridDim.x, n = P.n;
  const size_t ld = (size_t)P.ld;
  for (int c = threadIdx.x; c < nv; c += LZ_BLOCK) sh.hv[c] = (VT)__ldg(&ctl->h1[c]);
  extern __shared__ __align__(16) unsigned char st_dyn[];
  AT* sacc = (AT*)st_dyn;
  for (int c = 0; c < nv; ++c) sacc[c * LZ_BLOCK + threadIdx.x] = (AT)0;
  __syncthreads();
  const int nch = (n + CROWS - 1) / CROWS;
  const int c0 = (int)((long long)nch * blockIdx.x / R);
  const int c1 = (int)((long long)nch * (blockIdx.x + 1) / R);
  VT* v = P.vbuf + (size_t)buf * ld;
  for (int ch = c0; ch < c1; ++ch) {
    const int r0 = ch * CROWS + RW * threadIdx.x;
    if (r0 >= n) continue;
    const bool full = r0 + RW <= n;
    VT q[MP1][RW];
#pragma unroll
    for (int c = 0; c < MP1; ++c)
      if (c < nv) {
        const VT* src = P.Q + (size_t)c * ld + r0;
        if constexpr (RW == 2) {
          if (full) {
            const float2 a = __ldg((const float2*)src);
            q[c][0] = a.x; q[c][1] = a.y;
          } else {
            q[c][0] = __ldg(src); q[c][1] = (VT)0;
          }
        } else {
          q[c][0] = __ldg(src);
        }
      }
    VT x[RW], s[RW];
#pragma unroll
    for (int j = 0; j < RW; ++j) {
      x[j] = (r0 + j < n) ? __ldcg(v + r0 + j) : (VT)0;
      s[j] = (VT)0;
    }
#pragma unroll
    for (int c = 0; c < MP1; ++c)
      if (c < nv) {
        const VT h = sh.hv[c];
#pragma unroll
        for (int j = 0; j < RW; ++j) s[j] += q[c][j] * h;
      }
#pragma unroll
    for (int j = 0; j < RW; ++j) {
      x[j] -= s[j];
      if (r0 + j < n) v[r0 + j] = x[j];
    }
#pragma unroll
    for (int c = 0; c < MP1; ++c)
      if (c < nv) {
        AT d = (AT)0;
#pragma unroll
        for (int j = 0; j < RW; ++j) d += (AT)q[c][j] * (AT)x[j];
        sacc[c * LZ_BLOCK + threadIdx.x] += d;
      }
  }
  double* part = P.part + (size_t)MP1 * R;
  st_block_cols(sacc, nv, part + blockIdx.x, R);
  if (!st_last_cta(&ctl->ticket[1], sh)) return;
  st_reduce<VT>(part, R, nv, sh);
  for (int c = threadIdx.x; c < nv; c += LZ_BLOCK) ctl->h2[c] = sh.h[c];
  if (threadIdx.x == 0) {
    if (mode == SM_STEP) ctl->alpha[i] = __ldcg(&ctl->h1[i]) + sh.h[i];
    ctl->ticket[1] = 0u;
  }
}

// C: v -= Q h2 (c < nv), ||v||^2; the last CTA advances the loop state
template <typename VT>
__global__ void __launch_bounds__(LZ_BLOCK) st_update_norm_kernel(
    const __grid_constant__ TeamDesc<VT> P, StreamCtl* ctl) {
  st_pdl_prologue();
  typedef typename Acc<VT>::type AT;
  __shared__ StShared<VT> sh;
  int i, nv, buf;
  const int mode = st_mode(ctl, P.m, &i, &nv, &buf);
  if (mode == SM_SKIP) return;
  const int R = gridDim.x;
  const size_t ld = (size_t)P.ld;
  for (int c = threadIdx.x; c < nv; c += LZ_BLOCK) sh.hv[c] = (VT)__ldg(&ctl->h2[c]);
  __syncthreads();
  int c0, c1;
  st_chunks(P.n, &c0, &c1);
  VT* v = P.vbuf + (size_t)buf * ld;
  AT nrm[MP1];
  nrm[0] = (AT)0;
  for (int ch = c0; ch < c1; ++ch) {
    const int r4 = ch * ST_ROWS + 4 * threadIdx.x;
    if (r4 >= P.n) continue;
    Row4<VT> x = ld4<VT, false>(v, r4, P.n);
    const Row4<VT> s = st_combine(P.Q, ld, r4, P.n, nv, sh.hv);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      x.v[j] -= s.v[j];
      nrm[0] += (AT)x.v[j] * (AT)x.v[j];
    }
    st4(v, r4, P.n, x);
  }
  double* part = P.part + (size_t)2 * MP1 * R;
  block_reduce_cols(nrm, 1, sh, part + blockIdx.x, R);
  if (!st_last_cta(&ctl->ticket[2], sh)) return;
  st_reduce<VT>(part, R, 1, sh);
  if (threadIdx.x == 0) {
    const double nrm2 = sh.h[0];
    if (mode == SM_STEP) {
      // solver/lanczos.py:95-105 and the breakdown test of :107
      const double b = sqrt(nrm2);
      ctl->beta[i] = b;
      ctl->steps += 1;
      ctl->sum_nv += i + 1;
      ctl->cur = buf ^ 1;
      ctl->i = i + 1;
      if (b < 1e-15) {
        ctl->bd = 1;
        ctl->breakdowns += 1;
      } else {
        ctl->invb = 1.0 / b;
      }
    } else {
      ctl->invb = 1.0 / sqrt(nrm2);
      ctl->bd = 0;
    }
    ctl->ticket[2] = 0u;
  }
}

// restart, one CTA: the projected eigenproblem and the thick-restart choice
// (solver/lanczos.py:128-168, 202-221) once the cycle's m steps are done
template <typename VT>
__global__ void __launch_bounds__(LZ_BLOCK, 1) st_restart_kernel(
    const __grid_constant__ TeamDesc<VT> P, StreamCtl* ctl) {
  st_pdl_prologue();
  __shared__ LzShared<VT> sh;
  const int m = P.m, tid = threadIdx.x;
  if (ctl->stop || ctl->rot || ctl->bd || ctl->i < m) return;
  if (tid == 0) sh.eig_cycles = 0;
  if (tid < m) { sh.alpha[tid] = ctl->alpha[tid]; sh.beta[tid] = ctl->beta[tid]; }
  __syncthreads();
  const int k = ctl->k;
  const long long c0 = clock64();
  restart_select<false>(P, sh, k);
  if (tid < m) { ctl->alpha[tid] = sh.alpha[tid]; ctl->beta[tid] = sh.beta[tid]; }
  if (tid == 0) {
    const int kn = sh.k_next;
    ctl->stepped = (k < m) ? 1 : 0;
    ctl->k = kn;
    ctl->nconv = sh.nconv;
    ctl->restarts += 1;
    ctl->sum_kn += kn;
    ctl->rot = 1;
    const bool bad = (*(volatile int*)P.status & ST_NONFINITE) != 0;
    if (bad || sh.nconv >= P.num_desired || ctl->restarts >= P.max_restarts) ctl->stop = 1;
    P.ctl[2] = ctl->restarts;
    P.ctl[3] = ctl->breakdowns;
    P.ctl[4] = ctl->steps;
    P.ctl[6] += (int)((clock64() - c0) >> 10);
    P.ctl[13] = ctl->sum_nv;
    P.ctl[14] = ctl->sum_kn;
    P.ctl[15] += (int)(sh.eig_cycles >> 10);
  }
}

// restart rotation, full grid: Q[:, :kn] = Q[:, :m] Y, then Q[:, kn] (and
// Q[:, m]) = the last normalised vector (solver/lanczos.py:217-221)
template <typename VT>
__global__ void __launch_bounds__(LZ_BLOCK) st_rotate_kernel(const __grid_constant__ TeamDesc<VT> P,
                                                              StreamCtl* ctl) {
  st_pdl_prologue();
  __shared__ StShared<VT> sh;
  if (!__ldg(&ctl->rot)) return;
  const int m = P.m, kn = __ldg(&ctl->k);
  const bool stepped = __ldg(&ctl->stepped) != 0;
  const VT invb = (VT)__ldg(&ctl->invb);
  const size_t ld = (size_t)P.ld;
  const VT* lastv = P.vbuf + (size_t)(__ldg(&ctl->cur) ^ 1) * ld;
  for (int e = threadIdx.x; e < m * MAXM; e += LZ_BLOCK) {
    const int j = e / MAXM, c = e - j * MAXM;
    sh.u.Ys[e] = (c < kn) ? (VT)__ldcg(P.Ybuf + j * m + c) : (VT)0;
  }
  __syncthreads();
  const int R = gridDim.x, ntiles = (P.n + LZ_BLOCK - 1) / LZ_BLOCK;
  const int t0 = (int)((long long)ntiles * blockIdx.x / R);
  const int t1 = (int)((long long)ntiles * (blockIdx.x + 1) / R);
  for (int tile = t0; tile < t1; ++tile) {
    const int row = tile * LZ_BLOCK + threadIdx.x;
    if (row < P.n) {
      VT qr[MAXM];
#pragma unroll
      for (int j = 0; j < MAXM; ++j) qr[j] = (j < m) ? P.Q[(size_t)j * ld + row] : (VT)0;
      const VT xl = stepped ? lastv[row] * invb : P.Q[(size_t)m * ld + row];
      // four output columns per pass, their Y entries read together (Y is
      // zero past column kn, so the last pass may overrun kn harmlessly)
      for (int c0 = 0; c0 < kn; c0 += 4) {
        VT s[4] = {(VT)0, (VT)0, (VT)0, (VT)0};
#pragma unroll
        for (int j = 0; j < MAXM; ++j)
          if (j < m) {
            VT y4[4];
            if constexpr (sizeof(VT) == 4) {
              const float4 a = *(const float4*)&sh.u.Ys[j * MAXM + c0];
              y4[0] = a.x; y4[1] = a.y; y4[2] = a.z; y4[3] = a.w;
            } else {
              const double2 a = *(const double2*)&sh.u.Ys[j * MAXM + c0];
              const double2 b = *(const double2*)&sh.u.Ys[j * MAXM + c0 + 2];
              y4[0] = a.x; y4[1] = a.y; y4[2] = b.x; y4[3] = b.y;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) s[u] += qr[j] * y4[u];
          }
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (c0 + u < kn) P.Q[(size_t)(c0 + u) * ld + row] = s[u];
      }
      P.Q[(size_t)kn * ld + row] = xl;
      if (kn != m) P.Q[(size_t)m * ld + row] = xl;
    }
  }
  if (!st_last_cta(&ctl->ticket[3], sh)) return;
  if (threadIdx.x == 0) {
    ctl->i = kn;     // the next cycle starts from Q[:, kn]
    ctl->rot = 0;
    ctl->ticket[3] = 0u;
  }
}

// ---------------------------------------------------------------- cluster path
// A problem of at most CL_MAX_CTAS x rc rows runs as one thread-block cluster.
// CTA r of the cluster owns rows [r rc, (r+1) rc) and keeps, for the whole
// eigsh call, its rows of the basis Q (column-major, stride rc), the two work
// vectors and, when it fits, its slice of the operator (CSR with the column
// pre-split into owner CTA and local row) in shared memory.  The SpMV gathers
// x straight from the owner CTAs' shared memory (distributed shared memory,
// mapa + ld.shared::cluster); each phase's per-CTA partial sums are written to
// the CTA's own shared memory and, after a hardware cluster barrier, summed by
// every CTA over the cluster in the same fixed order, so all CTAs hold
// bit-identical coefficients and take identical branches.  The restart's
// projected eigenproblem is solved redundantly by every CTA (identical inputs,
// identical results), which needs no broadcast.  A cluster is co-scheduled by
// the hardware, so there is no software barrier and no spin-wait.
constexpr int CL_MAX_CTAS = 16;

template <typename VT>
struct ClusterDesc {
  int n, ld, m, num_desired, max_restarts, lanes, rc, csr_cap;
  long long nnz;
  double tol;
  const int* rowptr;
  const int* col;
  const VT* val;
  VT* Q;
  double* alpha;
  double* beta;
  int* ctl;
  int* status;
};

template <typename VT>
struct ClusterBatch {
  int count, csize;
  ClusterDesc<VT> t[MAX_TEAMS];
};

__device__ __forceinline__ unsigned cl_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cl_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t cl_map(const void* p, unsigned rank) {
  uint32_t a = (uint32_t)__cvta_generic_to_shared(p), r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ float cl_ld(uint32_t a, float) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ double cl_ld(uint32_t a, double) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a) : "memory");
  return v;
}

// per-CTA shared-memory layout of the cluster kernel (byte offsets)
struct ClLayout {
  size_t q, vb, part, rp, cg, val, total;
};
__host__ __device__ inline size_t cl_al(size_t b) { return (b + 15) & ~(size_t)15; }
template <typename VT>
__host__ __device__ inline ClLayout cl_layout(int m, int rc, int csr_cap) {
  ClLayout L;
  L.q = 0;
  L.vb = L.q + cl_al((size_t)(m + 1) * rc * sizeof(VT));
  L.part = L.vb + cl_al((size_t)2 * rc * sizeof(VT));
  L.rp = L.part + cl_al((size_t)3 * MP1 * sizeof(double));
  L.cg = L.rp + cl_al((size_t)(rc + 1) * sizeof(int));
  L.val = L.cg + cl_al((size_t)csr_cap * sizeof(int));
  L.total = L.val + cl_al((size_t)csr_cap * sizeof(VT));
  return L;
}

// h[c] = sum over the cluster's CTAs r = 0..C-1 of part_r[c], c < nv, summed
// as a fixed pairwise tree over 16 slots (slots r >= C hold 0): level one adds
// slots r and r+8, level two r and r+4, level three r and r+2, level four r and
// r+1.  An FP64 add holds its SM sub-partition's FP64 pipe for ~64 cycles, so
// warps 0..3 (one per sub-partition) each form one level-two sum
// R_w = (v_w + v_{w+8}) + (v_{w+4} + v_{w+12}), and warp 0 then forms
// (R_0 + R_2) + (R_1 + R_3): the tree's association, spread over four pipes.
// With norm set (nv = 1), lane 0 also forms sh.bnorm = sqrt(h[0]) and
// sh.binv = 1 / bnorm once for the CTA (FP64 square roots and divisions are
// long dependent chains on this part's narrow FP64 pipe).
static_assert(CL_MAX_CTAS == 16, "the reduction tree below is written for 16 slots");
template <typename VT>
__device__ __forceinline__ void cl_reduce(const double* part, int C, int nv, LzShared<VT>& sh,
                                          bool norm = false) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (wid < 4) {
    for (int c = lane; c < nv; c += 32) {
      const double a = (wid < C) ? cl_ld(cl_map(part + c, wid), 0.0) : 0.0;
      const double b = (wid + 8 < C) ? cl_ld(cl_map(part + c, wid + 8), 0.0) : 0.0;
      const double d = (wid + 4 < C) ? cl_ld(cl_map(part + c, wid + 4), 0.0) : 0.0;
      const double e = (wid + 12 < C) ? cl_ld(cl_map(part + c, wid + 12), 0.0) : 0.0;
      sh.u.red4[wid][c] = (a + b) + (d + e);
    }
  }
  __syncthreads();
  if (wid == 0) {
    for (int c = lane; c < nv; c += 32) {
      const double v = (sh.u.red4[0][c] + sh.u.red4[2][c]) + (sh.u.red4[1][c] + sh.u.red4[3][c]);
      sh.h[c] = v;
      sh.hv[c] = (VT)v;
      if (norm) {
        const double b = sqrt(v);
        sh.bnorm = b;
        sh.binv = (VT)(1.0 / b);
      }
    }
  }
  __syncthreads();
}

template <typename VT>
struct ClCtx {
  const ClusterDesc<VT>* P;
  int rank, C, r0, rows;
  bool staged;          // CSR slice in shared memory
  int p0;               // first entry of the slice
  VT* Qs;               // (m+1) x rc
  VT* vb;               // 2 x rc
  double* part;         // 3 x MP1
  int* rp;              // rows+1, relative to p0
  int* cg;              // (owner << 24) | local row
  VT* vs;
};

// Phase A: y = Op (x * xscale) for own rows -> vout, partial Q[:, c] . y (c <= i).
// x is column `xcol` of the cluster's vectors: xq selects Qs (else vb); the
// gathers read the owner CTA's copy.  If wq, Qs[:, i] = x * xscale (own rows).
template <typename VT, int L>
__device__ void cl_phase_spmv(const ClCtx<VT>& X, LzShared<VT>& sh, int i, const VT* xbase,
                              VT xscale, bool wq, VT* vout, double* part_out) {
  typedef typename Acc<VT>::type AT;
  const ClusterDesc<VT>& P = *X.P;
  const int tid = threadIdx.x, rc = P.rc;
  constexpr int GPP = LZ_BLOCK / L;
  const int g = tid / L, lig = tid - (tid / L) * L;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  for (int base = 0; base < X.rows; base += LZ_BLOCK) {
    // SpMV of rows base..base+255 (L lanes per row) into sh.u.st.ys; groups of
    // up to 4 passes load their row bounds and first entries before any gather
    constexpr int CH = L < 4 ? L : 4;
#pragma unroll 1
    for (int q0 = 0; q0 < L; q0 += CH) {
      int pb[CH], pe[CH];
#pragma unroll
      for (int q = 0; q < CH; ++q) {
        const int lr = base + (q0 + q) * GPP + g;
        pb[q] = 0; pe[q] = 0;
        if (lr < X.rows) {
          if (X.staged) { pb[q] = X.rp[lr] + lig; pe[q] = X.rp[lr + 1]; }
          else { pb[q] = P.rowptr[X.r0 + lr] + lig; pe[q] = P.rowptr[X.r0 + lr + 1]; }
        }
      }
      // the first entry of each of the CH rows: all gathers in flight at once
      VT av[CH], xv[CH];
#pragma unroll
      for (int q = 0; q < CH; ++q) {
        av[q] = (VT)0;
        xv[q] = (VT)0;
        if (pb[q] < pe[q]) {
          if (X.staged) {
            const int w = X.cg[pb[q]];
            av[q] = X.vs[pb[q]];
            xv[q] = cl_ld(cl_map(xbase + (w & 0xffffff), (unsigned)w >> 24), (VT)0);
          } else {
            const int gc = P.col[pb[q]];
            const int o = gc / rc;
            av[q] = P.val[pb[q]];
            xv[q] = cl_ld(cl_map(xbase + (gc - o * rc), (unsigned)o), (VT)0);
          }
        }
      }
      AT sacc[CH];
#pragma unroll
      for (int q = 0; q < CH; ++q) {
        sacc[q] = (AT)0;
        if (pb[q] < pe[q]) sacc[q] += (AT)av[q] * (AT)xv[q];
        if (X.staged) {
          for (int p = pb[q] + L; p < pe[q]; p += L) {
            const int w = X.cg[p];
            sacc[q] += (AT)X.vs[p] * (AT)cl_ld(cl_map(xbase + (w & 0xffffff), (unsigned)w >> 24), (VT)0);
          }
        } else {
          for (int p = pb[q] + L; p < pe[q]; p += L) {
            const int gc = P.col[p];
            const int o = gc / rc;
            sacc[q] += (AT)P.val[p] * (AT)cl_ld(cl_map(xbase + (gc - o * rc), (unsigned)o), (VT)0);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < CH; ++q) {
#pragma unroll
        for (int o = L >> 1; o > 0; o >>= 1) sacc[q] += __shfl_xor_sync(0xffffffffu, sacc[q], o);
        if (lig == 0) sh.u.cys[(q0 + q) * GPP + g] = (VT)sacc[q];
      }
    }
    __syncthreads();
    const int lr = base + tid;
    if (lr < X.rows) {
      const VT y = sh.u.cys[tid] * xscale;
      vout[lr] = y;
      VT xn = (VT)0;
      if (wq) {
        xn = xbase[lr] * xscale;
        X.Qs[(size_t)i * rc + lr] = xn;
      }
#pragma unroll
      for (int c = 0; c < MP1; ++c) {
        if (c <= i) {
          const VT qc = (wq && c == i) ? xn : X.Qs[(size_t)c * rc + lr];
          acc[c] += (AT)qc * (AT)y;
        }
      }
    }
    __syncthreads();
  }
  block_reduce_cols(acc, i + 1, sh, part_out, 1);
}

template <typename VT>
__device__ void cl_phase_random(const ClCtx<VT>& X, LzShared<VT>& sh, int nv, uint64_t key,
                                VT* buf, double* part_out) {
  typedef typename Acc<VT>::type AT;
  const int rc = X.P->rc;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  for (int lr = threadIdx.x; lr < X.rows; lr += LZ_BLOCK) {
    const VT r = (VT)hash_normal(key, (uint64_t)(X.r0 + lr));
    buf[lr] = r;
#pragma unroll
    for (int c = 0; c < MP1; ++c)
      if (c < nv) acc[c] += (AT)X.Qs[(size_t)c * rc + lr] * (AT)r;
  }
  block_reduce_cols(acc, nv, sh, part_out, 1);
}

template <typename VT>
__device__ void cl_phase_update_dot(const ClCtx<VT>& X, LzShared<VT>& sh, int nv, VT* buf,
                                    double* part_out) {
  typedef typename Acc<VT>::type AT;
  const int rc = X.P->rc;
  AT acc[MP1];
#pragma unroll
  for (int c = 0; c < MP1; ++c) acc[c] = (AT)0;
  for (int lr = threadIdx.x; lr < X.rows; lr += LZ_BLOCK) {
    VT qr[MP1];
    VT s = (VT)0;
#pragma unroll
    for (int c = 0; c < MP1; ++c) {
      if (c < nv) {
        qr[c] = X.Qs[(size_t)c * rc + lr];
        s += qr[c] * sh.hv[c];
      }
    }
    const VT q1 = buf[lr] - s;
    buf[lr] = q1;
#pragma unroll
    for (int c = 0; c < MP1; ++c)
      if (c < nv) acc[c] += (AT)qr[c] * (AT)q1;
  }
  block_reduce_cols(acc, nv, sh, part_out, 1);
}

template <typename VT>
__device__ void cl_phase_update_norm(const ClCtx<VT>& X, LzShared<VT>& sh, int nv, VT* buf,
                                     double* part_out) {
  typedef typename Acc<VT>::type AT;
  const int rc = X.P->rc;
  AT nrm = (AT)0;
  for (int lr = threadIdx.x; lr < X.rows; lr += LZ_BLOCK) {
    VT s = (VT)0;
#pragma unroll
    for (int c = 0; c < MP1; ++c)
      if (c < nv) s += X.Qs[(size_t)c * rc + lr] * sh.hv[c];
    const VT q2 = buf[lr] - s;
    buf[lr] = q2;
    nrm += (AT)q2 * (AT)q2;
  }
  AT one[MP1];
  one[0] = nrm;
  block_reduce_cols(one, 1, sh, part_out, 1);
}

template <typename VT>
__device__ void cl_spmv_dispatch(const ClCtx<VT>& X, LzShared<VT>& sh, int i, const VT* xbase,
                                 VT xscale, bool wq, VT* vout, double* part_out) {
  switch (X.P->lanes) {
    case 1: cl_phase_spmv<VT, 1>(X, sh, i, xbase, xscale, wq, vout, part_out); break;
    case 2: cl_phase_spmv<VT, 2>(X, sh, i, xbase, xscale, wq, vout, part_out); break;
    case 4: cl_phase_spmv<VT, 4>(X, sh, i, xbase, xscale, wq, vout, part_out); break;
    case 8: cl_phase_spmv<VT, 8>(X, sh, i, xbase, xscale, wq, vout, part_out); break;
    case 16: cl_phase_spmv<VT, 16>(X, sh, i, xbase, xscale, wq, vout, part_out); break;
    default: cl_phase_spmv<VT, 32>(X, sh, i, xbase, xscale, wq, vout, part_out); break;
  }
}

template <typename VT>
__global__ void __launch_bounds__(LZ_BLOCK, 1)
lanczos_cluster_kernel(const __grid_constant__ ClusterBatch<VT> batch) {
  __shared__ LzShared<VT> sh;
  extern __shared__ __align__(16) unsigned char cl_dyn[];
  const int C = batch.csize;
  const ClusterDesc<VT>& P = batch.t[blockIdx.x / C];
  const int rank = (int)cl_rank();
  const int tid = threadIdx.x;
  const int n = P.n, m = P.m, rc = P.rc;
  const size_t ld = (size_t)P.ld;
  const ClLayout Lo = cl_layout<VT>(m, rc, P.csr_cap);
  ClCtx<VT> X;
  X.P = &P;
  X.rank = rank;
  X.C = C;
  X.r0 = rank * rc;
  X.rows = max(0, min(rc, n - X.r0));
  X.Qs = (VT*)(cl_dyn + Lo.q);
  X.vb = (VT*)(cl_dyn + Lo.vb);
  X.part = (double*)(cl_dyn + Lo.part);
  X.rp = (int*)(cl_dyn + Lo.rp);
  X.cg = (int*)(cl_dyn + Lo.cg);
  X.vs = (VT*)(cl_dyn + Lo.val);
  double* part0 = X.part;
  double* part1 = X.part + MP1;
  double* part2 = X.part + 2 * MP1;
  // stage Q[:, 0] (the start vector) and, if it fits, the operator slice
  for (int lr = tid; lr < X.rows; lr += LZ_BLOCK) X.Qs[lr] = P.Q[X.r0 + lr];
  X.p0 = (X.rows > 0) ? P.rowptr[X.r0] : 0;
  const int p1 = (X.rows > 0) ? P.rowptr[X.r0 + X.rows] : 0;
  X.staged = (p1 - X.p0) <= P.csr_cap;
  if (X.staged) {
    for (int lr = tid; lr <= X.rows; lr += LZ_BLOCK) X.rp[lr] = P.rowptr[X.r0 + lr] - X.p0;
    for (int p = X.p0 + tid; p < p1; p += LZ_BLOCK) {
      const int gc = P.col[p];
      const int o = gc / rc;
      X.cg[p - X.p0] = (o << 24) | (gc - o * rc);
      X.vs[p - X.p0] = P.val[p];
    }
  }
  int k = 0, nconv = 0, restart = 0, breakdowns = 0, steps = 0, sum_nv = 0, sum_kn = 0;
  long long clk_start = clock64(), clk_restart = 0;
  long long tp[5] = {0, 0, 0, 0, 0}, tmark = clock64();
  const bool timing = (rank == 0 && tid == 0);
  if (tid < MAXM) { sh.alpha[tid] = 0.0; sh.beta[tid] = 0.0; }
  if (tid == 0) sh.eig_cycles = 0;
  __syncthreads();
  cl_sync();
  int prev = 0;
  VT invb = (VT)1;
  while (nconv < P.num_desired && restart < P.max_restarts) {
    int cur = 0;
    for (int i = k; i < m; ++i) {
      const VT* xbase;
      bool wq;
      if (i == k) {
        xbase = X.Qs + (size_t)k * rc;
        invb = (VT)1;
        wq = false;
      } else {
        cl_reduce(part2, C, 1, sh, true);
        const double b = sh.bnorm;
        if (tid == 0) sh.beta[i - 1] = b;
        if (b < 1e-15) {
          // Krylov space exhausted: random vector orthogonalised twice
          // against Q[:, :i] (solver/lanczos.py:107-117)
          ++breakdowns;
          VT* buf = X.vb + (size_t)prev * rc;
          cl_phase_random(X, sh, i, (uint64_t)i, buf, part0);
          cl_sync();
          cl_reduce(part0, C, i, sh);
          cl_phase_update_dot(X, sh, i, buf, part1);
          cl_sync();
          cl_reduce(part1, C, i, sh);
          cl_phase_update_norm(X, sh, i, buf, part2);
          cl_sync();
          cl_reduce(part2, C, 1, sh, true);
          invb = sh.binv;
        } else {
          invb = sh.binv;
        }
        xbase = X.vb + (size_t)prev * rc;
        wq = true;
      }
      VT* vout = X.vb + (size_t)cur * rc;
      if (timing) { const long long c = clock64(); tp[1] += c - tmark; tmark = c; }
      cl_spmv_dispatch(X, sh, i, xbase, invb, wq, vout, part0);
      if (timing) { const long long c = clock64(); tp[2] += c - tmark; tmark = c; }
      cl_sync();
      if (timing) { const long long c = clock64(); tp[0] += c - tmark; tmark = c; }
      cl_reduce(part0, C, i + 1, sh);
      if (timing) { const long long c = clock64(); tp[1] += c - tmark; tmark = c; }
      const double h1i = sh.h[i];
      cl_phase_update_dot(X, sh, i + 1, vout, part1);
      if (timing) { const long long c = clock64(); tp[3] += c - tmark; tmark = c; }
      cl_sync();
      if (timing) { const long long c = clock64(); tp[0] += c - tmark; tmark = c; }
      cl_reduce(part1, C, i + 1, sh);
      if (timing) { const long long c = clock64(); tp[1] += c - tmark; tmark = c; }
      if (tid == 0) sh.alpha[i] = h1i + sh.h[i];
      cl_phase_update_norm(X, sh, i + 1, vout, part2);
      if (timing) { const long long c = clock64(); tp[4] += c - tmark; tmark = c; }
      cl_sync();
      if (timing) { const long long c = clock64(); tp[0] += c - tmark; tmark = c; }
      prev = cur;
      cur ^= 1;
      ++steps;
      sum_nv += i + 1;
    }
    // ---- restart ----
    const bool stepped = (k < m);
    if (stepped) {
      cl_reduce(part2, C, 1, sh, true);
      const double b = sh.bnorm;
      if (tid == 0) sh.beta[m - 1] = b;
      if (b < 1e-15) {
        ++breakdowns;
        VT* buf = X.vb + (size_t)prev * rc;
        cl_phase_random(X, sh, m, (uint64_t)m, buf, part0);
        cl_sync();
        cl_reduce(part0, C, m, sh);
        cl_phase_update_dot(X, sh, m, buf, part1);
        cl_sync();
        cl_reduce(part1, C, m, sh);
        cl_phase_update_norm(X, sh, m, buf, part2);
        cl_sync();
        cl_reduce(part2, C, 1, sh, true);
        invb = sh.binv;
      } else {
        invb = sh.binv;
      }
    }
    __syncthreads();
    const long long c0 = clock64();
    restart_select<true>(P, sh, k, /*write_out=*/rank == 0);
    if (timing) clk_restart += clock64() - c0;
    // every CTA of the cluster found the same projected matrix, so all of
    // them see their own ST_NONFINITE here and leave together
    if (*(volatile int*)P.status & ST_NONFINITE) { ++restart; break; }
    const int kn = sh.k_next;
    nconv = sh.nconv;
    const VT* last = stepped ? (X.vb + (size_t)prev * rc) : (X.Qs + (size_t)m * rc);
    const VT lscale = stepped ? invb : (VT)1;
    for (int lr = tid; lr < X.rows; lr += LZ_BLOCK) {
      VT qr[MAXM];
#pragma unroll
      for (int j = 0; j < MAXM; ++j) qr[j] = (j < m) ? X.Qs[(size_t)j * rc + lr] : (VT)0;
      const VT xl = last[lr] * lscale;
      for (int c = 0; c < kn; ++c) {
        if (c >= m) break;
        VT s = (VT)0;
#pragma unroll
        for (int j = 0; j < MAXM; ++j)
          if (j < m) s += qr[j] * sh.u.Ys[j * MAXM + c];
        X.Qs[(size_t)c * rc + lr] = s;
      }
      X.Qs[(size_t)kn * rc + lr] = xl;
      if (kn != m) X.Qs[(size_t)m * rc + lr] = xl;
    }
    k = kn;
    sum_kn += kn;
    ++restart;
    __syncthreads();
    cl_sync();   // rotated rows visible to the next cycle's gathers
    if (timing) tmark = clock64();
  }
  // the basis back to global memory (own rows; untouched if no cycle ran)
  if (restart > 0) {
    for (int c = 0; c <= m; ++c)
      for (int lr = tid; lr < X.rows; lr += LZ_BLOCK)
        P.Q[(size_t)c * ld + X.r0 + lr] = X.Qs[(size_t)c * rc + lr];
  }
  if (rank == 0 && tid == 0) {
    P.ctl[2] = restart;
    P.ctl[3] = breakdowns;
    P.ctl[4] = steps;
    P.ctl[6] = (int)(clk_restart >> 10);
    P.ctl[7] = (int)((clock64() - clk_start) >> 10);
    for (int j = 0; j < 5; ++j) P.ctl[8 + j] = (int)(tp[j] >> 10);
    P.ctl[13] = sum_nv;
    P.ctl[14] = sum_kn;
    P.ctl[15] = (int)(sh.eig_cycles >> 10);
    if (restart == 0) P.ctl[0] = 0;
  }
  cl_sync();   // no CTA leaves while a peer may still read its shared memory
}

// ---------------------------------------------------------------- host side

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

static thread_local int t_launches = 0;   // kernels the last lanczos_run launched (this thread)

// x of a team-kernel problem is staged in shared memory; larger problems take
// the stream path
static bool x_fits_smem(int n, size_t vt) { return (size_t)n * vt <= (size_t)LZ_XS_BYTES; }

// team path: 3 work vectors, [pass][column][cta] partials, the Ritz vectors
// and the barrier counters.  Stream path (nctas = its grid): 2 work vectors
// and the control block in the third vector's place, the same partials and
// Ritz vectors.
// entries per row a stream-path slice holds (longer rows finish from the CSR)
static int sell_wcap(int n, long long nnz) {
  const long long avg = n > 0 ? (nnz + n - 1) / n : 1;
  const long long w = avg + avg / 2 + 2;
  return (int)(w < 4 ? 4 : (w > 64 ? 64 : w));
}
static size_t sell_bytes(int n, long long nnz, size_t vt) {
  const size_t ns = ((size_t)n + 31) / 32;
  return align256((ns + 1) * sizeof(int)) + align256(ns * 32) +
         align256(ns * 32 * (size_t)sell_wcap(n, nnz) * sizeof(int)) +
         align256(ns * 32 * (size_t)sell_wcap(n, nnz) * vt);
}

size_t lanczos_workspace_bytes(int n, long long nnz, int ld, int m, int prec, int nctas,
                               bool stream) {
  (void)m;
  const size_t vt = (prec == 64) ? 8 : 4;
  size_t b = align256(3 * (size_t)ld * vt);
  b += align256((size_t)3 * nctas * MP1 * sizeof(double));
  b += align256((size_t)MAXM * MAXM * sizeof(double));
  b += 256;  // barrier counters
  if (stream || !x_fits_smem(n, vt)) b += sell_bytes(n, nnz, vt);
  return b;
}
static_assert(sizeof(StreamCtl) <= 32 * 4 * 32, "the control block takes one 32-row vector slot");

int lanczos_lanes(int n, long long nnz) {
  const double avg = n > 0 ? (double)nnz / n : 1.0;
  int L = 1;
  while (L < 32 && L * 2 <= avg * 0.75 + 1) L *= 2;
  return L;
}

int lanczos_team_size(const DeviceInfo& di, int n, int prec, bool stream) {
  if (stream || !x_fits_smem(n, prec == 64 ? 8 : 4)) {
    // stream path: the grid of its partial-sum kernels, one wave
    const int tiles = (n + LZ_BLOCK - 1) / LZ_BLOCK;
    const int occ = (prec == 64) ? di.stream_occ64 : di.stream_occ32;
    const int g = di.sm_count * (occ > 0 ? occ : 1);
    return tiles < g ? tiles : g;
  }
  const int occ = (prec == 64) ? di.lanczos_occ64 : di.lanczos_occ32;
  // two SMs stay free for the single-CTA kernels that run beside the team
  const int maxc = (di.sm_count > 4 ? di.sm_count - 2 : di.sm_count) * (occ > 0 ? occ : 1);
  const int tiles = (n + LZ_BLOCK - 1) / LZ_BLOCK;
  // at least 4 tiles per CTA: small problems are latency bound, and every
  // extra CTA costs barrier arrivals and partial sums on each phase
  int want = (tiles + 3) / 4;
  // USBS_LANCZOS_CTAS overrides the team size (tuning experiments)
  static const int forced = [] {
    const char* e = getenv("USBS_LANCZOS_CTAS");
    return e ? atoi(e) : 0;
  }();
  if (forced > 0) want = forced;
  if (want > tiles) want = tiles;
  if (want > maxc) want = maxc;
  if (want < 1) want = 1;
  return want;
}

// team kernel: dynamic shared memory it may use (the staged x)
template <typename VT>
constexpr size_t tm_dyn_max() {
  return (227 * 1024 - sizeof(LzShared<VT>) - 1024) / 128 * 128;
}
static_assert(tm_dyn_max<double>() >= (size_t)LZ_XS_BYTES, "staged x must fit");

template <typename VT>
static int run_typed(const DeviceInfo& di, const LanczosProblem* probs, int count,
                     cudaStream_t stream) {
  const int occ = (sizeof(VT) == 8) ? di.lanczos_occ64 : di.lanczos_occ32;
  const int maxc = (di.sm_count > 4 ? di.sm_count - 2 : di.sm_count) * (occ > 0 ? occ : 1);
  for (int base = 0; base < count; base += MAX_TEAMS) {
    const int cnt = (count - base < MAX_TEAMS) ? (count - base) : MAX_TEAMS;
    TeamBatch<VT> batch;
    batch.count = cnt;
    int total = 0;
    int want[MAX_TEAMS];   // cnt <= MAX_TEAMS; no heap allocation on the launch path
    for (int i = 0; i < cnt; ++i) {
      want[i] = lanczos_team_size(di, probs[base + i].n, sizeof(VT) == 8 ? 64 : 32);
      total += want[i];
    }
    if (total > maxc) {
      // shrink teams proportionally so that every CTA is co-resident
      int tot2 = 0;
      for (int i = 0; i < cnt; ++i) {
        want[i] = (int)((long long)want[i] * maxc / total);
        if (want[i] < 1) want[i] = 1;
        tot2 += want[i];
      }
      if (tot2 > maxc) {
        set_error("lanczos: %d problems need more co-resident CTAs (%d) than the device holds (%d)",
                  cnt, tot2, maxc);
        return -3;
      }
      total = tot2;
    }
    int first = 0;
    size_t dyn = 0;
    for (int i = 0; i < cnt; ++i) {
      const LanczosProblem& p = probs[base + i];
      if (p.m > MAXM || p.m < 1 || p.n < 1 || p.ld < p.n) {
        set_error("lanczos: unsupported sizes n=%d ld=%d m=%d (m must be in [1, %d])", p.n,
                  p.ld, p.m, MAXM);
        return -2;
      }
      TeamDesc<VT>& t = batch.t[i];
      t.n = p.n; t.ld = p.ld; t.m = p.m; t.num_desired = p.num_desired;
      t.max_restarts = p.max_restarts; t.tol = p.tol;
      t.lanes = lanczos_lanes(p.n, p.nnz);
      t.xsmem = ((size_t)p.n * sizeof(VT) <= (size_t)LZ_XS_BYTES) ? 1 : 0;
      if (t.xsmem && (size_t)p.n * sizeof(VT) > dyn) dyn = (size_t)p.n * sizeof(VT);
      t.first_cta = first;
      t.nctas = want[i];
      t.rowptr = p.rowptr; t.col = p.col; t.val = (const VT*)p.val;
      t.nnz = p.nnz;
      t.Q = (VT*)p.Q;
      char* w = (char*)p.work;
      t.vbuf = (VT*)w; w += align256(3 * (size_t)p.ld * sizeof(VT));
      t.part = (double*)w; w += align256((size_t)3 * want[i] * MP1 * sizeof(double));
      t.Ybuf = (double*)w; w += align256((size_t)MAXM * MAXM * sizeof(double));
      t.bar = (unsigned int*)w; w += 256;
      t.Qw = t.Q;
      t.qts = LZ_BLOCK;
      t.qcs = p.ld;
      t.alpha = p.alpha; t.beta = p.beta; t.ctl = p.ctl; t.status = p.status;
      first += want[i];
      if (cudaMemsetAsync(t.bar, 0, 2 * sizeof(unsigned int), stream) != cudaSuccess ||
          cudaMemsetAsync(p.ctl, 0, 16 * sizeof(int), stream) != cudaSuccess) {
        set_error("lanczos: memset failed");
        return -4;
      }
    }
    void* args[] = {(void*)&batch};
    static bool attr_set = false;
    if (!attr_set) {
      cudaFuncSetAttribute((const void*)lanczos_team_kernel<VT>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tm_dyn_max<VT>());
      attr_set = true;
    }
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)lanczos_team_kernel<VT>,
                                                dim3(total), dim3(LZ_BLOCK), args, dyn, stream);
    ++t_launches;
    if (e != cudaSuccess) {
      set_error("lanczos: cooperative launch of %d CTAs failed: %s", total,
                cudaGetErrorString(e));
      return -5;
    }
  }
  return 0;
}

// CTAs per SM of each partial-sum kernel of the stream path (A2, B, C, the
// rotation), measured once per precision; each kernel runs one wave of its
// own size.  Sets the dot kernels' dynamic shared memory limit on the way.
template <typename VT>
static const int* stream_occ() {
  static int occ[4] = {0, 0, 0, 0};
  static std::once_flag once;
  std::call_once(once, [] {
    const void* ks[] = {(const void*)st_dot_kernel<VT>, (const void*)st_update_dot1_kernel<VT>,
                        (const void*)st_update_norm_kernel<VT>,
                        (const void*)st_rotate_kernel<VT>};
    const size_t dyn[] = {st_sacc_bytes<VT>(), st_sacc_bytes<VT>(), 0, 0};
    for (int j = 0; j < 4; ++j) {
      if (dyn[j])
        cudaFuncSetAttribute(ks[j], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn[j]);
      int o = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, ks[j], LZ_BLOCK, dyn[j]) !=
          cudaSuccess) {
        cudaGetLastError();
        o = 1;
      }
      occ[j] = o < 1 ? 1 : o;
    }
  });
  return occ;
}
// the largest of them (sizes the partial-sum buffers)
int lanczos_stream_occupancy(int prec) {
  const int* o = prec == 64 ? stream_occ<double>() : stream_occ<float>();
  int b = 1;
  for (int j = 0; j < 4; ++j) b = o[j] > b ? o[j] : b;
  return b;
}

// Stream path of one problem.  The host enqueues a cycle's steps (m - i of
// them, one more after a breakdown), the restart and the rotation, then reads
// the control block back once (a synchronisation of `stream`) to learn where
// the next cycle starts and whether the loop has ended.  The loop state is
// on the device, so a step that is not needed only returns.
// a stream kernel launched with programmatic stream serialisation (see
// st_pdl_prologue)
template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*kernel)(KArgs...), int grid, size_t smem,
                              cudaStream_t stream, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(LZ_BLOCK);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <typename VT>
static int run_stream(const DeviceInfo& di, const LanczosProblem& p, cudaStream_t stream) {
  if (p.m > MAXM || p.m < 1 || p.n < 1 || p.ld < p.n) {
    set_error("lanczos: unsupported sizes n=%d ld=%d m=%d (m must be in [1, %d])", p.n, p.ld,
              p.m, MAXM);
    return -2;
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    set_error("lanczos: a problem of n=%d rows reads its loop state back once per restart and "
              "cannot run inside a stream capture", p.n);
    return -2;
  }
  const int ntiles = (p.n + LZ_BLOCK - 1) / LZ_BLOCK;
  const int G = lanczos_team_size(di, p.n, sizeof(VT) == 8 ? 64 : 32, true);   // partials per pass
  const int* occ = stream_occ<VT>();
  // each kernel: at most one wave, and every CTA the same number of row
  // chunks (A2 and C use 4 rows per thread, B 8 bytes per thread), so no
  // CTA runs a last chunk alone
  int g[4];
  for (int j = 0; j < 4; ++j) {
    const int rows = (j == 1) ? (8 / (int)sizeof(VT)) * LZ_BLOCK : (j == 3 ? LZ_BLOCK : ST_ROWS);
    const int nch = (p.n + rows - 1) / rows;
    int gmax = di.sm_count * occ[j];
    if (gmax > G) gmax = G;
    if (gmax < 1) gmax = 1;
    const int per = (nch + gmax - 1) / gmax;
    g[j] = (nch + per - 1) / per;
    if (g[j] < 1) g[j] = 1;
  }
  TeamDesc<VT> t;
  memset(&t, 0, sizeof(t));
  t.n = p.n; t.ld = p.ld; t.m = p.m; t.num_desired = p.num_desired;
  t.max_restarts = p.max_restarts; t.tol = p.tol;
  t.lanes = lanczos_lanes(p.n, p.nnz);
  t.first_cta = 0; t.nctas = G; t.xsmem = 0; t.nnz = p.nnz;
  t.rowptr = p.rowptr; t.col = p.col; t.val = (const VT*)p.val;
  t.Q = (VT*)p.Q; t.Qw = t.Q; t.qts = LZ_BLOCK; t.qcs = p.ld;
  char* w = (char*)p.work;
  t.vbuf = (VT*)w;
  StreamCtl* ctl = (StreamCtl*)(t.vbuf + 2 * (size_t)p.ld);
  w += align256(3 * (size_t)p.ld * sizeof(VT));
  t.part = (double*)w; w += align256((size_t)3 * G * MP1 * sizeof(double));
  t.Ybuf = (double*)w; w += align256((size_t)MAXM * MAXM * sizeof(double));
  t.bar = nullptr;
  w += 256;
  const int ns = (p.n + 31) / 32;
  t.wcap = sell_wcap(p.n, p.nnz);
  if ((long long)ns * 32 * t.wcap > 0x7fffffffLL) {
    set_error("lanczos: n=%d is too large for the stream path's operator layout", p.n);
    return -2;
  }
  t.sl_ptr = (int*)w; w += align256((size_t)(ns + 1) * sizeof(int));
  t.sl_row = (unsigned char*)w; w += align256((size_t)ns * 32);
  t.sl_col = (int*)w; w += align256((size_t)ns * 32 * t.wcap * sizeof(int));
  t.sl_val = (VT*)w;
  t.alpha = p.alpha; t.beta = p.beta; t.ctl = p.ctl; t.status = p.status;
  st_sell_order_kernel<VT><<<ntiles, LZ_BLOCK, 0, stream>>>(t);
  st_sell_scan_kernel<<<1, 1024, 0, stream>>>(ns, t.sl_ptr);
  st_sell_fill_kernel<VT><<<ntiles, LZ_BLOCK, 0, stream>>>(t);
  t_launches += 3;
  if (cudaMemsetAsync(ctl, 0, sizeof(StreamCtl), stream) != cudaSuccess ||
      cudaMemsetAsync(p.ctl, 0, 16 * sizeof(int), stream) != cudaSuccess) {
    set_error("lanczos: memset failed");
    return -4;
  }
  if (p.max_restarts == 0 || p.num_desired < 1) return 0;   // no cycle runs
  StreamCtl h;
  int i_host = 0, bd_host = 0;
  for (int guard = 0;; ++guard) {
    if (guard > 4 * p.max_restarts + 16) {
      set_error("lanczos: the stream path did not finish its %d restarts", p.max_restarts);
      return -5;
    }
    const int slots = (p.m - i_host) + (bd_host ? 1 : 0);
    cudaError_t e = cudaSuccess;
    for (int j = 0; j < slots && e == cudaSuccess; ++j) {
      e = launch_pdl(st_sell_spmv_kernel<VT>, ntiles, 0, stream, t, ctl);
      if (e == cudaSuccess) e = launch_pdl(st_dot_kernel<VT>, g[0], st_sacc_bytes<VT>(), stream, t, ctl);
      if (e == cudaSuccess)
        e = launch_pdl(st_update_dot1_kernel<VT>, g[1], st_sacc_bytes<VT>(), stream, t, ctl);
      if (e == cudaSuccess) e = launch_pdl(st_update_norm_kernel<VT>, g[2], 0, stream, t, ctl);
    }
    if (e == cudaSuccess) e = launch_pdl(st_restart_kernel<VT>, 1, 0, stream, t, ctl);
    if (e == cudaSuccess) e = launch_pdl(st_rotate_kernel<VT>, g[3], 0, stream, t, ctl);
    t_launches += 4 * slots + 2;
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error("lanczos: stream-path launch failed: %s", cudaGetErrorString(e));
      return -5;
    }
    if (cudaMemcpyAsync(&h, ctl, sizeof(h), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess) {
      set_error("lanczos: stream-path state read failed: %s",
                cudaGetErrorString(cudaGetLastError()));
      return -5;
    }
    if (h.stop) break;
    i_host = h.i;
    bd_host = h.bd;
  }
  return 0;
}

// team-kernel problems (x staged in shared memory) in batched cooperative
// launches; larger ones one after another on the stream path
template <typename VT>
static int run_noncluster(const DeviceInfo& di, const LanczosProblem* probs, int count,
                          cudaStream_t stream) {
  LanczosProblem team[MAX_TEAMS];
  for (int base = 0; base < count; base += MAX_TEAMS) {
    const int cnt = (count - base < MAX_TEAMS) ? (count - base) : MAX_TEAMS;
    int nt = 0;
    for (int i = 0; i < cnt; ++i) {
      const LanczosProblem& p = probs[base + i];
      if (x_fits_smem(p.n, sizeof(VT)) && !p.no_coop) {
        team[nt++] = p;
      } else {
        const int rc = run_stream<VT>(di, p, stream);
        if (rc) return rc;
      }
    }
    if (nt) {
      const int rc = run_typed<VT>(di, team, nt, stream);
      if (rc) return rc;
    }
  }
  return 0;
}

// shared memory left for the cluster kernel's dynamic layout
template <typename VT>
constexpr size_t cl_budget() { return 227 * 1024 - sizeof(LzShared<VT>) - 1024; }
// ---- cluster-size policy and its autotuner ----
// A launch's cluster size is ceil(n_max / target) CTAs (at most 16), for a
// target number of rows per CTA.  Each step's phases scale with the rows per
// CTA and its cluster reductions with the CTAs, and clusters of one launch
// (or of concurrent solves) compete for the SMs: on GB300 a lone problem runs
// fastest spread over 16 CTAs (FP32 n = 5000: 4.8 ms at 16 CTAs, 8.7 ms at 8),
// while 48 problems in one launch run fastest packed at 640 rows per CTA
// (17 ms against 27 ms spread).  A caller that knows its launch shares the
// GPU (a solve service) passes its own rows per CTA in the problem; otherwise
// the class's measured choice is used (usbs_lanczos_autotune times the
// candidates on a caller's batch and records the fastest for its precision,
// batch and size class), else 64 rows per CTA for one problem and 640 for a
// batch.
constexpr int TUNE_NCAND = 5;
constexpr int TUNE_CAND[TUNE_NCAND] = {64, 128, 256, 640, 1280};
static std::mutex g_tune_mu;
static std::map<long long, int> g_tune;            // class key -> rows per CTA
static thread_local int t_forced_target = 0;       // set by the tuner while it measures

static int log2_bucket(long long v) {
  int b = 0;
  while (v > 1) { v >>= 1; ++b; }
  return b;
}
// class key: precision << 32 | floor(log2(problems)) << 16 | floor(log2(largest n))
static long long tune_key(int prec, int count, int nmax) {
  return ((long long)prec << 32) | ((long long)log2_bucket(count < 1 ? 1 : count) << 16) |
         log2_bucket(nmax);
}
static int cl_target(int prec, int count, int nmax, int requested) {
  if (t_forced_target) return t_forced_target;
  if (requested > 0) return requested;
  if (const char* e = getenv(prec == 64 ? "USBS_CL_TARGET64" : "USBS_CL_TARGET32"))
    if (atoi(e) >= 32) return atoi(e);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(prec, count, nmax));
    if (it != g_tune.end()) return it->second;
  }
  return count <= 1 ? 64 : 640;
}
static int cl_csize_for(int n, int target) {
  const int c = (n + target - 1) / target;
  return c < 1 ? 1 : (c > CL_MAX_CTAS ? CL_MAX_CTAS : c);
}
template <typename VT>
inline int cl_csize(int n) {
  return cl_csize_for(n, cl_target(sizeof(VT) == 8 ? 64 : 32, 1, n, 0));
}
template <typename VT>
static bool cl_fits(int n, int m) {
  const int csize = cl_csize<VT>(n);
  if (csize > CL_MAX_CTAS || m > MAXM || m < 1 || n < 1) return false;
  const int rc = (n + csize - 1) / csize;
  return cl_layout<VT>(m, rc, 0).total <= cl_budget<VT>();
}

int lanczos_kernel_kind(int n, int m, int prec) {
  static const int enabled = [] {
    const char* e = getenv("USBS_LANCZOS_CLUSTER");
    return e ? atoi(e) : 1;
  }();
  if (enabled && (prec == 64 ? cl_fits<double>(n, m) : cl_fits<float>(n, m))) return 1;
  return x_fits_smem(n, prec == 64 ? 8 : 4) ? 0 : 2;
}

// Cluster path: every problem of the launch as one cluster of `csize` CTAs.
// Returns 1 if the problems do not fit (the caller then runs the team kernel),
// 0 on success, negative on a launch error.
template <typename VT>
static int run_cluster(const LanczosProblem* probs, int count, cudaStream_t stream) {
  static const int enabled = [] {
    const char* e = getenv("USBS_LANCZOS_CLUSTER");   // 0 forces the team kernel
    return e ? atoi(e) : 1;
  }();
  if (!enabled || count < 1 || count > MAX_TEAMS) return 1;
  constexpr size_t BUDGET = cl_budget<VT>();
  int nmax = 1, req = 0;
  for (int i = 0; i < count; ++i) {
    nmax = probs[i].n > nmax ? probs[i].n : nmax;
    req = probs[i].rows_per_cta > req ? probs[i].rows_per_cta : req;
  }
  const int csize = cl_csize_for(nmax, cl_target(sizeof(VT) == 8 ? 64 : 32, count, nmax, req));
  if (csize > CL_MAX_CTAS) return 1;
  ClusterBatch<VT> batch;
  batch.count = count;
  size_t dyn = 0;
  for (int i = 0; i < count; ++i) {
    const LanczosProblem& p = probs[i];
    if (p.m > MAXM || p.m < 1 || p.n < 1 || p.ld < p.n) return 1;
    const int rc = (p.n + csize - 1) / csize;
    const ClLayout base = cl_layout<VT>(p.m, rc, 0);
    if (base.total > BUDGET) return 1;
    // whatever is left holds the operator slice (else it is read from L2)
    const int cap = (int)((BUDGET - base.total) / (sizeof(int) + sizeof(VT))) - 8;
    ClusterDesc<VT>& t = batch.t[i];
    t.n = p.n; t.ld = p.ld; t.m = p.m; t.num_desired = p.num_desired;
    t.max_restarts = p.max_restarts; t.tol = p.tol; t.nnz = p.nnz;
    t.lanes = lanczos_lanes(p.n, p.nnz);
    t.rc = rc;
    t.csr_cap = cap > 0 ? cap : 0;
    t.rowptr = p.rowptr; t.col = p.col; t.val = (const VT*)p.val;
    t.Q = (VT*)p.Q; t.alpha = p.alpha; t.beta = p.beta; t.ctl = p.ctl; t.status = p.status;
    const size_t tot = cl_layout<VT>(p.m, rc, t.csr_cap).total;
    dyn = tot > dyn ? tot : dyn;
  }
  batch.csize = csize;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute((const void*)lanczos_cluster_kernel<VT>,
                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaFuncSetAttribute((const void*)lanczos_cluster_kernel<VT>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BUDGET);
    attr_set = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(csize * count));
  cfg.blockDim = dim3(LZ_BLOCK);
  cfg.dynamicSmemBytes = dyn;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  cudaLaunchConfig_t qcfg = cfg;     // the query needs no stream (this one may be capturing)
  qcfg.stream = nullptr;
  if (cudaOccupancyMaxActiveClusters(&nclusters, (const void*)lanczos_cluster_kernel<VT>, &qcfg) !=
          cudaSuccess || nclusters < 1) {
    cudaGetLastError();
    return 1;
  }
  for (int i = 0; i < count; ++i) {
    if (cudaMemsetAsync(probs[i].ctl, 0, 16 * sizeof(int), stream) != cudaSuccess) {
      set_error("lanczos: memset failed");
      return -4;
    }
  }
  cudaError_t e = cudaLaunchKernelEx(&cfg, lanczos_cluster_kernel<VT>, batch);
  ++t_launches;
  if (e != cudaSuccess) {
    set_error("lanczos: cluster launch (%d x %d CTAs) failed: %s", count, csize,
              cudaGetErrorString(e));
    return -5;
  }
  return 0;
}

int lanczos_last_launches() { return t_launches; }

int lanczos_run(const DeviceInfo& di, const LanczosProblem* probs, int count, int prec,
                cudaStream_t stream) {
  t_launches = 0;
  if (prec == 64) {
    const int rc = run_cluster<double>(probs, count, stream);
    if (rc <= 0) return rc;
    return run_noncluster<double>(di, probs, count, stream);
  }
  if (prec == 32) {
    const int rc = run_cluster<float>(probs, count, stream);
    if (rc <= 0) return rc;
    return run_noncluster<float>(di, probs, count, stream);
  }
  set_error("lanczos: precision must be 32 or 64");
  return -2;
}

int lanczos_tune_candidates(int i) { return (i >= 0 && i < TUNE_NCAND) ? TUNE_CAND[i] : 0; }

void lanczos_force_target(int target) { t_forced_target = target; }

// cluster size a launch of `count` problems of at most nmax rows gets with `target`
int lanczos_cluster_size(int nmax, int target) { return cl_csize_for(nmax, target); }

void lanczos_tune_record(int prec, int count, int nmax, int target) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (target > 0) g_tune[tune_key(prec, count, nmax)] = target;
  else g_tune.erase(tune_key(prec, count, nmax));
}

int lanczos_tune_entries(long long* keys, int* targets, int cap) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  int i = 0;
  for (const auto& kv : g_tune) {
    if (i < cap) { keys[i] = kv.first; targets[i] = kv.second; }
    ++i;
  }
  return i;
}

void lanczos_tune_clear() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
}

int lanczos_occupancy(int prec) {
  // occupancy with the largest staged x, so any launch stays co-resident
  int occ = 0;
  if (prec == 64) {
    cudaFuncSetAttribute((const void*)lanczos_team_kernel<double>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tm_dyn_max<double>());
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, lanczos_team_kernel<double>, LZ_BLOCK,
                                                  tm_dyn_max<double>());
  } else {
    cudaFuncSetAttribute((const void*)lanczos_team_kernel<float>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tm_dyn_max<float>());
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, lanczos_team_kernel<float>, LZ_BLOCK,
                                                  tm_dyn_max<float>());
  }
  return occ;
}

}  // namespace usbs
