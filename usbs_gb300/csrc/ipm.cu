// k x k bundle subproblems and small dense steps of the USBS iteration, FP64,
// one CTA per instance.
//
//  * ipm_kernel  mode 0: solve_quad_subprob_ipm  (solver/usbs.py:25-192)
//                mode 1: compute_lb_spec_est_ipm (solver/usbs.py:195-356)
//    Primal-dual interior point on (S, eta, T, zeta, omega) in svec
//    coordinates: Newton system (s x s) assembled from the symmetric Kronecker
//    product T (x) S^-1 and solved by LU; line search over the step grid
//    0.9^j, j < ipm_max_iters, keeping the largest step at which S + a dS and
//    T + a dT stay positive definite (tested by Cholesky, one grid point per
//    thread), exactly the reference's "smallest eigenvalue > 0" rule.
//  * eigS_kernel  eigh(S) of the bundle matrix and everything the outer
//    iteration derives from it (solver/usbs.py:409-412, 568-585, 627-644).
//  * cholqr_kernel  R^-1 of one (shifted) Cholesky-QR pass for the new bundle
//    basis (replaces the Householder QR of solver/usbs.py:641-642).
#include "common.cuh"
#include "dense.cuh"
#include "internal.h"
#include "solver.h"

namespace usbs {

constexpr double RSQ2 = 0.70710678118654752440;

__device__ __forceinline__ double nanmin2(double a, double b) {
  if (isnan(a) || isnan(b)) return __longlong_as_double(0x7ff8000000000000ll);
  return a < b ? a : b;
}

struct IpmShared {
  int bi[IPM_MAXS], ci[IPM_MAXS];
  double q12[IPM_MAXS], h1[IPM_MAXS], sI[IPM_MAXS], sS[IPM_MAXS], sT[IPM_MAXS];
  double F1[IPM_MAXS], ord[IPM_MAXS], dsT[IPM_MAXS], sSi[IPM_MAXS];
  double S[IPM_MAXK * IPM_MAXK], T[IPM_MAXK * IPM_MAXK], Si[IPM_MAXK * IPM_MAXK];
  double dS[IPM_MAXK * IPM_MAXK], dT[IPM_MAXK * IPM_MAXK], wk[IPM_MAXK * IPM_MAXK];
  double redv[IPM_BLOCK / 32];
  int redi[IPM_BLOCK / 32];
  double lcol[IPM_MAXS];
  double dinv[IPM_MAXS];
  double u2[IPM_MAXS], w2[IPM_MAXS];   // per-column terms of the rank-2 correction
  int cord[IPM_MAXS];                  // svec indices, off-diagonal ones first
  double part3[3 * IPM_MAXS];          // partial sums of cta_matvec3
};

// sum_a x[a] y[a], computed redundantly by every warp (identical in all threads)
__device__ __forceinline__ double dot_s(const double* x, const double* y, int s) {
  double v = 0.0;
  for (int a = threadIdx.x & 31; a < s; a += 32) v += x[a] * y[a];
  return warp_sum(v);
}

__device__ __forceinline__ double svec_of(const double* M, int k, int b, int c) {
  return (b == c) ? M[b * k + b] : (RSQ2 * M[c * k + b] + RSQ2 * M[b * k + c]);
}

__device__ __forceinline__ void svec_inv_to(const double* v, int k, int s, const int* bi,
                                            const int* ci, double* M) {
  for (int a = threadIdx.x; a < s; a += blockDim.x) {
    const int b = bi[a], c = ci[a];
    if (b == c) M[b * k + b] = v[a];
    else { M[b * k + c] = RSQ2 * v[a]; M[c * k + b] = RSQ2 * v[a]; }
  }
}

// 0.5 * [U (T (x) X + X (x) T) U^T]_{a, a2}, U the svec isometry.
// The same entry with each distinct product summed once: of the 2 na nb
// products of the definition every one appears twice (T_ii2 X_jj2 for the
// ordering (i, j) equals X_jj2 T_ii2 for (j, i)), and 0.5 * 2 is exact, so
//   entry = w * sum over the orderings (i2, j2) of a2 of T_b,i2 X_c,j2 + X_b,i2 T_c,j2
// (one ordering when a is diagonal), w = 1/2 when a and a2 are both diagonal or
// both off-diagonal, 1/sqrt(2) otherwise.
__device__ __forceinline__ double symkron_sum(const double* T, const double* X, int k, int b,
                                              int c, int b2, int c2) {
  double S = T[b * k + b2] * X[c * k + c2];
  S = fma(X[b * k + b2], T[c * k + c2], S);
  if (b2 != c2 && b != c) {
    S = fma(T[b * k + c2], X[c * k + b2], S);
    S = fma(X[b * k + c2], T[c * k + b2], S);
  }
  return (((b == c) == (b2 == c2)) ? 0.5 : RSQ2) * S;
}

// Positive-definiteness test of A + s dA (k x k, lower triangle) by LDL^T
// without pivoting: PD iff every pivot is positive (equivalent to Cholesky
// succeeding, i.e. to the smallest eigenvalue being > 0, up to round-off at the
// boundary).  One reciprocal per column, no square roots.
// L holds the unit lower factor l_ip and U the unscaled l_ip d_p (packed lower
// triangles), so each update term l_ip (l_jp d_p) is one FMA.
__device__ __forceinline__ bool pd_test(const double* A, const double* dA, double s, int k) {
  double L[IPM_MAXS], U[IPM_MAXS];
  for (int j = 0; j < k; ++j) {
    const int rj = j * (j + 1) / 2;
    double d = A[j * k + j] + s * dA[j * k + j];
    for (int p = 0; p < j; ++p) d -= L[rj + p] * U[rj + p];
    if (!(d > 0.0)) return false;
    const double inv = 1.0 / d;
    for (int i = j + 1; i < k; ++i) {
      const int ri = i * (i + 1) / 2;
      double v = A[i * k + j] + s * dA[i * k + j];
      for (int p = 0; p < j; ++p) v -= L[ri + p] * U[rj + p];
      U[ri + j] = v;
      L[ri + j] = v * inv;
    }
  }
  return true;
}

struct IpmScal {
  double eta, zeta, omega, mu, step, trS, k1, k2, den, ze, F2, d_eta, d_omega, d_zeta, st, cS,
      cT, q22, h2, t1, t2, t3, t4, rden;
  int cont, it;
};

// sum_a x[a] y[a] by one warp (lane 0 holds the result)
__device__ __forceinline__ double wdot(const double* x, const double* y, int s) {
  double v = 0.0;
  for (int a = threadIdx.x & 31; a < s; a += 32) v += x[a] * y[a];
  return warp_sum(v);
}

// |x| of a double as an integer key: for finite values the ordering of the keys
// is the ordering of |x|, so pivot comparisons stay off the FP64 pipe.
__device__ __forceinline__ unsigned long long abs_key(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

// Inverse of an n x n matrix (n <= IPM_MAXK, row-major, lda = n) by Gauss-Jordan
// elimination with partial pivoting on [A | I], whole CTA: per pivot, warp 0
// picks the row (largest |a|, ties to the smaller index), every thread then
// updates one or two entries of the 2n-wide augmented rows.  Per element the
// arithmetic is that of the row-by-row algorithm (pivot row scaled by 1/a_jj,
// a_ic - a_ij * row_c).  A is destroyed.  Returns false if a pivot is zero.
__device__ bool cta_inverse(double* A, int n, double* Ainv, double* fcol, int* piv_s,
                            double* inv_s) {
  const int tid = threadIdx.x, lane = tid & 31, nt = blockDim.x;
  for (int e = tid; e < n * n; e += nt) Ainv[e] = ((e / n) == (e % n)) ? 1.0 : 0.0;
  bool ok = true;
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    if (tid < 32) {
      // largest |a| key among rows j.., ties to the smaller row: warp reduction
      // instructions on the high word, then the low word among the lanes
      // holding the top high word, then the smallest row among ties
      const bool valid = lane >= j && lane < n;
      const unsigned long long key = valid ? abs_key(A[lane * n + j]) : 0ull;
      const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
      const unsigned mhi = __reduce_max_sync(0xffffffffu, valid ? hi : 0u);
      const bool th = valid && hi == mhi;
      const unsigned mlo = __reduce_max_sync(0xffffffffu, th ? lo : 0u);
      const bool tl = th && lo == mlo;
      const unsigned mrow = __reduce_min_sync(0xffffffffu, tl ? (unsigned)lane : 0xffffffffu);
      int bi = (mrow == 0xffffffffu) ? 0x7fffffff : (int)mrow;
      if (lane == 0) {
        if (bi == 0x7fffffff) bi = j;
        *piv_s = bi;
        const double pv = A[bi * n + j];
        *inv_s = (pv == 0.0) ? 0.0 : 1.0 / pv;
      }
    }
    __syncthreads();
    const int piv = *piv_s;
    const double inv = *inv_s;
    if (inv == 0.0) ok = false;
    if (piv != j) {
      for (int c = tid; c < 2 * n; c += nt) {
        double* M = (c < n) ? A : Ainv;
        const int cc = (c < n) ? c : c - n;
        const double t = M[j * n + cc];
        M[j * n + cc] = M[piv * n + cc];
        M[piv * n + cc] = t;
      }
      __syncthreads();
    }
    for (int i = tid; i < n; i += nt) fcol[i] = A[i * n + j];
    __syncthreads();
    for (int c = tid; c < 2 * n; c += nt) {
      double* M = (c < n) ? A : Ainv;
      const int cc = (c < n) ? c : c - n;
      M[j * n + cc] *= inv;
    }
    __syncthreads();
    for (int e = tid; e < n * 2 * n; e += nt) {
      const int i = e / (2 * n), c = e - i * 2 * n;
      if (i == j) continue;
      double* M = (c < n) ? A : Ainv;
      const int cc = (c < n) ? c : c - n;
      M[i * n + cc] -= fcol[i] * M[j * n + cc];
    }
    __syncthreads();
  }
  return ok;
}

// y[a] = sum_b M[a, b] x[b] (s x s, row-major) as three partial chains per row,
// combined in a fixed order (a 66-long dependent FP64 chain costs ~4k cycles)
__device__ void cta_matvec3(const double* M, const double* x, int s, double* part, double* y) {
  const int tid = threadIdx.x;
  if (tid < 3 * s) {
    const int a = tid / 3, q = tid - 3 * (tid / 3);
    const int b0 = (q * s) / 3, b1 = ((q + 1) * s) / 3;
    double v = 0.0;
    for (int b = b0; b < b1; ++b) v += M[a * s + b] * x[b];
    part[tid] = v;
  }
  __syncthreads();
  for (int a = tid; a < s; a += blockDim.x) y[a] = (part[3 * a] + part[3 * a + 1]) + part[3 * a + 2];
  __syncthreads();
}

// LU with partial pivoting and solve, whole CTA (G&VL Alg. 3.4.1, right-looking
// with a one-column look-ahead).  A is stored column-major (A[c * lda + i] is
// row i, column c), so every column access of the pivot chain is contiguous.
// On GB300 an FP64 warp instruction holds its SM sub-partition's FP64 pipe for
// 64 cycles, so the pivot chain of each column is kept off the critical path:
// while warps 1..7 eliminate b and apply the rank-1 update of column j to
// columns j+2.., warp 0 updates column j+1 (lane q holds rows j+1+q, j+33+q,
// j+65+q in registers, and only the blocks that still hold rows take part),
// picks the next pivot from those registers (largest |a|, ties to the smaller
// row index as in LAPACK; warp reduction instructions on the integer keys of
// |a|), forms its reciprocal and the next multipliers.  Rows are swapped
// physically at the start of each column.  L is not stored: b is eliminated
// alongside.  Every element sees the arithmetic of the textbook algorithm
// (a_ic - l_i a_jc, l_i = a_ij * (1/a_jj)).  Partial pivoting is needed: in
// the bundle subproblems' Newton systems about two thirds of the
// factorisations exchange rows somewhere.
constexpr int LU_RPL = (IPM_MAXS + 31) / 32;   // rows per lane of warp 0
__device__ void ipm_lu_solve(double* A, int lda, double* b, int n, double* dinv, double* lcol,
                             int* ok_out) {
  const int tid = threadIdx.x, lane = tid & 31;
  __shared__ double lnext[IPM_MAXS];
  __shared__ int pnext[2];   // pivot of column j in pnext[j & 1] (written one column ahead)
  double* lc = lcol;         // multipliers of the current column (indexed by row)
  double* ln = lnext;        // multipliers of the next column
  // warp 0: rows r = j + lane + 32 q of column j are in v[q] (q < nq); pivot,
  // reciprocal and multipliers of column j
  auto pick = [&](int j, const double (&v)[LU_RPL], double* lout, int nq) {
    // lane-local candidate: largest |a| key, smallest row among equal keys
    unsigned long long best = 0ull;
    int bi = 0x7fffffff;
#pragma unroll
    for (int q = 0; q < LU_RPL; ++q) {
      const int i = j + lane + 32 * q;
      if (q < nq && i < n) {
        const unsigned long long kk = abs_key(v[q]);
        if (bi == 0x7fffffff || kk > best) { best = kk; bi = i; }
      }
    }
    // warp argmax by reduction instructions: high word, then low word among
    // the lanes holding the top high word, then the smallest row among ties
    const unsigned hi = (unsigned)(best >> 32), lo = (unsigned)best;
    const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
    const bool th = (bi != 0x7fffffff) && hi == mhi;
    const unsigned mlo = __reduce_max_sync(0xffffffffu, th ? lo : 0u);
    const bool tl = th && lo == mlo;
    const unsigned mrow = __reduce_min_sync(0xffffffffu, tl ? (unsigned)bi : 0xffffffffu);
    double bv;
    if (mrow == 0xffffffffu) {
      bi = j;
      bv = A[(size_t)j * lda + j];
    } else {
      bi = (int)mrow;
      const int off = bi - j;           // the row's owner lane and register
      double sel = 0.0;
#pragma unroll
      for (int q = 0; q < LU_RPL; ++q) if (q == (off >> 5)) sel = v[q];
      bv = __shfl_sync(0xffffffffu, sel, off & 31);
    }
    const double inv = (bv == 0.0) ? 1.0 : 1.0 / bv;
#pragma unroll
    for (int q = 0; q < LU_RPL; ++q) {
      const int i = j + lane + 32 * q;
      if (q < nq && i < n) lout[i] = v[q] * inv;
    }
    if (lane == 0) {
      pnext[j & 1] = bi;
      dinv[j] = inv;
      if (bv == 0.0) *ok_out = 0;
    }
  };
  if (tid == 0) *ok_out = 1;
  __syncthreads();
  if (tid < 32) {
    double v[LU_RPL];
#pragma unroll
    for (int q = 0; q < LU_RPL; ++q) {
      const int i = lane + 32 * q;
      v[q] = (i < n) ? A[i] : 0.0;
    }
    pick(0, v, lc, LU_RPL);
  }
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    const int piv = pnext[j & 1];
    // swap rows j and piv (columns j.., b and the multipliers of column j)
    if (piv != j) {
      for (int c = j + tid; c < n; c += blockDim.x) {
        const double t = A[c * lda + j];
        A[c * lda + j] = A[c * lda + piv];
        A[c * lda + piv] = t;
      }
      if (tid == 0) {
        const double t = b[j]; b[j] = b[piv]; b[piv] = t;
        lc[piv] = lc[j];
      }
      __syncthreads();
    }
    const int w = n - j - 1;
    if (w == 0) break;
    if (tid < 32) {
      // column j+1 for rows j+1.. (all loads first), then the look-ahead
      const double* colj1 = A + (size_t)(j + 1) * lda;
      const double ujn = colj1[j];
      const int nq = (w + 31) >> 5;   // register blocks holding rows, warp-uniform
      double a[LU_RPL], l[LU_RPL];
#pragma unroll
      for (int q = 0; q < LU_RPL; ++q) {
        const int i = j + 1 + lane + 32 * q;
        a[q] = (q < nq && i < n) ? colj1[i] : 0.0;
        l[q] = (q < nq && i < n) ? lc[i] : 0.0;
      }
      double v[LU_RPL];
#pragma unroll
      for (int q = 0; q < LU_RPL; ++q) {
        if (q < nq) {
          const int i = j + 1 + lane + 32 * q;
          v[q] = a[q] - l[q] * ujn;
          if (i < n) A[(size_t)(j + 1) * lda + i] = v[q];
        } else {
          v[q] = 0.0;
        }
      }
      pick(j + 1, v, ln, nq);
    } else {
      const int nt = (int)blockDim.x - 32, t = tid - 32;
      // b for rows j+1.. (forward elimination of the right-hand side)
      if (t < w) {
        const int i = j + 1 + t;
        b[i] = b[i] - lc[i] * b[j];
      }
      if (w > 1) {
        // columns j+2.. of rows j+1..: flat over warps 1..7, lanes along rows
        const int cpp = nt / w;                 // columns per pass
        const int cc = t / w, r = t - (t / w) * w;
        if (cc < cpp) {
          const int i = j + 1 + r;
          const double li = lc[i];
          for (int c = j + 2 + cc; c < n; c += cpp) {
            double* col = A + (size_t)c * lda;
            col[i] = col[i] - li * col[j];
          }
        }
      }
    }
    __syncthreads();
    double* tsw = lc; lc = ln; ln = tsw;
  }
  __syncthreads();
  // U x = b by one warp: lane l keeps b[l], b[l + 32], b[l + 64] in registers;
  // x_j = b_j * (1 / u_jj) with the pivot reciprocal of the factorisation (as
  // the multipliers), then every lane updates its rows above j.
  if (tid < 32) {
    double br[LU_RPL];
#pragma unroll
    for (int q = 0; q < LU_RPL; ++q) br[q] = (lane + 32 * q < n) ? b[lane + 32 * q] : 0.0;
    for (int j = n - 1; j >= 0; --j) {
      const int oq = j >> 5, ol = j & 31;
      double bj = 0.0;
#pragma unroll
      for (int q = 0; q < LU_RPL; ++q) if (q == oq) bj = br[q];
      bj = __shfl_sync(0xffffffffu, bj, ol) * dinv[j];
      const double* colj = A + (size_t)j * lda;
#pragma unroll
      for (int q = 0; q < LU_RPL; ++q) {
        if (q <= oq) {   // blocks holding rows at or above j, warp-uniform
          const int i = lane + 32 * q;
          if (i == j) br[q] = bj;
          else if (i < j) br[q] -= colj[i] * bj;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < LU_RPL; ++q) if (lane + 32 * q < n) b[lane + 32 * q] = br[q];
  }
  __syncthreads();
}

__global__ void __launch_bounds__(IPM_BLOCK, 1) ipm_kernel(const __grid_constant__ IpmArgs A) {
  extern __shared__ double dyn[];
  __shared__ IpmShared sh;
  __shared__ IpmScal sc;
  __shared__ double grid[256];
  __shared__ int s_piv, s_ok;
  if (A.skip && *A.skip) return;
  const int k = A.k, s = k * (k + 1) / 2, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int nw = IPM_BLOCK / 32;
  double* Q11 = dyn;            // s*s (mode 0)
  double* coeff = dyn + s * s;  // s*s
  double* sm = A.smalls;
  if (tid == 0) {
    int a = 0, o = 0;
    for (int b = 0; b < k; ++b)
      for (int c = 0; c <= b; ++c) {
        sh.bi[a] = b; sh.ci[a] = c;
        if (b != c) sh.cord[o++] = a;
        ++a;
      }
    for (int b = 0; b < k; ++b) sh.cord[o++] = b * (b + 1) / 2 + b;
  }
  const int ngrid = A.ipm_grid;
  for (int j = tid; j < ngrid && j < 256; j += IPM_BLOCK) grid[j] = pow(0.9, (double)j);
  __syncthreads();
  const double tr = A.trace_ub;
  const double tXb_raw = sm[A.o_sc + SC_TRXBAR];
  const double tX = (tXb_raw > 0.0) ? tXb_raw : tr;
  const double bpo = sm[A.o_sc + SC_BPO];
  for (int a = tid; a < s; a += IPM_BLOCK) sh.sI[a] = (sh.bi[a] == sh.ci[a]) ? 1.0 : 0.0;
  if (A.mode == 0) {
    const double rho = A.rho;
    const double* QB = sm + A.o_QB;
    const double qs = tr * tr / rho;
    for (int e = tid; e < s * s; e += IPM_BLOCK) Q11[e] = qs * QB[e];
    const double* GZ = sm + A.o_GZ;
    const double* GYmC = sm + A.o_GYmC;
    const double* GB = sm + A.o_GB;
    const double q12s = tr * tr / (rho * tX);
    for (int a = tid; a < s; a += IPM_BLOCK) {
      const int b = sh.bi[a], c = sh.ci[a];
      sh.q12[a] = q12s * svec_of(GZ, k, b, c);
      // svec(V^T (A*(y) - C - A*(b - ups)/rho) V)
      sh.h1[a] = tr * (svec_of(GYmC, k, b, c) - svec_of(GB, k, b, c) / rho);
    }
    if (tid == 0) {
      sc.q22 = (tr * tr / (rho * tX * tX)) * sm[A.o_sc + SC_ZZ];
      sc.h2 = (tr / tX) * (sm[A.o_sc + SC_ZY] - bpo - sm[A.o_sc + SC_ZBMU] / rho);
    }
  } else {
    const double* GYC = sm + A.o_GYC;  // V^T (A*(y_cand) - C) V
    for (int a = tid; a < s; a += IPM_BLOCK) {
      sh.h1[a] = tr * svec_of(GYC, k, sh.bi[a], sh.ci[a]);   // g_1
      sh.q12[a] = 0.0;
    }
    if (tid == 0) { sc.q22 = 0.0; sc.h2 = (tr / tX) * (sm[A.o_sc + SC_ZYC] - bpo); }   // g_2
  }
  // ---- initial point ----
  if (A.mode == 0) {
    const double* S0 = sm + A.o_Ssub;
    for (int e = tid; e < k * k; e += IPM_BLOCK) sh.S[e] = S0[e] / tr;
    if (tid == 0) sc.eta = (tX / tr) * sm[A.o_sc + SC_ETA_SUB];
  } else {
    for (int e = tid; e < k * k; e += IPM_BLOCK) {
      const int r = e / k, c = e - r * k;
      sh.S[e] = (r == c) ? 0.99 * (1.0 / (k + 1.0)) : 0.0;
    }
    if (tid == 0) sc.eta = (bpo == 0.0) ? 0.00001 : 0.99 * (1.0 / (k + 1.0));
  }
  __syncthreads();
  for (int a = tid; a < s; a += IPM_BLOCK) sh.sS[a] = svec_of(sh.S, k, sh.bi[a], sh.ci[a]);
  __syncthreads();
  const double q22 = sc.q22, h2 = sc.h2;
  double eta = sc.eta;
  // T_svec -> sh.ord (temporary)
  for (int a = tid; a < s; a += IPM_BLOCK) {
    if (A.mode == 0) {
      double v = 0.0;
      for (int b = 0; b < s; ++b) v += Q11[a * s + b] * sh.sS[b];
      sh.ord[a] = v + eta * sh.q12[a] + sh.h1[a];
    } else {
      sh.ord[a] = sh.h1[a];
    }
  }
  if (wid == 0) {
    const double d = wdot(sh.q12, sh.sS, s);
    if (lane == 0) sc.zeta = (A.mode == 0) ? (d + eta * q22 + h2) : h2;
  }
  __syncthreads();
  svec_inv_to(sh.ord, k, s, sh.bi, sh.ci, sh.T);
  __syncthreads();
  if (tid == 0) {
    double zeta = sc.zeta, vmax = zeta, vmin = zeta;
    for (int b = 0; b < k; ++b) { vmax = fmax(vmax, sh.T[b * k + b]); vmin = fmin(vmin, sh.T[b * k + b]); }
    double width = vmax - vmin;
    width = (width < 100.0) ? 100.0 : width;
    double omega = -1.01 * vmin;
    omega = (omega < width) ? width : omega;
    for (int b = 0; b < k; ++b) sh.T[b * k + b] += omega;
    sc.zeta = zeta + omega;
    sc.omega = omega;
    double trS = 0.0;
    for (int b = 0; b < k; ++b) trS += sh.S[b * k + b];
    sc.trS = trS;
    sc.step = 1.0;
    sc.it = 0;
  }
  __syncthreads();
  for (int a = tid; a < s; a += IPM_BLOCK) sh.sT[a] = svec_of(sh.T, k, sh.bi[a], sh.ci[a]);
  __syncthreads();
  if (wid == 0) {
    const double d = wdot(sh.sS, sh.sT, s);
    if (lane == 0)
      sc.mu = (d + sc.eta * sc.zeta + sc.omega * (1 - sc.trS - sc.eta)) / (2 * k + 4.0);
  }
  __syncthreads();
  const int maxit = A.max_iters;
  const double eps = A.eps;
  long long ph0 = 0, ph1 = 0, ph2 = 0, ph3 = 0, tclk = 0;
  while (true) {
    if (tid == 0) tclk = clock64();
    if (tid == 0) {
      const bool cont = (sc.it < maxit) &&
          ((A.mode == 0) ? (sc.mu > eps && sc.step > eps * eps) : (sc.mu > eps));
      sc.cont = cont;
    }
    __syncthreads();
    if (!sc.cont) break;
    const double mu = sc.mu, eta_ = sc.eta, zeta = sc.zeta, omega = sc.omega, tIS = sc.trS;
    // ---- Newton system ----
    // The step's scalar coefficients are chains of FP64 divisions, each
    // holding an SM sub-partition's FP64 pipe for hundreds of cycles: the last
    // warp forms them once (k1, k2, den, ze, F2, 1/den and, for the quadratic
    // subproblem, t1 and t2), while the other warps form F1 = Q11 svec(S) + ...
    // They are read after the barrier that follows the copy of S below.
    if (wid == IPM_BLOCK / 32 - 1) {
      double F2 = 0.0;
      if (A.mode == 0) {
        const double d = wdot(sh.q12, sh.sS, s);
        F2 = d + eta_ * q22 + h2;
        F2 = F2 + (-zeta + omega);
      }
      if (lane == 0) {
        const double k1 = (1 - tIS - eta_) / omega;
        const double k2 = zeta / eta_ + q22;
        const double den = k1 * k2 + 1;
        const double ze = zeta / eta_;
        sc.k1 = k1; sc.k2 = k2; sc.den = den; sc.ze = ze;
        sc.F2 = F2;
        sc.rden = 1.0 / den;
        if (A.mode == 0) {
          sc.t1 = (mu / omega + tIS + eta_ - 1 + k1 * (F2 - mu / eta_ + zeta)) / den;
          sc.t2 = (F2 - mu / eta_ + zeta - k2 * (mu / omega + tIS + eta_ - 1)) / den;
        }
      }
    }
    if (A.mode == 0) {
      cta_matvec3(Q11, sh.sS, s, sh.part3, sh.F1);
      for (int a = tid; a < s; a += IPM_BLOCK) {
        const double f = sh.F1[a] + eta_ * sh.q12[a] + sh.h1[a];
        sh.F1[a] = f + (-sh.sT[a] + omega * sh.sI[a]);
      }
    }
    // S^-1 (the reference's jnp.linalg.inv, solver/usbs.py:91)
    for (int e = tid; e < k * k; e += IPM_BLOCK) sh.wk[e] = sh.S[e];
    __syncthreads();
    const double k1 = sc.k1, k2 = sc.k2, den = sc.den, ze = sc.ze;
    {
      const bool okinv = cta_inverse(sh.wk, k, sh.Si, sh.lcol, &s_piv, sh.redv);
      if (!okinv && tid == 0) atomicOr(A.status, ST_SMALL_DENSE_FAIL);
    }
    __syncthreads();
    const double F2 = (A.mode == 0) ? sc.F2 : 0.0;
    for (int a = tid; a < s; a += IPM_BLOCK) sh.sSi[a] = svec_of(sh.Si, k, sh.bi[a], sh.ci[a]);
    // coefficient matrix, every entry computed (S^-1 is not exactly symmetric in
    // floating point; mirroring one triangle measurably degrades the Newton
    // steps once the system is ill-conditioned near the end of the IPM)
    const double lbc = (A.mode == 1) ? (ze / (k1 * ze + 1)) : 0.0;
    const double rden = sc.rden;
    if (A.mode == 0) {
      for (int a2 = tid; a2 < s; a2 += IPM_BLOCK) {
        sh.u2[a2] = k1 * sh.q12[a2] + sh.sI[a2];
        sh.w2[a2] = sh.q12[a2] - k2 * sh.sI[a2];
      }
      __syncthreads();
    }
    // every entry of the s x s matrix, flat over the CTA; columns in cord order
    // so that the off-diagonal / diagonal branch is uniform across most warps
    // (stored column-major for the LU: coeff[a2 * s + a] is row a, column a2;
    // consecutive threads take consecutive rows of one column)
    for (int e = tid; e < s * s; e += IPM_BLOCK) {
      const int ca = e / s, a = e - ca * s, a2 = sh.cord[ca];
      double v = symkron_sum(sh.T, sh.Si, k, sh.bi[a], sh.ci[a], sh.bi[a2], sh.ci[a2]);
      if (A.mode == 0) {
        v = Q11[a * s + a2] + v;
        v -= (sh.q12[a] * sh.u2[a2] + sh.sI[a] * sh.w2[a2]) * rden;
      } else {
        v += lbc * (sh.sI[a] * sh.sI[a2]);
      }
      coeff[a2 * s + a] = v;
    }
    if (tid == 0 && A.mode == 1) {
      sc.t1 = ze * (-k1 * (mu / eta_ - h2 - omega) + mu / omega + tIS + eta_ - 1) / (-k1 * ze - 1);
      sc.t2 = h2 - mu / eta_;
    }
    __syncthreads();
    for (int a = tid; a < s; a += IPM_BLOCK) {
      double o;
      if (A.mode == 0) {
        o = -sh.F1[a] + mu * sh.sSi[a] - sh.sT[a];
        o += sc.t1 * sh.q12[a];
        o += sc.t2 * sh.sI[a];
      } else {
        o = sc.t1 * sh.sI[a];
        o += sc.t2 * sh.sI[a] - sh.h1[a];
        o += mu * sh.sSi[a];
      }
      sh.ord[a] = o;
    }
    __syncthreads();
    if (tid == 0) { const long long c = clock64(); ph0 += c - tclk; tclk = c; }
    ipm_lu_solve(coeff, s, sh.ord, s, sh.dinv, sh.lcol, &s_ok);
    if (tid == 0) { const long long c = clock64(); ph1 += c - tclk; tclk = c; }
    if (tid == 0 && !s_ok) atomicOr(A.status, ST_SMALL_DENSE_FAIL);
    // sh.ord now holds dsS
    if (wid == 0) {
      double t1 = 0.0, t2 = 0.0, t3 = 0.0;
      for (int a = lane; a < s; a += 32) {
        const double x = sh.ord[a];
        if (A.mode == 0) {
          t1 += (k1 * sh.q12[a] + sh.sI[a]) * x;
          t2 += (sh.q12[a] - k2 * sh.sI[a]) * x;
          t3 += sh.q12[a] * x;
        } else {
          t1 += sh.sI[a] * x;
        }
      }
      t1 = warp_sum(t1);
      if (A.mode == 0) { t2 = warp_sum(t2); t3 = warp_sum(t3); }
      if (lane == 0) {
        double d_eta, d_omega, d_zeta;
        if (A.mode == 0) {
          d_eta = (-t1 - (mu / omega) - tIS - eta_ + 1 + k1 * (-F2 + mu / eta_ - zeta)) / den;
          d_omega = (-F2 + mu / eta_ - zeta + k2 * (mu / omega + tIS + eta_ - 1) - t2) / den;
          d_zeta = t3 + d_eta * q22 + d_omega + F2;
        } else {
          d_eta = (t1 - k1 * (mu / eta_ - h2 - omega) + mu / omega + tIS + eta_ - 1) / (-k1 * ze - 1);
          d_omega = -ze * d_eta + mu / eta_;
          d_omega = d_omega + (-h2 - omega);
          d_zeta = d_omega - zeta + h2 + omega;
        }
        sc.d_eta = d_eta; sc.d_omega = d_omega; sc.d_zeta = d_zeta;
        // step size from the linear variables (solver/usbs.py:128-132)
        const double r = nanmin2(nanmin2(d_eta / eta_, d_zeta / zeta), d_omega / omega);
        double st = -1.0 / r;
        if (!isnan(st) && st > 1.0) st = 1.0;
        sc.st = 0.99 * ((st <= 0.0) ? 1.0 : st);
      }
    }
    __syncthreads();
    const double d_eta = sc.d_eta, d_omega = sc.d_omega;
    if (A.mode == 0) {
      cta_matvec3(Q11, sh.ord, s, sh.part3, sh.dsT);
      for (int a = tid; a < s; a += IPM_BLOCK)
        sh.dsT[a] = sh.dsT[a] + d_eta * sh.q12[a] + d_omega * sh.sI[a] + sh.F1[a];
    } else {
      for (int a = tid; a < s; a += IPM_BLOCK)
        sh.dsT[a] = d_omega * sh.sI[a] - sh.sT[a] + sh.h1[a] + omega * sh.sI[a];
    }
    __syncthreads();
    svec_inv_to(sh.ord, k, s, sh.bi, sh.ci, sh.dS);
    svec_inv_to(sh.dsT, k, s, sh.bi, sh.ci, sh.dT);
    __syncthreads();
    // ---- line search over the grid 0.9^j (solver/usbs.py:134-154): the largest
    // grid step keeping S (lanes 0-15) and T (lanes 16-31) positive definite is the
    // first positive-definite grid index ----
    if (wid == 0) {
      const int half = lane >> 4, sub = lane & 15;
      const double* M = half ? sh.T : sh.S;
      const double* dM = half ? sh.dT : sh.dS;
      // PD-ness of A + a dA is monotone along the grid (the PD steps form an
      // interval containing 0), so after the first 16 points the first PD
      // index is bracketed by testing every 16th point, then resolved inside
      // the bracket: at most three rounds of 16 tests per matrix.
      auto gstep = [&](int j) { return (j < 256) ? grid[j] : pow(0.9, (double)j); };
      int first = -1;
      {
        const bool pd = (sub < ngrid) && pd_test(M, dM, gstep(sub), k);
        const unsigned bal = __ballot_sync(0xffffffffu, pd);
        const unsigned mine = half ? (bal >> 16) : (bal & 0xffffu);
        if (mine) first = __ffs(mine) - 1;
      }
      const bool need2 = (first < 0) && (ngrid > 16);
      if (__any_sync(0xffffffffu, need2)) {
        const int jc = min(31 + 16 * sub, ngrid - 1);
        const bool pd = need2 && (16 + 16 * sub < ngrid) && pd_test(M, dM, gstep(jc), k);
        const unsigned bal = __ballot_sync(0xffffffffu, pd);
        const unsigned mine = half ? (bal >> 16) : (bal & 0xffffu);
        const int q = mine ? (__ffs(mine) - 1) : -1;
        const bool need3 = need2 && q >= 0;
        const int j3 = 16 + 16 * (q < 0 ? 0 : q) + sub;
        const int jq = min(31 + 16 * (q < 0 ? 0 : q), ngrid - 1);
        const bool pd3 = need3 && j3 <= jq && pd_test(M, dM, gstep(j3), k);
        const unsigned bal3 = __ballot_sync(0xffffffffu, pd3);
        const unsigned mine3 = half ? (bal3 >> 16) : (bal3 & 0xffffu);
        if (need3 && mine3) first = 16 + 16 * q + __ffs(mine3) - 1;
      }
      const int firstS = __shfl_sync(0xffffffffu, first, 0);
      const int firstT = __shfl_sync(0xffffffffu, first, 16);
      if (lane == 0) {
        const double cS = (firstS < 0) ? 0.0 : (firstS < 256 ? grid[firstS] : pow(0.9, (double)firstS));
        const double cT = (firstT < 0) ? 0.0 : (firstT < 256 ? grid[firstT] : pow(0.9, (double)firstT));
        const double cand = (cS < cT) ? cS : cT;
        double st = sc.st;
        st = (st < cand) ? st : cand;
        sc.st = st;
        sc.eta = eta_ + st * d_eta;
        sc.zeta = zeta + st * sc.d_zeta;
        sc.omega = omega + st * d_omega;
      }
    }
    __syncthreads();
    if (tid == 0) { const long long c = clock64(); ph2 += c - tclk; tclk = c; }
    const double st = sc.st;
    for (int e = tid; e < k * k; e += IPM_BLOCK) {
      sh.S[e] = sh.S[e] + st * sh.dS[e];
      sh.T[e] = sh.T[e] + st * sh.dT[e];
    }
    __syncthreads();
    for (int a = tid; a < s; a += IPM_BLOCK) {
      sh.sS[a] = svec_of(sh.S, k, sh.bi[a], sh.ci[a]);
      sh.sT[a] = svec_of(sh.T, k, sh.bi[a], sh.ci[a]);
    }
    __syncthreads();
    if (wid == 0) {
      const double d = wdot(sh.sS, sh.sT, s);
      if (lane == 0) {
        double trS = 0.0;
        for (int b = 0; b < k; ++b) trS += sh.S[b * k + b];
        double mun = (d + sc.eta * sc.zeta + sc.omega * (1 - trS - sc.eta)) / (2 * k + 4.0);
        mun *= (st > 0.2) ? (0.5 - 0.4 * st * st) : 1.0;
        if (!(isnan(mun) || mun <= mu)) mun = mu;
        if (A.dbg && sc.it < 128) {
          double* d = A.dbg + sc.it * 8;
          d[0] = mun; d[1] = st; d[2] = sc.eta; d[3] = sc.zeta; d[4] = sc.omega;
          d[5] = sc.d_eta; d[6] = sc.d_omega; d[7] = trS;
        }
        sc.mu = mun;
        sc.trS = trS;
        sc.step = st;
        sc.it = sc.it + 1;
      }
    }
    __syncthreads();
    if (tid == 0) { const long long c = clock64(); ph3 += c - tclk; }
  }
  if (tid == 0 && A.prof) {
    A.prof[0] += (double)ph0; A.prof[1] += (double)ph1; A.prof[2] += (double)ph2;
    A.prof[3] += (double)ph3;
  }
  // ---- outputs ----
  if (A.mode == 0) {
    for (int e = tid; e < k * k; e += IPM_BLOCK) sm[A.o_Sout + e] = tr * sh.S[e];
    if (tid == 0) {
      sm[A.o_sc + SC_ETA] = (tr / tX) * sc.eta;
      sm[A.o_sc + SC_QITERS] = sc.it;
    }
  } else {
    if (wid == 0) {
      const double g1S = wdot(sh.h1, sh.sS, s);
      if (lane == 0) {
        sm[A.o_sc + SC_LB] = sm[A.o_sc + SC_BYC] - g1S - sc.eta * h2;
        sm[A.o_sc + SC_LITERS] = sc.it;
      }
    }
  }
}

// eigh(S) and the quantities the outer iteration derives from it.  One warp.
__global__ void __launch_bounds__(IPM_BLOCK) eigS_kernel(EigSArgs A) {
  if (A.skip && *A.skip) return;
  constexpr int L = 16;                               // ld of the FP64 k x k blocks
  __shared__ double Sd[L * L], Z[L * L], R[L * L], S2[L * L], Wb[L * L], lam[L];
  __shared__ double GW[IPM_MAXK * IPM_MAXK], red[IPM_BLOCK / 32];
  __shared__ float Af[2 * (L + 1) + L * L + L], Af2[2 * (L + 1) + L * L + L], Zf[L * (L + 1)];
  __shared__ float wf[L], redf[32];
  __shared__ int order[L];
  const int k = A.k, kc = A.k_curr, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  double* sm = A.smalls;
  const double* S = sm + A.o_Sout;
  // eigh(S) (solver/usbs.py:568): FP32 parallel Jacobi at order 16, refined to
  // FP64 accuracy by two Ogita-Aishima steps, then sorted ascending
  for (int e = tid; e < k * k; e += IPM_BLOCK) {
    const int r = e / k, c = e - r * k;
    Sd[r * L + c] = S[e];
    Af[r * (L + 1) + c] = (float)S[e];
  }
  __syncthreads();
  bool ok = cta_jacobi_f32<L>(Af, Af2, L + 1, k, wf, Zf, L + 1, redf);
  for (int e = tid; e < k * k; e += IPM_BLOCK) {
    const int r = e / k, c = e - r * k;
    Z[r * L + c] = (double)Zf[r * (L + 1) + c];
  }
  __syncthreads();
  cta_refine_eig(Sd, Z, R, S2, Wb, lam, red, k, L);
  cta_refine_eig(Sd, Z, R, S2, Wb, lam, red, k, L);
  if (tid < k) {
    const double v = lam[tid];
    int r = 0;
    for (int j = 0; j < k; ++j) {
      const double u = lam[j];
      r += (u < v || (u == v && j < tid)) ? 1 : 0;
    }
    order[r] = tid;
  }
  __syncthreads();
  for (int e = tid; e < k * k; e += IPM_BLOCK) {
    const int r = e / k, c = e - r * k;
    S2[r * L + c] = Z[r * L + order[c]];
  }
  double lv = (tid < k) ? lam[order[tid]] : 0.0;
  __syncthreads();
  for (int e = tid; e < k * k; e += IPM_BLOCK) {
    const int r = e / k, c = e - r * k;
    Z[r * L + c] = S2[r * L + c];
  }
  if (tid < k) lam[tid] = fmax(lv, 0.0);   // clip(eigvals, 0)
  if (!ok && tid == 0) atomicOr(A.status, ST_SMALL_DENSE_FAIL);
  __syncthreads();
  double* W = sm + A.o_W;
  double* Sp = sm + A.o_Splus;
  double* Scp = sm + A.o_Scplus;
  for (int e = tid; e < k * k; e += IPM_BLOCK) {
    const int r = e / k, c = e - r * k;
    W[e] = Z[r * L + c];
    double a = 0.0, b = 0.0;
    for (int j = 0; j < k; ++j) {
      const double t = Z[r * L + j] * lam[j] * Z[c * L + j];
      a += t;
      if (j < kc) b += t;
    }
    Sp[e] = a;
    Scp[e] = b;
  }
  // trace(F^T C F) = sum_j lam_j (W^T G_C W)_jj
  const double* GC = sm + A.o_GC;
  for (int e = tid; e < k * k; e += IPM_BLOCK) {
    const int r = e / k, j = e - r * k;
    double v = 0.0;
    for (int c = 0; c < k; ++c) v += GC[r * k + c] * Z[c * L + j];
    GW[e] = v;   // (G_C W)[r][j]
  }
  __syncthreads();
  if (wid == 0) {
    double pj = 0.0;
    if (lane < k) {
      for (int r = 0; r < k; ++r) pj += Z[r * L + lane] * GW[r * k + lane];
      pj *= lam[lane];
    }
    const double pall = warp_sum(pj);
    const double pcur = warp_sum(lane < kc ? pj : 0.0);
    const double lc = warp_sum(lane < kc ? lam[lane] : 0.0);
    if (lane == 0) {
      double trS = 0.0;
      for (int b = 0; b < k; ++b) trS += S[b * k + b];
      sm[A.o_sc + SC_TRS] = trS;
      sm[A.o_sc + SC_SUMLAMC] = lc;
      sm[A.o_sc + SC_PFULL] = pall;
      sm[A.o_sc + SC_PCUR] = pcur;
    }
  }
  // W_past = W[:, kc:]
  const int kp = k - kc;
  for (int e = tid; e < k * kp; e += IPM_BLOCK) {
    const int r = e / kp, c = e - r * kp;
    sm[A.o_Wpast + e] = Z[r * L + kc + c];
  }
  // M = S+ (V^T Omega), Mc = Sc+ (V^T Omega)    (k x ssk)
  if (A.ssk > 0) {
    __syncthreads();
    const double* VtO = sm + A.o_VtO;
    for (int e = tid; e < k * A.ssk; e += IPM_BLOCK) {
      const int r = e / A.ssk, c = e - r * A.ssk;
      double a = 0.0, b = 0.0;
      for (int j = 0; j < k; ++j) {
        a += Sp[r * k + j] * VtO[j * A.ssk + c];
        b += Scp[r * k + j] * VtO[j * A.ssk + c];
      }
      sm[A.o_M + e] = a;
      sm[A.o_Mc + e] = b;
    }
  }
}

// One pass of (shifted) Cholesky QR: R^T R = G (+ shift I), output R^-1
// (upper), one warp.  Column j of R: lanes i >= j form G_ji - sum_p R_pj R_pi,
// lane j's value gives r_jj = sqrt(.), the others are scaled by 1 / r_jj.
// R^-1 by back substitution with one lane per column (reciprocals of the
// diagonal computed once).
__global__ void cholqr_kernel(CholQRArgs A) {
  if (A.skip && *A.skip) return;
  __shared__ double R[IPM_MAXK * IPM_MAXK], Ri[IPM_MAXK * IPM_MAXK], rd[IPM_MAXK];
  const int k = A.k, lane = threadIdx.x;
  double* sm = A.smalls;
  const double* G = sm + A.o_G;
  double shift = 0.0;
  if (A.shifted) {
    double tr = 0.0;
    for (int b = 0; b < k; ++b) tr += G[b * k + b];
    // Fukaya et al. (SIAM J. Sci. Comput. 42(1), 2020): s = 11 (m n + n (n + 1)) u ||A||_2^2
    shift = 11.0 * ((double)A.n * k + (double)k * (k + 1)) * 1.1102230246251565e-16 * tr;
  }
  for (int e = lane; e < k * k; e += 32) R[e] = 0.0;
  __syncwarp();
  bool ok = true;
  for (int j = 0; j < k; ++j) {
    double v = 0.0;
    if (lane >= j && lane < k) {
      v = G[j * k + lane] + ((lane == j) ? shift : 0.0);
      for (int p = 0; p < j; ++p) v -= R[p * k + j] * R[p * k + lane];
    }
    double d = __shfl_sync(0xffffffffu, v, j);
    if (!(d > 0.0)) { ok = false; d = 1.0; }
    const double rjj = sqrt(d);
    const double inv = 1.0 / rjj;
    if (lane == j) { R[j * k + j] = rjj; rd[j] = inv; }
    else if (lane > j && lane < k) R[j * k + lane] = v * inv;
    __syncwarp();
  }
  if (lane < k) {
    const int c = lane;
    for (int r = k - 1; r >= 0; --r) {
      double v = (r == c) ? 1.0 : 0.0;
      for (int p = r + 1; p <= c; ++p) v -= R[r * k + p] * Ri[p * k + c];
      Ri[r * k + c] = (r > c) ? 0.0 : v * rd[r];
    }
  }
  if (!ok && lane == 0) atomicOr(A.status, ST_SMALL_DENSE_FAIL);
  __syncwarp();
  for (int e = lane; e < k * k; e += 32) sm[A.o_Rinv + e] = Ri[e];
}

int launch_ipm(const IpmArgs& a, cudaStream_t st) {
  const int s = a.k * (a.k + 1) / 2;
  const size_t dyn = (size_t)2 * s * s * sizeof(double);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(ipm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         2 * IPM_MAXS * IPM_MAXS * (int)sizeof(double));
    attr = true;
  }
  ipm_kernel<<<1, IPM_BLOCK, dyn, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_error("ipm launch: %s", cudaGetErrorString(e)); return -5; }
  return 0;
}

int launch_eigS(const EigSArgs& a, cudaStream_t st) {
  eigS_kernel<<<1, IPM_BLOCK, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_error("eigS launch: %s", cudaGetErrorString(e)); return -5; }
  return 0;
}

int launch_cholqr(const CholQRArgs& a, cudaStream_t st) {
  cholqr_kernel<<<1, 32, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_error("cholqr launch: %s", cudaGetErrorString(e)); return -5; }
  return 0;
}

}  // namespace usbs
