// Small dense FP64 linear algebra executed by one warp or one CTA in shared
// memory: the projected Lanczos eigenproblem (m <= 32), the k x k bundle
// matrices (k <= 16) and the s x s IPM Newton systems (s <= 136).
//
// Methods (textbook, own code):
//  * symmetric eigensolver: Householder tridiagonalisation followed by the
//    implicit symmetric QR iteration with Wilkinson shift (Golub & Van Loan,
//    Matrix Computations, 4th ed., Alg. 8.3.1 and 8.3.3), eigenvectors
//    accumulated, eigenvalues sorted ascending;
//  * LU with partial pivoting and forward/back substitution (G&VL Alg. 3.4.1);
//  * Cholesky (G&VL Alg. 4.2.1) as the positive-definiteness test.
#pragma once
#include "common.cuh"

namespace usbs {

// Eigen-decomposition of the symmetric n x n matrix A (row-major, lda) by one
// warp.  On return w[0..n-1] holds the eigenvalues in ascending order and
// Z (row-major, ldz) the eigenvectors as columns.  A is destroyed.  Returns
// false if the QR iteration did not converge in 30 n sweeps.  n <= 32.
__device__ inline bool warp_syev(double* A, int lda, int n, double* w, double* Z, int ldz) {
  const int lane = threadIdx.x & 31;
  // Z = I
  for (int j = 0; j < n; ++j)
    if (lane < n) Z[lane * ldz + j] = (lane == j) ? 1.0 : 0.0;
  __syncwarp();
  // ---- Householder tridiagonalisation: A <- H A H, Z <- Z H ----
  for (int j = 0; j + 2 < n; ++j) {
    const int r0 = j + 1;  // reflector acts on rows/cols r0..n-1
    double xi = (lane > r0 && lane < n) ? A[lane * lda + j] : 0.0;
    double sigma = warp_sum(xi * xi);
    double alpha = A[r0 * lda + j];
    if (sigma == 0.0) continue;  // already tridiagonal in this column
    double nrm = sqrt(alpha * alpha + sigma);
    double v0 = (alpha <= 0.0) ? (alpha - nrm) : (-sigma / (alpha + nrm));
    double beta = 2.0 * v0 * v0 / (sigma + v0 * v0);
    // v (length n, zero outside r0..n-1), v[r0] = 1
    double vi = (lane == r0) ? 1.0 : ((lane > r0 && lane < n) ? xi / v0 : 0.0);
    // p = beta * A_sub v  (lane i computes component i); every lane shuffles
    double p = 0.0;
    for (int l = r0; l < n; ++l) {
      double vl = __shfl_sync(0xffffffffu, vi, l);
      if (lane >= r0 && lane < n) p += A[lane * lda + l] * vl;
    }
    p *= beta;
    double K = 0.5 * beta * warp_sum(p * vi);
    double wv = p - K * vi;
    __syncwarp();
    // A_sub -= v w^T + w v^T
    for (int l = r0; l < n; ++l) {
      double vl = __shfl_sync(0xffffffffu, vi, l);
      double wl = __shfl_sync(0xffffffffu, wv, l);
      if (lane >= r0 && lane < n) A[lane * lda + l] -= vi * wl + wv * vl;
    }
    __syncwarp();
    if (lane == r0) { A[r0 * lda + j] = nrm; A[j * lda + r0] = nrm; }
    if (lane > r0 && lane < n) { A[lane * lda + j] = 0.0; A[j * lda + lane] = 0.0; }
    // Z <- Z (I - beta v v^T): row i of Z: z_i -= beta (z_i . v) v^T
    for (int i = 0; i < n; ++i) {
      double zv = warp_sum((lane < n) ? Z[i * ldz + lane] * vi : 0.0);
      if (lane < n) Z[i * ldz + lane] -= beta * zv * vi;
    }
    __syncwarp();
  }
  // ---- implicit symmetric QR with Wilkinson shift on (d, e) ----
  // d/e held redundantly by all lanes in registers would need dynamic indexing;
  // keep them in A's diagonal / subdiagonal (shared memory), lane 0 writes.
  double* d = w;                 // eigenvalues end up here
  for (int i = lane; i < n; i += 32) d[i] = A[i * lda + i];
  __syncwarp();
  // subdiagonal e[i] = A[i+1][i] stored in A[(i+1)*lda + i]
  const double eps = 1.1102230246251565e-16;
  int iters = 0, maxit = 30 * n;
  int hi = n - 1;
  while (hi > 0) {
    // deflate the trailing off-diagonal if negligible
    {
      double e = A[hi * lda + hi - 1];
      if (fabs(e) <= eps * (fabs(d[hi - 1]) + fabs(d[hi])) || fabs(e) < 1e-300) {
        __syncwarp();
        if (lane == 0) A[hi * lda + hi - 1] = 0.0;
        __syncwarp();
        --hi;
        continue;
      }
    }
    // start p of the unreduced block ending at hi
    int p = hi - 1;
    while (p > 0) {
      double e = A[p * lda + p - 1];
      if (fabs(e) <= eps * (fabs(d[p - 1]) + fabs(d[p])) || fabs(e) < 1e-300) {
        __syncwarp();
        if (lane == 0) A[p * lda + p - 1] = 0.0;
        __syncwarp();
        break;
      }
      --p;
    }
    if (++iters > maxit) return false;
    // Wilkinson shift from the trailing 2x2
    double a1 = d[hi - 1], a2 = d[hi], b = A[hi * lda + hi - 1];
    double dd = 0.5 * (a1 - a2);
    double den = dd + copysign(hypot(dd, b), dd == 0.0 ? 1.0 : dd);
    double mu = a2 - b * b / den;
    double x = d[p] - mu, z = A[(p + 1) * lda + p];
    for (int k = p; k < hi; ++k) {
      double r = hypot(x, z);
      double c = (r == 0.0) ? 1.0 : x / r;
      double s = (r == 0.0) ? 0.0 : z / r;
      double ak = d[k], ak1 = d[k + 1], bk = A[(k + 1) * lda + k];
      double f = (k + 1 < hi) ? A[(k + 2) * lda + k + 1] : 0.0;
      // new 2x2 block
      double nak = c * c * ak + 2.0 * c * s * bk + s * s * ak1;
      double nak1 = s * s * ak - 2.0 * c * s * bk + c * c * ak1;
      double nbk = c * s * (ak1 - ak) + (c * c - s * s) * bk;
      __syncwarp();
      if (lane == 0) {
        if (k > p) A[k * lda + k - 1] = r;   // e[k-1] after removing the bulge
        d[k] = nak;
        d[k + 1] = nak1;
        A[(k + 1) * lda + k] = nbk;
        if (k + 1 < hi) A[(k + 2) * lda + k + 1] = c * f;
      }
      // rotate eigenvector columns k, k+1: (Z P^T)
      if (lane < n) {
        double zk = Z[lane * ldz + k], zk1 = Z[lane * ldz + k + 1];
        Z[lane * ldz + k] = c * zk + s * zk1;
        Z[lane * ldz + k + 1] = -s * zk + c * zk1;
      }
      __syncwarp();
      if (k + 1 < hi) { x = nbk; z = s * f; }
    }
  }
  __syncwarp();
  // sort ascending (selection sort, swap columns of Z)
  for (int i = 0; i < n - 1; ++i) {
    int kmin = i;
    double vmin = d[i];
    for (int j = i + 1; j < n; ++j)
      if (d[j] < vmin) { vmin = d[j]; kmin = j; }
    if (kmin != i) {
      __syncwarp();
      double di = d[i];
      if (lane < n) {
        double t = Z[lane * ldz + i];
        Z[lane * ldz + i] = Z[lane * ldz + kmin];
        Z[lane * ldz + kmin] = t;
      }
      if (lane == 0) { d[kmin] = di; d[i] = vmin; }
      __syncwarp();
    }
  }
  return true;
}

// Rotation (c, s) that zeroes the (p, q) entry of the symmetric 2 x 2 block
// [[app, apq], [apq, aqq]] (Rutishauser's formulas).
__device__ __forceinline__ void jacobi_rot(float app, float aqq, float apq, float& c, float& sn) {
  c = 1.0f;
  sn = 0.0f;
  if (apq != 0.0f) {
    const float theta = (aqq - app) / (2.0f * apq);
    const float t = copysignf(1.0f, theta) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
    c = rsqrtf(t * t + 1.0f);
    sn = t * c;
  }
}

// Pair i (0 <= i < M/2) of round r (0 <= r < M-1) of the round-robin
// ("chess tournament") order, p < q: index 0 stays, 1..M-1 rotate.
template <int M>
__device__ __forceinline__ void jacobi_pair(int r, int i, int& p, int& q) {
  if (i == 0) {
    p = 0;
    q = 1 + r;
  } else {
    p = r + i;
    p = (p >= M - 1) ? p - (M - 1) : p;
    p += 1;
    q = r - i + M - 1;
    q = (q >= M - 1) ? q - (M - 1) : q;
    q += 1;
  }
  if (p > q) { const int t = p; p = q; q = t; }
}

// Cyclic parallel Jacobi eigensolver (float) for a symmetric n x n matrix, run
// by a whole CTA (blockDim a multiple of 32) at order M (32 or 16; indices >= n
// are padding that couples to nothing): M/2 disjoint rotations per round in
// round-robin order, sweeps until the off-diagonal Frobenius norm is below
// 4 eps ||A||_F.
// One CTA barrier per round: A is double-buffered (a round reads one buffer
// and writes the other), and every warp forms the round's M/2 rotations itself
// (lane l: pair l mod M/2) and hands them to its threads by shuffle.  Thread
// (I, J) maps the 2 x 2 block of pairs (I, J) through the row rotation of I
// and the column rotation of J (the pairs are disjoint, so the block depends
// only on itself), and rotates rows J and J + M/2 of Z by pair I.
// A and A2 (row-major, lda >= M, each with room for 2 lda + n M floats) are
// destroyed; w receives the eigenvalues ascending, Z (row-major, ldz >= M) the
// eigenvectors as columns.  Returns false (uniformly) if 20 sweeps do not
// converge.  red needs 2 floats.
template <int M>
__device__ inline bool cta_jacobi_f32(float* A, float* A2, int lda, int n, float* w, float* Z,
                                      int ldz, float* red) {
  static_assert(M == 16 || M == 32, "order 16 or 32");
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5;
  constexpr int H = M / 2;
  for (int e = tid; e < M * M; e += nt) {
    const int i = e / M, j = e % M;
    Z[i * ldz + j] = (i == j) ? 1.0f : 0.0f;
    if (i >= n || j >= n) A[i * lda + j] = 0.0f;
  }
  __syncthreads();
  if (wid == 0) {
    float fro = 0.0f;
    for (int i = 0; i < M; ++i) { const float a = (lane < M) ? A[i * lda + lane] : 0.0f; fro += a * a; }
    fro = warp_sum(fro);
    if (lane == 0) red[0] = fro * (4.0f * 1.2e-7f) * (4.0f * 1.2e-7f);
  }
  __syncthreads();
  const float tol2 = red[0];
  float* cur = A;
  float* nxt = A2;
  bool ok = false;
  for (int sweep = 0; sweep < 20; ++sweep) {
    if (wid == 0) {
      float off = 0.0f;
      for (int i = 0; i < M; ++i) {
        const float a = (lane < M && lane != i) ? cur[i * lda + lane] : 0.0f;
        off += a * a;
      }
      off = warp_sum(off);
      if (lane == 0) red[1] = off;
    }
    __syncthreads();
    if (red[1] <= tol2) { ok = true; break; }
    for (int r = 0; r < M - 1; ++r) {
      int pl, ql;
      jacobi_pair<M>(r, lane % H, pl, ql);
      float cl, sl;
      jacobi_rot(cur[pl * lda + pl], cur[ql * lda + ql], cur[pl * lda + ql], cl, sl);
      for (int base = 0; base < H * H; base += nt) {      // trip count uniform over the CTA
        const int e = base + tid;
        const int I = (e / H) % H, J = e % H;
        const float c = __shfl_sync(0xffffffffu, cl, I), sn = __shfl_sync(0xffffffffu, sl, I);
        const float c2 = __shfl_sync(0xffffffffu, cl, J), s2 = __shfl_sync(0xffffffffu, sl, J);
        if (e < H * H) {
          int p, q, p2, q2;
          jacobi_pair<M>(r, I, p, q);
          jacobi_pair<M>(r, J, p2, q2);
          const float app = cur[p * lda + p2], apq = cur[p * lda + q2];
          const float aqp = cur[q * lda + p2], aqq = cur[q * lda + q2];
          // rows
          const float bpp = c * app - sn * aqp, bpq = c * apq - sn * aqq;
          const float bqp = sn * app + c * aqp, bqq = sn * apq + c * aqq;
          // columns
          nxt[p * lda + p2] = c2 * bpp - s2 * bpq;
          nxt[p * lda + q2] = s2 * bpp + c2 * bpq;
          nxt[q * lda + p2] = c2 * bqp - s2 * bqq;
          nxt[q * lda + q2] = s2 * bqp + c2 * bqq;
#pragma unroll
          for (int j = J; j < M; j += H) {
            const float zp = Z[j * ldz + p], zq = Z[j * ldz + q];
            Z[j * ldz + p] = c * zp - sn * zq;
            Z[j * ldz + q] = sn * zp + c * zq;
          }
        }
      }
      __syncthreads();
      float* t = cur;
      cur = nxt;
      nxt = t;
    }
  }
  // eigenvalues from the diagonal, sorted ascending with their vectors: each
  // value's rank (ties by index) is its position; the spare buffer's first
  // row holds the values, its second the ranks, the rest the old Z
  float* wv = nxt;
  int* rk = (int*)(nxt + lda);
  if (tid < M) wv[tid] = (tid < n) ? cur[tid * lda + tid] : 0.0f;
  __syncthreads();
  if (tid < n) {
    const float v = wv[tid];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const float u = wv[j];
      r += (u < v || (u == v && j < tid)) ? 1 : 0;
    }
    rk[tid] = r;
    w[r] = v;
  }
  __syncthreads();
  // permute Z's columns: Z[:, rank[c]] = Z_old[:, c]
  float* zs = nxt + 2 * lda;   // n x n, stride M
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, c = e - (e / n) * n;
    zs[i * M + c] = Z[i * ldz + c];
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, c = e - (e / n) * n;
    Z[i * ldz + rk[c]] = zs[i * M + c];
  }
  __syncthreads();
  return ok;
}

// One step of the iterative refinement of a symmetric eigen-decomposition of
// Ogita & Aishima ("Iterative refinement for symmetric eigenvalue
// decomposition", Japan J. Indust. Appl. Math. 35, 2018), FP64, whole CTA.
//   R = I - X^T X,  S = X^T A X,  lam_i = S_ii / (1 - R_ii),
//   E_ij = (S_ij + lam_j R_ij) / (lam_j - lam_i)  if |lam_i - lam_j| > delta,
//          R_ij / 2                                 otherwise,
//   X <- X + X E.
// A, X, R, S, W: n x n row-major with leading dimension ld (shared memory);
// A is multiplied as a dense matrix.  lam receives the refined eigenvalues.
__device__ inline void cta_refine_eig(const double* A, double* X, double* R, double* S,
                                      double* W, double* lam, double* red, int n, int ld) {
  const int tid = threadIdx.x, nt = blockDim.x;
  // W = A X
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, j = e - i * n;
    double v = 0.0;
    for (int l = 0; l < n; ++l) {
      const double a = A[i * ld + l];
      if (a != 0.0) v += a * X[l * ld + j];
    }
    W[i * ld + j] = v;
  }
  __syncthreads();
  // R = I - X^T X,  S = X^T W
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, j = e - i * n;
    double r = 0.0, s = 0.0;
    for (int l = 0; l < n; ++l) {
      r += X[l * ld + i] * X[l * ld + j];
      s += X[l * ld + i] * W[l * ld + j];
    }
    R[i * ld + j] = ((i == j) ? 1.0 : 0.0) - r;
    S[i * ld + j] = s;
  }
  __syncthreads();
  if (tid < n) lam[tid] = S[tid * ld + tid] / (1.0 - R[tid * ld + tid]);
  __syncthreads();
  // delta = 2 (||S - diag(lam)||_F + ||A||_F ||R||_F)
  double sa = 0.0, aa = 0.0, rr = 0.0;
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, j = e - i * n;
    const double d = S[i * ld + j] - ((i == j) ? lam[i] : 0.0);
    sa += d * d;
    aa += A[i * ld + j] * A[i * ld + j];
    rr += R[i * ld + j] * R[i * ld + j];
  }
  sa = block_sum(sa, red);
  __syncthreads();
  aa = block_sum(aa, red);
  __syncthreads();
  rr = block_sum(rr, red);
  const double delta = 2.0 * (sqrt(sa) + sqrt(aa) * sqrt(rr));
  // E into W
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, j = e - i * n;
    const double dl = lam[j] - lam[i];
    W[i * ld + j] = (fabs(dl) > delta) ? (S[i * ld + j] + lam[j] * R[i * ld + j]) / dl
                                       : 0.5 * R[i * ld + j];
  }
  __syncthreads();
  // X <- X + X E   (result into S, then copied back)
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, j = e - i * n;
    double v = 0.0;
    for (int l = 0; l < n; ++l) v += X[i * ld + l] * W[l * ld + j];
    S[i * ld + j] = X[i * ld + j] + v;
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, j = e - i * n;
    X[i * ld + j] = S[i * ld + j];
  }
  __syncthreads();
}

}  // namespace usbs
