// Sketch reconstruction and the rounding callbacks on the device (reference:
// utils/common.py:99-116 reconstruct_from_sketch, utils/maxcut_helpers.py:
// 292-302 compute_max_cut, utils/qap_helpers.py:624-653 qap_round).
//
// The reference forms P_rho = P + rho Omega with rho = sqrt(n) eps ||P||_2,
// B = sym(Omega^T P_rho), L = chol(B), M = P_rho L^-T (its lstsq), the thin SVD
// M = E diag(Rho) V^T, and Lambda = max(Rho^2 - rho, 0).  Here the n-sized work
// is one pass over the rows forming P^T P, Omega^T P and Omega^T Omega; the
// s x s algebra runs in one warp in FP64:
//   ||P||_2^2      = lambda_max(P^T P),
//   P_rho^T P_rho  = P^T P + rho (Omega^T P + P^T Omega) + rho^2 Omega^T Omega,
//   M^T M          = L^-1 (P_rho^T P_rho) L^-T = V diag(Rho^2) V^T,
//   E              = P_rho T,  T = L^-T V diag(1/Rho).
// For the sketch P = X Omega of a PSD X, rho lifts the small eigenvalues of the
// Nystrom approximation to about rho ~ n eps lambda_max(X), so
// cond(M)^2 ~ 1/(n eps) and the Gram route keeps FP64 accuracy for the
// reference's eps = 1e-6.  The rounding needs only the signs of E, one bit per
// column packed in a 32-bit word per row, after which
//   w_j^T C w_j = sum_(r,c) C_rc (1 - 2 [bit_j(r) != bit_j(c)])
// is one CSR pass gathering 4 bytes per entry.  Column order follows the
// reference's SVD (Rho descending).  Where B is not positive definite (a zero
// sketch, for one) jnp.linalg.cholesky returns NaNs: E and Lambda are NaN and
// every sign is -1, as (NaN > 0) is false.
#include "../../include/usbs_gb300.h"
#include "common.cuh"
#include "dense.cuh"
#include "internal.h"

namespace usbs {

constexpr int RD_BLOCK = 256;
constexpr int RD_ROWS = 16;      // rows per Gram tile
constexpr int RD_MAXS = 32;      // widest sketch (one sign word per row)
constexpr int RD_MAXB = 512;     // most blocks of the Gram and cut passes
constexpr int RD_LD = RD_MAXS + 1;

// small buffer layout (doubles)
constexpr int RD_T = 0;                          // T, s x s row-major (ld RD_MAXS)
constexpr int RD_LAM = RD_MAXS * RD_MAXS;        // Lambda, s
constexpr int RD_RHO = RD_LAM + RD_MAXS;         // rho
constexpr int RD_OK = RD_RHO + 1;                // 1 if B was positive definite
constexpr int RD_SMALL = RD_OK + 7;

struct RoundWs {
  double* gpart;     // RD_MAXB x 3 s^2
  double* small;     // RD_SMALL
  double* cpart;     // RD_MAXB x s
  unsigned* bits;    // n
};

static size_t rd_align(size_t b) { return (b + 255) / 256 * 256; }

static RoundWs rd_carve(void* ws, int n, int s) {
  char* w = (char*)ws;
  RoundWs r;
  r.gpart = (double*)w; w += rd_align((size_t)RD_MAXB * 3 * s * s * sizeof(double));
  r.small = (double*)w; w += rd_align((size_t)RD_SMALL * sizeof(double));
  r.cpart = (double*)w; w += rd_align((size_t)RD_MAXB * s * sizeof(double));
  r.bits = (unsigned*)w;
  return r;
}

static size_t rd_bytes(int n, int s) {
  return rd_align((size_t)RD_MAXB * 3 * s * s * sizeof(double)) +
         rd_align((size_t)RD_SMALL * sizeof(double)) +
         rd_align((size_t)RD_MAXB * s * sizeof(double)) + rd_align((size_t)n * sizeof(unsigned));
}

// per-block partials of G = [P^T P | Omega^T P | Omega^T Omega] (three s x s
// blocks, entry (b, p, q) at b s^2 + p s + q) over this block's row tiles
template <int EPT>
__global__ void __launch_bounds__(RD_BLOCK) rd_gram_kernel(int n, int s, int ld,
                                                           const double* __restrict__ P,
                                                           const double* __restrict__ Om,
                                                           double* __restrict__ part) {
  __shared__ double ps[RD_ROWS][RD_LD], os[RD_ROWS][RD_LD];
  const int tid = threadIdx.x, s2 = s * s, E = 3 * s2;
  double acc[EPT];
#pragma unroll
  for (int j = 0; j < EPT; ++j) acc[j] = 0.0;
  const int ntiles = (n + RD_ROWS - 1) / RD_ROWS;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int r0 = tile * RD_ROWS;
    for (int e = tid; e < RD_ROWS * s; e += RD_BLOCK) {
      const int c = e / RD_ROWS, r = e - c * RD_ROWS;
      const bool in = r0 + r < n;
      ps[r][c] = in ? P[(size_t)c * ld + r0 + r] : 0.0;
      os[r][c] = in ? Om[(size_t)c * ld + r0 + r] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < EPT; ++j) {
      const int e = tid + j * RD_BLOCK;
      if (e < E) {
        const int b = e / s2, pq = e - b * s2, p = pq / s, q = pq - p * s;
        double a = acc[j];
        if (b == 0) {
#pragma unroll
          for (int r = 0; r < RD_ROWS; ++r) a += ps[r][p] * ps[r][q];
        } else if (b == 1) {
#pragma unroll
          for (int r = 0; r < RD_ROWS; ++r) a += os[r][p] * ps[r][q];
        } else {
#pragma unroll
          for (int r = 0; r < RD_ROWS; ++r) a += os[r][p] * os[r][q];
        }
        acc[j] = a;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < EPT; ++j) {
    const int e = tid + j * RD_BLOCK;
    if (e < E) part[(size_t)blockIdx.x * E + e] = acc[j];
  }
}

// one CTA: sums the Gram partials in block order, then warp 0 forms rho, L,
// M^T M and its eigen-decomposition, T and Lambda (see the file comment)
__global__ void __launch_bounds__(RD_BLOCK) rd_small_kernel(int n, int s, int nblocks,
                                                            double eps,
                                                            const double* __restrict__ gpart,
                                                            double* __restrict__ small) {
  __shared__ double G[3 * RD_MAXS * RD_MAXS];
  __shared__ double A[RD_MAXS * RD_LD], Lm[RD_MAXS * RD_LD], K[RD_MAXS * RD_LD];
  __shared__ double Z[RD_MAXS * RD_LD], w[RD_MAXS];
  const int tid = threadIdx.x, lane = tid & 31, s2 = s * s, E = 3 * s2;
  for (int e = tid; e < E; e += RD_BLOCK) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int b = 0;
    for (; b + 3 < nblocks; b += 4) {
      a0 += gpart[(size_t)b * E + e];
      a1 += gpart[(size_t)(b + 1) * E + e];
      a2 += gpart[(size_t)(b + 2) * E + e];
      a3 += gpart[(size_t)(b + 3) * E + e];
    }
    for (; b < nblocks; ++b) a0 += gpart[(size_t)b * E + e];
    G[e] = (a0 + a1) + (a2 + a3);
  }
  __syncthreads();
  if (tid >= 32) return;
  const double* PtP = G;
  const double* OtP = G + s2;
  const double* OtO = G + 2 * s2;
  // ||P||_2 from the largest eigenvalue of P^T P
  for (int i = 0; i < s; ++i)
    if (lane < s) A[i * RD_LD + lane] = PtP[i * s + lane];
  __syncwarp();
  bool conv = warp_syev(A, RD_LD, s, w, Z, RD_LD);
  __syncwarp();
  const double lmax = w[s - 1];
  const double rho = sqrt((double)n) * eps * sqrt(lmax > 0.0 ? lmax : 0.0);
  // B = sym(Omega^T P + rho Omega^T Omega) into Lm, then its Cholesky factor
  for (int i = 0; i < s; ++i)
    if (lane < s)
      Lm[i * RD_LD + lane] = 0.5 * ((OtP[i * s + lane] + rho * OtO[i * s + lane]) +
                                    (OtP[lane * s + i] + rho * OtO[lane * s + i]));
  __syncwarp();
  bool pd = true;
  for (int j = 0; j < s && pd; ++j) {
    // lane i >= j: B[i][j] - sum_k<j L[i][k] L[j][k]
    double v = 0.0;
    if (lane >= j && lane < s) {
      v = Lm[lane * RD_LD + j];
      for (int k = 0; k < j; ++k) v -= Lm[lane * RD_LD + k] * Lm[j * RD_LD + k];
    }
    const double d = __shfl_sync(0xffffffffu, v, j);
    if (!(d > 0.0)) { pd = false; break; }
    const double ljj = sqrt(d);
    __syncwarp();
    if (lane == j) Lm[j * RD_LD + j] = ljj;
    else if (lane > j && lane < s) Lm[lane * RD_LD + j] = v / ljj;
    __syncwarp();
  }
  if (pd) {
    // K = P_rho^T P_rho
    for (int i = 0; i < s; ++i)
      if (lane < s)
        K[i * RD_LD + lane] = PtP[i * s + lane] +
                              rho * (OtP[i * s + lane] + OtP[lane * s + i]) +
                              rho * rho * OtO[i * s + lane];
    __syncwarp();
    // Z = L^-1 K (lane c: column c, forward substitution)
    if (lane < s) {
      for (int i = 0; i < s; ++i) {
        double v = K[i * RD_LD + lane];
        for (int k = 0; k < i; ++k) v -= Lm[i * RD_LD + k] * Z[k * RD_LD + lane];
        Z[i * RD_LD + lane] = v / Lm[i * RD_LD + i];
      }
    }
    __syncwarp();
    // A = Z L^-T (lane r: row r of Z, forward substitution against L)
    if (lane < s) {
      for (int i = 0; i < s; ++i) {
        double v = Z[lane * RD_LD + i];
        for (int k = 0; k < i; ++k) v -= A[lane * RD_LD + k] * Lm[i * RD_LD + k];
        A[lane * RD_LD + i] = v / Lm[i * RD_LD + i];
      }
    }
    __syncwarp();
    for (int i = 0; i < s; ++i)
      if (lane < s && lane > i) {
        const double m = 0.5 * (A[i * RD_LD + lane] + A[lane * RD_LD + i]);
        A[i * RD_LD + lane] = m;
        A[lane * RD_LD + i] = m;
      }
    __syncwarp();
    conv = warp_syev(A, RD_LD, s, w, Z, RD_LD) && conv;
    __syncwarp();
    // column c of the output is eigenpair s-1-c (Rho descending); lane c
    // back-substitutes L^T t = v and scales by 1/Rho
    if (lane < s) {
      const int src = s - 1 - lane;
      const double sig2 = w[src];
      const double rh = sqrt(sig2 > 0.0 ? sig2 : 0.0);
      const double inv = rh > 0.0 ? 1.0 / rh : 0.0;
      double t[RD_MAXS];
#pragma unroll
      for (int i = RD_MAXS - 1; i >= 0; --i) {
        if (i < s) {
          double v = Z[i * RD_LD + src];
#pragma unroll
          for (int k = i + 1; k < RD_MAXS; ++k)
            if (k < s) v -= Lm[k * RD_LD + i] * t[k];
          t[i] = v / Lm[i * RD_LD + i];
        } else {
          t[i] = 0.0;
        }
      }
#pragma unroll
      for (int i = 0; i < RD_MAXS; ++i)
        if (i < s) small[RD_T + i * RD_MAXS + lane] = t[i] * inv;
      const double lam = rh * rh - rho;
      small[RD_LAM + lane] = lam > 0.0 ? lam : 0.0;
    }
  } else {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    for (int i = 0; i < s; ++i)
      if (lane < s) small[RD_T + i * RD_MAXS + lane] = nan;
    if (lane < s) small[RD_LAM + lane] = nan;
  }
  if (lane == 0) {
    small[RD_RHO] = rho;
    small[RD_OK] = (pd && conv) ? 1.0 : 0.0;
  }
}

// E = P_rho T (optional) and the sign word of each row (bit j: E[r, j] > 0)
__global__ void __launch_bounds__(RD_BLOCK) rd_sign_kernel(int n, int s, int ld,
                                                           const double* __restrict__ P,
                                                           const double* __restrict__ Om,
                                                           const double* __restrict__ small,
                                                           unsigned* __restrict__ bits,
                                                           double* __restrict__ E, int lde) {
  __shared__ double T[RD_MAXS * RD_MAXS];
  for (int e = threadIdx.x; e < s * RD_MAXS; e += RD_BLOCK) T[e] = small[RD_T + e];
  __syncthreads();
  const double rho = small[RD_RHO];
  const bool ok = small[RD_OK] != 0.0;
  for (int r = blockIdx.x * RD_BLOCK + threadIdx.x; r < n; r += gridDim.x * RD_BLOCK) {
    double pr[RD_MAXS];
#pragma unroll
    for (int i = 0; i < RD_MAXS; ++i)
      pr[i] = (i < s) ? P[(size_t)i * ld + r] + rho * Om[(size_t)i * ld + r] : 0.0;
    unsigned word = 0u;
    for (int j = 0; j < s; ++j) {
      double e = 0.0;
#pragma unroll
      for (int i = 0; i < RD_MAXS; ++i)
        if (i < s) e += pr[i] * T[i * RD_MAXS + j];
      if (ok && e > 0.0) word |= 1u << j;
      if (E) E[(size_t)j * lde + r] = e;
    }
    bits[r] = word;
  }
}

// per-block partials of w_j^T C w_j over this block's rows (thread per row)
__global__ void __launch_bounds__(RD_BLOCK) rd_cut_kernel(int n, int s,
                                                          const int* __restrict__ rowptr,
                                                          const int* __restrict__ col,
                                                          const double* __restrict__ val,
                                                          const unsigned* __restrict__ bits,
                                                          double* __restrict__ cpart) {
  __shared__ double red[RD_BLOCK / 32][RD_MAXS];
  double acc[RD_MAXS];
#pragma unroll
  for (int j = 0; j < RD_MAXS; ++j) acc[j] = 0.0;
  for (int r = blockIdx.x * RD_BLOCK + threadIdx.x; r < n; r += gridDim.x * RD_BLOCK) {
    const unsigned br = bits[r];
    const int e = rowptr[r + 1];
    for (int p = rowptr[r]; p < e; ++p) {
      const unsigned x = br ^ __ldg(bits + col[p]);
      const double v = val[p];
#pragma unroll
      for (int j = 0; j < RD_MAXS; ++j)
        if (j < s) acc[j] += ((x >> j) & 1u) ? -v : v;
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < RD_MAXS; ++j) {
    if (j < s) {
      const double t = warp_sum(acc[j]);
      if (lane == 0) red[wid][j] = t;
    }
  }
  __syncthreads();
  if (threadIdx.x < s) {
    double t = 0.0;
    for (int q = 0; q < RD_BLOCK / 32; ++q) t += red[q][threadIdx.x];
    cpart[(size_t)blockIdx.x * s + threadIdx.x] = t;
  }
}

// column values summed in block order; value = their maximum
__global__ void rd_final_kernel(int s, int nblocks, const double* __restrict__ cpart,
                                double* __restrict__ value, double* __restrict__ cols) {
  __shared__ double v[RD_MAXS];
  const int j = threadIdx.x;
  if (j < s) {
    double a = 0.0;
    for (int b = 0; b < nblocks; ++b) a += cpart[(size_t)b * s + j];
    v[j] = a;
    if (cols) cols[j] = a;
  }
  __syncthreads();
  if (j == 0) {
    double m = v[0];
    for (int q = 1; q < s; ++q) m = v[q] > m ? v[q] : m;
    *value = m;
  }
}

// ---------------------------------------------------------------- QAP rounding
// qap_round (utils/qap_helpers.py:624-653): for column i of E (i < min(l, s))
// and both signs, the l x l cost max(c) - c with c = +-E[1:, i] reshaped
// row-major (row = facility, column = location), an optimal assignment, and
// its objective trace(W P D P^T) = sum_fg W[f][g] D[pi(f)][pi(g)].  One warp
// per (column, sign): the shortest-augmenting-path Hungarian method with
// row and column potentials (Kuhn 1955, Munkres 1957; O(l^3)), lanes owning
// columns j = lane, lane + 32, ...  Every loop is bounded by l + 1.  A
// non-finite cost (E is NaN where the reconstruction's Cholesky failed)
// gives a NaN candidate, as min/compare over NaN does in the reference.
constexpr int QAP_MAXL = 64;

__global__ void __launch_bounds__(32) qap_lap_kernel(int l, int s2, const double* __restrict__ E,
                                                      int lde, const double* __restrict__ W,
                                                      const double* __restrict__ D,
                                                      double* __restrict__ vals,
                                                      int* __restrict__ perms) {
  __shared__ double a[QAP_MAXL * QAP_MAXL];
  __shared__ double u[QAP_MAXL + 1], v[QAP_MAXL + 1], minv[QAP_MAXL + 1];
  __shared__ int p[QAP_MAXL + 1], way[QAP_MAXL + 1], used[QAP_MAXL + 1], pi[QAP_MAXL];
  const int lane = threadIdx.x, n = l, nn = l * l;
  const int col = blockIdx.x % s2;
  const double sgn = (blockIdx.x < s2) ? 1.0 : -1.0;
  const double INF = __longlong_as_double(0x7ff0000000000000LL);
  const double NaN = __longlong_as_double(0x7ff8000000000000LL);
  // cost = max(c) - c
  double mx = -INF;
  bool finite = true;
  for (int e = lane; e < nn; e += 32) {
    const double c = sgn * E[(size_t)col * lde + 1 + e];
    finite = finite && isfinite(c);
    a[e] = c;
    mx = fmax(mx, c);
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  finite = __all_sync(0xffffffffu, finite);
  if (!finite) {
    if (lane == 0) vals[blockIdx.x] = NaN;
    for (int r = lane; r < n; r += 32) perms[(size_t)blockIdx.x * l + r] = -1;
    return;
  }
  for (int e = lane; e < nn; e += 32) a[e] = mx - a[e];
  for (int j = lane; j <= n; j += 32) { u[j] = 0.0; v[j] = 0.0; p[j] = 0; way[j] = 0; }
  __syncwarp();
  bool good = true;
  for (int i = 1; i <= n && good; ++i) {
    if (lane == 0) p[0] = i;
    for (int j = lane; j <= n; j += 32) { minv[j] = INF; used[j] = 0; }
    __syncwarp();
    int j0 = 0;
    bool closed = false;
    for (int it = 0; it <= n && !closed; ++it) {
      if (lane == 0) used[j0] = 1;
      __syncwarp();
      const int i0 = p[j0];
      const double ui0 = u[i0];
      double best = INF;
      int bj = 0x7fffffff;
      for (int j = lane; j <= n; j += 32) {
        if (j >= 1 && !used[j]) {
          const double cur = a[(i0 - 1) * n + (j - 1)] - ui0 - v[j];
          if (cur < minv[j]) { minv[j] = cur; way[j] = j0; }
          if (minv[j] < best || (minv[j] == best && j < bj)) { best = minv[j]; bj = j; }
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
        if (ob < best || (ob == best && oj < bj)) { best = ob; bj = oj; }
      }
      __syncwarp();
      if (bj == 0x7fffffff) { good = false; break; }
      for (int j = lane; j <= n; j += 32) {
        if (used[j]) { u[p[j]] += best; v[j] -= best; }
        else minv[j] -= best;
      }
      __syncwarp();
      j0 = bj;
      closed = (p[j0] == 0);
    }
    if (!closed) good = false;
    if (good && lane == 0) {
      int jj = j0;
      for (int g = 0; g <= n && jj != 0; ++g) {
        const int j1 = way[jj];
        p[jj] = p[j1];
        jj = j1;
      }
    }
    __syncwarp();
  }
  if (!good) {
    if (lane == 0) vals[blockIdx.x] = NaN;
    for (int r = lane; r < n; r += 32) perms[(size_t)blockIdx.x * l + r] = -1;
    return;
  }
  for (int j = lane + 1; j <= n; j += 32) pi[p[j] - 1] = j - 1;   // facility -> location
  __syncwarp();
  double acc = 0.0;
  for (int f = lane; f < n; f += 32) {
    const int pf = pi[f];
    for (int g = 0; g < n; ++g) acc += W[f * l + g] * D[pf * l + pi[g]];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) vals[blockIdx.x] = acc;
  for (int r = lane; r < n; r += 32) perms[(size_t)blockIdx.x * l + r] = pi[r];
}

// min over the positive candidates, min over the negative ones (NaN
// propagating, as jnp.min), then the reference's select(min_pos < min_neg)
__global__ void qap_final_kernel(int s2, const double* __restrict__ vals, double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  double mp = vals[0], mn = vals[s2];
  for (int i = 1; i < s2; ++i) {
    mp = (isnan(mp) || isnan(vals[i])) ? __longlong_as_double(0x7ff8000000000000LL) : fmin(mp, vals[i]);
    const double w = vals[s2 + i];
    mn = (isnan(mn) || isnan(w)) ? __longlong_as_double(0x7ff8000000000000LL) : fmin(mn, w);
  }
  *out = (mp < mn) ? mp : mn;
}

static int rd_blocks(long long work, long long per_block, int cap) {
  long long b = (work + per_block - 1) / per_block;
  if (b > cap) b = cap;
  if (b > RD_MAXB) b = RD_MAXB;
  return b < 1 ? 1 : (int)b;
}

// the Gram pass, the s x s algebra and the sign pass
static int rd_reconstruct(int n, int s, const double* Om, const double* P, int ld, double eps,
                          const RoundWs& w, double* E, int lde, cudaStream_t st) {
  const int E3 = 3 * s * s;
  const int tiles = (n + RD_ROWS - 1) / RD_ROWS;
  const int gb = rd_blocks((long long)n * E3, 16384, tiles);
  if (E3 <= RD_BLOCK) rd_gram_kernel<1><<<gb, RD_BLOCK, 0, st>>>(n, s, ld, P, Om, w.gpart);
  else if (E3 <= 4 * RD_BLOCK) rd_gram_kernel<4><<<gb, RD_BLOCK, 0, st>>>(n, s, ld, P, Om, w.gpart);
  else rd_gram_kernel<12><<<gb, RD_BLOCK, 0, st>>>(n, s, ld, P, Om, w.gpart);
  rd_small_kernel<<<1, RD_BLOCK, 0, st>>>(n, s, gb, eps, w.gpart, w.small);
  const int sb = rd_blocks(n, RD_BLOCK, 4 * 152);
  rd_sign_kernel<<<sb, RD_BLOCK, 0, st>>>(n, s, ld, P, Om, w.small, w.bits, E, lde);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("reconstruct_from_sketch: launch failed: %s", cudaGetErrorString(e));
    return -5;
  }
  return 0;
}

static int rd_check(int n, int s, int ld, const void* Om, const void* P, void* ws, size_t wsb,
                    const char* what) {
  if (n < 1 || s < 1 || s > RD_MAXS || ld < n) {
    set_error("%s: bad sizes n=%d s=%d ld=%d (s must be in [1, %d])", what, n, s, ld, RD_MAXS);
    return -2;
  }
  if (!Om || !P || !ws) { set_error("%s: null pointer", what); return -2; }
  if (wsb < rd_bytes(n, s)) {
    set_error("%s: workspace of %zu bytes, %zu needed", what, wsb, rd_bytes(n, s));
    return -2;
  }
  return 0;
}

}  // namespace usbs

using namespace usbs;

extern "C" {

size_t usbs_round_workspace_bytes(int n, int s) {
  if (n < 1 || s < 1 || s > RD_MAXS) return 0;
  return rd_bytes(n, s);
}

int usbs_reconstruct_from_sketch(int n, int s, const double* Omega, const double* P, int ld,
                                 double approx_eps, double* E, int lde, double* Lambda,
                                 void* workspace, size_t workspace_bytes, void* stream) {
  int rc = rd_check(n, s, ld, Omega, P, workspace, workspace_bytes, "reconstruct_from_sketch");
  if (rc) return rc;
  if (E && lde < n) { set_error("reconstruct_from_sketch: lde=%d < n=%d", lde, n); return -2; }
  const RoundWs w = rd_carve(workspace, n, s);
  cudaStream_t st = (cudaStream_t)stream;
  rc = rd_reconstruct(n, s, Omega, P, ld, approx_eps, w, E, lde, st);
  if (rc) return rc;
  if (Lambda &&
      cudaMemcpyAsync(Lambda, w.small + RD_LAM, (size_t)s * sizeof(double),
                      cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
    set_error("reconstruct_from_sketch: copy of Lambda failed");
    return -5;
  }
  return 0;
}

int usbs_maxcut_round(int n, int s, const double* Omega, const double* P, int ld,
                      const int* rowptr, const int* col, const double* val, double approx_eps,
                      double* value, double* column_values, unsigned* signs, void* workspace,
                      size_t workspace_bytes, void* stream) {
  int rc = rd_check(n, s, ld, Omega, P, workspace, workspace_bytes, "maxcut_round");
  if (rc) return rc;
  if (!rowptr || !col || !val || !value) { set_error("maxcut_round: null pointer"); return -2; }
  RoundWs w = rd_carve(workspace, n, s);
  if (signs) w.bits = signs;
  cudaStream_t st = (cudaStream_t)stream;
  rc = rd_reconstruct(n, s, Omega, P, ld, approx_eps, w, nullptr, n, st);
  if (rc) return rc;
  const int cb = rd_blocks(n, RD_BLOCK, 4 * 152);
  rd_cut_kernel<<<cb, RD_BLOCK, 0, st>>>(n, s, rowptr, col, val, w.bits, w.cpart);
  rd_final_kernel<<<1, 32, 0, st>>>(s, cb, w.cpart, value, column_values);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("maxcut_round: launch failed: %s", cudaGetErrorString(e));
    return -5;
  }
  return 0;
}

size_t usbs_qap_round_workspace_bytes(int l, int s) {
  if (l < 1 || l > QAP_MAXL || s < 1 || s > RD_MAXS) return 0;
  const int n = l * l + 1, s2 = s < l ? s : l;
  return rd_bytes(n, s) + rd_align((size_t)n * s * sizeof(double)) +
         rd_align((size_t)2 * s2 * sizeof(double)) + rd_align((size_t)2 * s2 * l * sizeof(int));
}

int usbs_qap_round(int l, int s, const double* Omega, const double* P, int ld, const double* W,
                   const double* D, double approx_eps, double* value, double* candidate_values,
                   int* candidate_perms, void* workspace, size_t workspace_bytes, void* stream) {
  if (l < 1 || l > QAP_MAXL) {
    set_error("qap_round: l=%d must be in [1, %d]", l, QAP_MAXL);
    return -2;
  }
  const int n = l * l + 1;
  int rc = rd_check(n, s, ld, Omega, P, workspace, workspace_bytes, "qap_round");
  if (rc) return rc;
  if (!W || !D || !value) { set_error("qap_round: null pointer"); return -2; }
  const size_t need = usbs_qap_round_workspace_bytes(l, s);
  if (workspace_bytes < need) {
    set_error("qap_round: workspace of %zu bytes, %zu needed", workspace_bytes, need);
    return -2;
  }
  const int s2 = s < l ? s : l;
  RoundWs w = rd_carve(workspace, n, s);
  char* q = (char*)workspace + rd_bytes(n, s);
  double* E = (double*)q; q += rd_align((size_t)n * s * sizeof(double));
  double* vals = candidate_values ? candidate_values : (double*)q;
  q += rd_align((size_t)2 * s2 * sizeof(double));
  int* perms = candidate_perms ? candidate_perms : (int*)q;
  cudaStream_t st = (cudaStream_t)stream;
  rc = rd_reconstruct(n, s, Omega, P, ld, approx_eps, w, E, n, st);
  if (rc) return rc;
  qap_lap_kernel<<<2 * s2, 32, 0, st>>>(l, s2, E, n, W, D, vals, perms);
  qap_final_kernel<<<1, 32, 0, st>>>(s2, vals, value);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("qap_round: launch failed: %s", cudaGetErrorString(e));
    return -5;
  }
  return 0;
}

}  // extern "C"
