// USBS outer iteration on the device (reference: solver/usbs.py:436-789).
//
// Every n- or m-sized step is a kernel over HBM-resident state; the k x k and
// s x s work runs in the single-CTA FP64 kernels of ipm.cu; the Lanczos step is
// the cooperative team kernel of lanczos.cu.  The host loop below only sequences
// launches and reads 3 doubles back per condition check (the reference's
// cond_func, solver/usbs.py:502-540), so an outer iteration has no other host
// synchronisation.  The per-iteration arithmetic follows body_func
// (solver/usbs.py:543-688); the notes at each step name the lines.
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <vector>
#include "../../include/usbs_gb300.h"
#include "common.cuh"
#include "dense.cuh"
#include "internal.h"
#include "solver.h"

namespace usbs {

constexpr int GR_ROWS = 16;          // rows per Gram tile
constexpr int GR_MAXC = IPM_MAXS;    // widest Gram operand (svec dimension)
constexpr int RED_BLOCK = 256;
constexpr double RSQ2_S = 0.70710678118654752440;

// ---------------------------------------------------------------- Gram

struct GramArgs {
  int n, kx, ky, ldx, ldy;
  const double* X;
  const double* Y;
  double* partial;        // gridDim.x * kx * ky
  unsigned int* counter;  // zero on entry, reset by the last block
  double* out;            // kx * ky, row-major [p][q] = sum_i X[i,p] Y[i,q]
  const int* skip;
};

// G = X^T Y over n rows (column-major operands).  Per-block partials are summed
// by the last block to finish, in block order (deterministic).
template <int EPT>
__global__ void __launch_bounds__(RED_BLOCK) gram_kernel(GramArgs a) {
  if (a.skip && *a.skip) return;
  __shared__ double xs[GR_ROWS][GR_MAXC + 1], ys[GR_ROWS][GR_MAXC + 1];
  __shared__ bool last;
  const int E = a.kx * a.ky, tid = threadIdx.x;
  double acc[EPT];
#pragma unroll
  for (int j = 0; j < EPT; ++j) acc[j] = 0.0;
  const int ntiles = (a.n + GR_ROWS - 1) / GR_ROWS;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int r0 = tile * GR_ROWS;
    for (int e = tid; e < GR_ROWS * a.kx; e += RED_BLOCK) {
      const int c = e / GR_ROWS, r = e - c * GR_ROWS;
      xs[r][c] = (r0 + r < a.n) ? a.X[(size_t)c * a.ldx + r0 + r] : 0.0;
    }
    for (int e = tid; e < GR_ROWS * a.ky; e += RED_BLOCK) {
      const int c = e / GR_ROWS, r = e - c * GR_ROWS;
      ys[r][c] = (r0 + r < a.n) ? a.Y[(size_t)c * a.ldy + r0 + r] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < EPT; ++j) {
      const int e = tid + j * RED_BLOCK;
      if (e < E) {
        const int p = e / a.ky, q = e - p * a.ky;
        double s = acc[j];
#pragma unroll
        for (int r = 0; r < GR_ROWS; ++r) s += xs[r][p] * ys[r][q];
        acc[j] = s;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < EPT; ++j) {
    const int e = tid + j * RED_BLOCK;
    if (e < E) a.partial[(size_t)blockIdx.x * E + e] = acc[j];
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // four interleaved chains over the blocks, combined in a fixed order (a
  // single chain of dependent FP64 adds costs ~64 cycles per block)
  const int nb = (int)gridDim.x;
  for (int e = tid; e < E; e += RED_BLOCK) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int b = 0;
    for (; b + 3 < nb; b += 4) {
      s0 += __ldcg(a.partial + (size_t)b * E + e);
      s1 += __ldcg(a.partial + (size_t)(b + 1) * E + e);
      s2 += __ldcg(a.partial + (size_t)(b + 2) * E + e);
      s3 += __ldcg(a.partial + (size_t)(b + 3) * E + e);
    }
    for (; b < nb; ++b) s0 += __ldcg(a.partial + (size_t)b * E + e);
    a.out[e] = (s0 + s1) + (s2 + s3);
  }
  if (tid == 0) *a.counter = 0u;
}

// Symmetric case G = X^T X of a wide X (create_Q_base): the same per-block
// tiles and accumulation order as gram_kernel, for the upper triangle only
// (x_p x_q and x_q x_p round alike, so the lower triangle is its mirror), and
// the partials are summed by gram_sym_reduce_kernel, one thread per entry,
// instead of by one block reading every partial: the same products summed
// in the same order as gram_kernel's.
__device__ __forceinline__ void tri_coords(int t, int k, int& p, int& q) {
  p = 0;
  while (t >= k - p) { t -= k - p; ++p; }
  q = p + t;
}

template <int EPT>
__global__ void __launch_bounds__(RED_BLOCK) gram_sym_kernel(GramArgs a) {
  if (a.skip && *a.skip) return;
  __shared__ double xs[GR_ROWS][GR_MAXC + 1];
  const int k = a.kx, ET = k * (k + 1) / 2, tid = threadIdx.x;
  double acc[EPT];
  int pj[EPT], qj[EPT];
#pragma unroll
  for (int j = 0; j < EPT; ++j) {
    acc[j] = 0.0;
    const int t = tid + j * RED_BLOCK;
    pj[j] = qj[j] = 0;
    if (t < ET) tri_coords(t, k, pj[j], qj[j]);
  }
  const int ntiles = (a.n + GR_ROWS - 1) / GR_ROWS;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int r0 = tile * GR_ROWS;
    for (int e = tid; e < GR_ROWS * k; e += RED_BLOCK) {
      const int c = e / GR_ROWS, r = e - c * GR_ROWS;
      xs[r][c] = (r0 + r < a.n) ? a.X[(size_t)c * a.ldx + r0 + r] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < EPT; ++j) {
      if (tid + j * RED_BLOCK < ET) {
        const int p = pj[j], q = qj[j];
        double s = acc[j];
#pragma unroll
        for (int r = 0; r < GR_ROWS; ++r) s += xs[r][p] * xs[r][q];
        acc[j] = s;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < EPT; ++j) {
    const int t = tid + j * RED_BLOCK;
    if (t < ET) a.partial[(size_t)blockIdx.x * ET + t] = acc[j];
  }
}

// Sums nb blocks' partials of the k(k+1)/2 upper-triangle entries in
// gram_kernel's order (four interleaved chains over the blocks) and writes
// both triangles of the k x k result.
__global__ void gram_sym_reduce_kernel(const double* __restrict__ partial, int nb, int k,
                                       double* __restrict__ out, const int* skip) {
  if (skip && *skip) return;
  const int ET = k * (k + 1) / 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ET) return;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int b = 0;
  for (; b + 3 < nb; b += 4) {
    s0 += partial[(size_t)b * ET + t];
    s1 += partial[(size_t)(b + 1) * ET + t];
    s2 += partial[(size_t)(b + 2) * ET + t];
    s3 += partial[(size_t)(b + 3) * ET + t];
  }
  for (; b < nb; ++b) s0 += partial[(size_t)b * ET + t];
  const double v = (s0 + s1) + (s2 + s3);
  int p, q;
  tri_coords(t, k, p, q);
  out[p * k + q] = v;
  out[q * k + p] = v;
}

// ---------------------------------------------------------------- SpMM

// Y[:, q] = M X[:, q] for q < k, CSR M with double values, L lanes per row.
__global__ void spmm_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                            const double* __restrict__ val, const double* __restrict__ X, int ldx,
                            int k, double* __restrict__ Y, int ldy, int L, const int* skip) {
  if (skip && *skip) return;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int total = gridDim.x * blockDim.x;
  const int lig = gid % L;
  const int lane = threadIdx.x & 31;
  // shuffles stay inside the L-lane group: groups of one warp may leave the
  // row loop at different iterations
  const unsigned gmask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << (lane & ~(L - 1)));
  for (int row = gid / L; row < n; row += total / L) {
    double acc[IPM_MAXK];
#pragma unroll
    for (int q = 0; q < IPM_MAXK; ++q) acc[q] = 0.0;
    const int e = rowptr[row + 1];
    for (int p = rowptr[row] + lig; p < e; p += L) {
      const double v = val[p];
      const int c = col[p];
#pragma unroll
      for (int q = 0; q < IPM_MAXK; ++q)
        if (q < k) acc[q] += v * X[(size_t)q * ldx + c];
    }
#pragma unroll
    for (int q = 0; q < IPM_MAXK; ++q) {
      if (q < k) {
        double s = acc[q];
        for (int o = L >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(gmask, s, o, L);
        if (lig == 0) Y[(size_t)q * ldy + row] = s;
      }
    }
  }
}

// ---------------------------------------------------------------- constraint passes

// svec(B_c), B_c = sum_{t in c} a_t V[i_t] V[j_t]^T: one warp per constraint,
// lanes over svec entries (solver/utils.py:55-61).
__global__ void svec_project_kernel(int m, const int* __restrict__ con_ptr,
                                    const int* __restrict__ t_row, const int* __restrict__ t_col,
                                    const double* __restrict__ t_a, const double* __restrict__ V,
                                    int ldv, int k, double* __restrict__ Pm, int ldm,
                                    const int* skip) {
  if (skip && *skip) return;
  const int lane = threadIdx.x & 31;
  const int s = k * (k + 1) / 2;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  int bb[3], cc[3];
  for (int u = 0; u < 3; ++u) {
    const int a = lane + 32 * u;
    int b = (int)((sqrt(8.0 * a + 1.0) - 1.0) * 0.5);
    while ((b + 1) * (b + 2) / 2 <= a) ++b;
    while (b * (b + 1) / 2 > a) --b;
    bb[u] = b;
    cc[u] = a - b * (b + 1) / 2;
  }
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < m; c += warps) {
    double acc[3] = {0.0, 0.0, 0.0};
    const int e = con_ptr[c + 1];
    for (int t = con_ptr[c]; t < e; ++t) {
      const int i = t_row[t], j = t_col[t];
      const double av = t_a[t];
#pragma unroll
      for (int u = 0; u < 3; ++u) {
        const int a = lane + 32 * u;
        if (a < s) {
          const int b = bb[u], q = cc[u];
          double v;
          if (b == q) v = V[(size_t)b * ldv + i] * V[(size_t)b * ldv + j];
          else v = RSQ2_S * (V[(size_t)q * ldv + i] * V[(size_t)b * ldv + j])
                 + RSQ2_S * (V[(size_t)b * ldv + i] * V[(size_t)q * ldv + j]);
          acc[u] += av * v;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      const int a = lane + 32 * u;
      if (a < s) Pm[(size_t)a * ldm + c] = acc[u];
    }
  }
}

// The three weight vectors of the A* projections side by side after Pm's s
// columns: W[:, 0] = y, W[:, 1] = z_bar, W[:, 2] = b - upsilon (m each).
__global__ void pack3_kernel(int m, const double* __restrict__ y, const double* __restrict__ zbar,
                             const double* __restrict__ bmu, double* __restrict__ W) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m; c += gridDim.x * blockDim.x) {
    W[c] = y[c];
    W[(size_t)m + c] = zbar[c];
    W[(size_t)2 * m + c] = bmu[c];
  }
}

// svec(V^T A*(w) V) = sum_c w_c Pm[c, :] for the three weight vectors (GW,
// s x 3 row-major) back to k x k blocks: GYmC = V^T A*(y) V - V^T C V,
// GZ = V^T A*(z_bar) V, GB = V^T A*(b - upsilon) V (symmetric: the IPM reads
// them through svec only).  One block.
__global__ void unpack_proj_kernel(int k, const double* __restrict__ GW,
                                   const double* __restrict__ GC, double* __restrict__ GYmC,
                                   double* __restrict__ GZ, double* __restrict__ GB) {
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
    const int i = e / k, j = e - (e / k) * k;
    const int b = i > j ? i : j, c = i > j ? j : i;
    const int a = b * (b + 1) / 2 + c;
    const double w = (b == c) ? 1.0 : RSQ2_S;
    GYmC[e] = w * GW[a * 3 + 0] - GC[e];
    GZ[e] = w * GW[a * 3 + 1];
    GB[e] = w * GW[a * 3 + 2];
  }
}

// S_init = trace_ub * 0.99 I / (k + 1): the alternating minimisation's start
__global__ void sinit_kernel(int k, double v, double* __restrict__ S) {
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) S[e] = (e % (k + 1) == 0) ? v : 0.0;
}

// AF[c] = sum_t a_t V[i_t] S+ V[j_t]^T = A(F F^T)_c and AFc[c] with Sc+
// (solver/usbs.py:411-412, 570-571, 627, 639).  One thread per constraint.
__global__ void quadform_kernel(int m, const int* __restrict__ con_ptr,
                                const int* __restrict__ t_row, const int* __restrict__ t_col,
                                const double* __restrict__ t_a, const double* __restrict__ V,
                                int ldv, int k, const double* __restrict__ Sp,
                                const double* __restrict__ Scp, double* __restrict__ AF,
                                double* __restrict__ AFc, const int* skip) {
  if (skip && *skip) return;
  __shared__ double sp[IPM_MAXK * IPM_MAXK], scp[IPM_MAXK * IPM_MAXK];
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) { sp[e] = Sp[e]; scp[e] = Scp[e]; }
  __syncthreads();
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m; c += gridDim.x * blockDim.x) {
    double a1 = 0.0, a2 = 0.0;
    const int e = con_ptr[c + 1];
    for (int t = con_ptr[c]; t < e; ++t) {
      const int i = t_row[t], j = t_col[t];
      double u[IPM_MAXK], w[IPM_MAXK];
#pragma unroll
      for (int q = 0; q < IPM_MAXK; ++q) {
        u[q] = (q < k) ? V[(size_t)q * ldv + i] : 0.0;
        w[q] = (q < k) ? V[(size_t)q * ldv + j] : 0.0;
      }
      double s1 = 0.0, s2 = 0.0;
#pragma unroll
      for (int p = 0; p < IPM_MAXK; ++p) {
        if (p < k) {
          double r1 = 0.0, r2 = 0.0;
#pragma unroll
          for (int q = 0; q < IPM_MAXK; ++q)
            if (q < k) { r1 += sp[p * k + q] * w[q]; r2 += scp[p * k + q] * w[q]; }
          s1 += u[p] * r1;
          s2 += u[p] * r2;
        }
      }
      a1 += t_a[t] * s1;
      a2 += t_a[t] * s2;
    }
    AF[c] = a1;
    if (AFc) AFc[c] = a2;
  }
}

// ---------------------------------------------------------------- m-vector passes

struct MvecArgs {
  int m;
  double* smalls;
  int o_sc;
  double* y;
  double* z;
  double* zbar;
  double* ups;
  double* ycand;
  double* bmu;
  const double* b;
  const double* mask;
  const double* scale_a;
  const double* AF;
  const double* AFc;
  double rho;
  double* partial;
  unsigned int* counter;
  const int* skip;
};

template <int NR>
__device__ __forceinline__ bool mvec_finish(const MvecArgs& a, double (&v)[NR], const bool* is_max,
                                            double* red) {
  __shared__ bool last;
  const int tid = threadIdx.x;
  for (int r = 0; r < NR; ++r) {
    double t = is_max[r] ? block_max(v[r], red) : block_sum(v[r], red);
    if (tid == 0) a.partial[(size_t)blockIdx.x * NR + r] = t;
    __syncthreads();
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return false;
  __threadfence();
  if (tid < NR) {
    double s = is_max[tid] ? 0.0 : 0.0;
    for (int bk = 0; bk < (int)gridDim.x; ++bk) {
      const double t = __ldcg(a.partial + (size_t)bk * NR + tid);
      s = is_max[tid] ? fmax(s, t) : s + t;
    }
    red[tid] = s;
  }
  __syncthreads();
  if (tid == 0) *a.counter = 0u;
  return true;
}

// Start of an iteration: dots with the old z_bar / y, b - upsilon, and the
// alternating-minimisation initial point (solver/usbs.py:422-427, 57, 61).
__global__ void __launch_bounds__(RED_BLOCK) mvec_pre_kernel(MvecArgs a, double trace_ub, int k,
                                                             int reset_eta) {
  if (a.skip && *a.skip) return;
  __shared__ double red[RED_BLOCK / 32];
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.m; c += gridDim.x * blockDim.x) {
    const double zb = a.zbar[c], bmu = a.b[c] - a.ups[c];
    a.bmu[c] = bmu;
    v[0] += zb * zb;
    v[1] += zb * a.y[c];
    v[2] += zb * bmu;
    v[3] += a.b[c] * a.y[c];
  }
  const bool is_max[4] = {false, false, false, false};
  if (!mvec_finish<4>(a, v, is_max, red)) return;
  if (threadIdx.x == 0) {
    double* sc = a.smalls + a.o_sc;
    sc[SC_ZZ] = red[0];
    sc[SC_ZY] = red[1];
    sc[SC_ZBMU] = red[2];
    sc[SC_BY] = red[3];
    if (!reset_eta) return;
    const double tXb = sc[SC_TRXBAR] > 0.0 ? sc[SC_TRXBAR] : trace_ub;
    const double eta0 = (sc[SC_BPO] == 0.0) ? 0.00001 : 0.99 * (1.0 / (k + 1.0));
    sc[SC_ETA_SUB] = (trace_ub / tXb) * eta0;
  }
}

// z = eta z_bar + A(F F^T); y_cand; infeasibility; z_bar <- eta z_bar + A(F_c F_c^T)
// (solver/usbs.py:582-583, 638-639, 648-652).
__global__ void __launch_bounds__(RED_BLOCK) mvec_update_kernel(MvecArgs a) {
  if (a.skip && *a.skip) return;
  __shared__ double red[RED_BLOCK / 32];
  const double eta = a.smalls[a.o_sc + SC_ETA];
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.m; c += gridDim.x * blockDim.x) {
    const double zb = a.zbar[c], bc = a.b[c];
    const double zn = eta * zb + a.AF[c];
    a.z[c] = zn;
    const double yc = a.y[c] - (1.0 / a.rho) * (bc - zn - a.ups[c]);
    a.ycand[c] = yc;
    v[0] += bc * yc;
    v[1] += zb * yc;
    const double inf = fmax(zn - bc, 0.0) + (1.0 - a.mask[c]) * fmax(bc - zn, 0.0);
    const double sa = inf / a.scale_a[c];
    v[2] += sa * sa;
    v[3] = fmax(v[3], fabs(inf) / a.scale_a[c]);
    a.zbar[c] = eta * zb + a.AFc[c];
  }
  const bool is_max[4] = {false, false, false, true};
  if (!mvec_finish<4>(a, v, is_max, red)) return;
  if (threadIdx.x == 0) {
    double* sc = a.smalls + a.o_sc;
    sc[SC_BYC] = red[0];
    sc[SC_ZYC] = red[1];
    sc[SC_INFSQ] = red[2];
    sc[SC_INFMAX] = red[3];
  }
}

// Alternating minimisation over upsilon (solver/usbs.py:413-415): z_next from
// the current S, upsilon_next = mask * max(b - z_next - rho y, 0), gap = max |d upsilon|.
__global__ void __launch_bounds__(RED_BLOCK) mvec_upsilon_kernel(MvecArgs a) {
  if (a.skip && *a.skip) return;
  __shared__ double red[RED_BLOCK / 32];
  const double eta = a.smalls[a.o_sc + SC_ETA];
  double v[1] = {0.0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.m; c += gridDim.x * blockDim.x) {
    const double zn = eta * a.zbar[c] + a.AF[c];
    const double un = a.mask[c] * fmax(a.b[c] - zn - a.rho * a.y[c], 0.0);
    v[0] = fmax(v[0], fabs(a.ups[c] - un));
    a.ups[c] = un;
  }
  const bool is_max[1] = {true};
  if (!mvec_finish<1>(a, v, is_max, red)) return;
  if (threadIdx.x == 0) {
    double* sc = a.smalls + a.o_sc;
    sc[SC_UPSGAP] = red[0];
    sc[SC_ETA_SUB] = sc[SC_ETA];
  }
}

// y <- y_cand after a descent step (solver/usbs.py:623-625)
__global__ void descent_copy_kernel(int m, const double* smalls, int o_sc, double* y,
                                    const double* ycand, const int* skip) {
  if (skip && *skip) return;
  if (smalls[o_sc + SC_DESCENT] == 0.0) return;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m; c += gridDim.x * blockDim.x)
    y[c] = ycand[c];
}

// ---------------------------------------------------------------- row passes

struct RowsArgs {
  int n, k, kp, ssk, mode;  // mode 0 sketch, 1 dense X (handled elsewhere), 2 diag
  const double* V;
  int ldv;
  double* P;
  double* Pbar;
  int ldp;
  const double* smalls;
  int o_sc, o_M, o_Mc, o_Splus, o_Scplus, o_Wpast;
  double* Vn;
  int ldvn;
  const int* skip;
  // constraint evaluation in the same pass (every constraint one diagonal
  // entry): row i is constraint row_con[i]; nullptr leaves it to quadform_kernel
  const int* row_con;
  const int* con_ptr;
  const double* t_a;
  double* AF;
  double* AFc;
};

// Constraint of each row when every constraint is a single diagonal entry
// (A(X)_c = a_c X_ii, as in MaxCut's diag(X) = b): row_con[i] = c.  row_con
// starts at -1 and row_con[n] at 0; row_con[n] becomes non-zero unless the
// map is a bijection between the constraints (m = n) and the rows.
__global__ void diag_map_kernel(int n, int m, const int* __restrict__ con_ptr,
                                const int* __restrict__ t_row, const int* __restrict__ t_col,
                                int* __restrict__ row_con) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m; c += gridDim.x * blockDim.x) {
    const int t0 = con_ptr[c], t1 = con_ptr[c + 1];
    bool ok = (t1 - t0 == 1);
    const int i = ok ? t_row[t0] : -1;
    if (ok && (t_col[t0] != i || i < 0 || i >= n)) ok = false;
    if (ok && atomicExch(&row_con[i], c) != -1) ok = false;
    if (!ok) atomicOr(&row_con[n], 1);
  }
}

// P <- eta P_bar + F (F^T Omega), P_bar <- eta P_bar + F_c (F_c^T Omega) and the
// kept directions V W[:, k_curr:] of the next basis (solver/usbs.py:572-580,
// 628-636, 640).  One thread per row.  With row_con, the same pass over V also
// evaluates the constraints A(F F^T) and A(F_c F_c^T) (solver/usbs.py:411-412,
// 570-571), each row's value computed as quadform_kernel computes it.
__global__ void rows_update_kernel(RowsArgs a) {
  if (a.skip && *a.skip) return;
  __shared__ double Ms[IPM_MAXK * 64], Mcs[IPM_MAXK * 64], Wp[IPM_MAXK * IPM_MAXK];
  __shared__ double Sp[IPM_MAXK * IPM_MAXK], Scp[IPM_MAXK * IPM_MAXK];
  const int k = a.k, kp = a.kp, ssk = a.ssk;
  const double* sm = a.smalls;
  if (a.mode == 0)
    for (int e = threadIdx.x; e < k * ssk; e += blockDim.x) { Ms[e] = sm[a.o_M + e]; Mcs[e] = sm[a.o_Mc + e]; }
  if (a.mode == 2 || a.row_con)
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) { Sp[e] = sm[a.o_Splus + e]; Scp[e] = sm[a.o_Scplus + e]; }
  for (int e = threadIdx.x; e < k * kp; e += blockDim.x) Wp[e] = sm[a.o_Wpast + e];
  __syncthreads();
  const double eta = sm[a.o_sc + SC_ETA];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
    double v[IPM_MAXK];
#pragma unroll
    for (int q = 0; q < IPM_MAXK; ++q) v[q] = (q < k) ? a.V[(size_t)q * a.ldv + i] : 0.0;
    if (a.row_con) {
      // v^T S+ v and v^T Sc+ v in quadform_kernel's order (u = w = v)
      double s1 = 0.0, s2 = 0.0;
#pragma unroll
      for (int p = 0; p < IPM_MAXK; ++p) {
        if (p < k) {
          double r1 = 0.0, r2 = 0.0;
#pragma unroll
          for (int q = 0; q < IPM_MAXK; ++q)
            if (q < k) { r1 += Sp[p * k + q] * v[q]; r2 += Scp[p * k + q] * v[q]; }
          s1 += v[p] * r1;
          s2 += v[p] * r2;
        }
      }
      const int c = a.row_con[i];
      const double ta = a.t_a[a.con_ptr[c]];
      double a1 = 0.0, a2 = 0.0;
      a1 += ta * s1;
      a2 += ta * s2;
      a.AF[c] = a1;
      if (a.AFc) a.AFc[c] = a2;
    }
    if (a.mode == 0) {
      for (int c = 0; c < ssk; ++c) {
        double s1 = 0.0, s2 = 0.0;
#pragma unroll
        for (int q = 0; q < IPM_MAXK; ++q)
          if (q < k) { s1 += v[q] * Ms[q * ssk + c]; s2 += v[q] * Mcs[q * ssk + c]; }
        const double pb = a.Pbar[(size_t)c * a.ldp + i];
        a.P[(size_t)c * a.ldp + i] = eta * pb + s1;
        a.Pbar[(size_t)c * a.ldp + i] = eta * pb + s2;
      }
    } else if (a.mode == 2) {
      double s1 = 0.0, s2 = 0.0;
#pragma unroll
      for (int p = 0; p < IPM_MAXK; ++p) {
        if (p < k) {
          double r1 = 0.0, r2 = 0.0;
#pragma unroll
          for (int q = 0; q < IPM_MAXK; ++q)
            if (q < k) { r1 += Sp[p * k + q] * v[q]; r2 += Scp[p * k + q] * v[q]; }
          s1 += v[p] * r1;
          s2 += v[p] * r2;
        }
      }
      const double pb = a.Pbar[i];
      a.P[i] = eta * pb + s1;
      a.Pbar[i] = eta * pb + s2;
    }
    for (int c = 0; c < kp; ++c) {
      double s = 0.0;
#pragma unroll
      for (int q = 0; q < IPM_MAXK; ++q)
        if (q < k) s += v[q] * Wp[q * kp + c];
      a.Vn[(size_t)c * a.ldvn + i] = s;
    }
  }
}

// Dense-X mode (sketch_dim = -1): X <- eta X_bar + V S V^T, X_bar <- eta X_bar + V Sc+ V^T
// (solver/usbs.py:575-576, 631-632).  X, X_bar row-major n x n.
__global__ void xmode_kernel(int n, int k, const double* __restrict__ V, int ldv,
                             const double* smalls, int o_sc, int o_S, int o_Scplus,
                             double* __restrict__ X, double* __restrict__ Xbar, const int* skip) {
  if (skip && *skip) return;
  __shared__ double S[IPM_MAXK * IPM_MAXK], Sc[IPM_MAXK * IPM_MAXK];
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) { S[e] = smalls[o_S + e]; Sc[e] = smalls[o_Scplus + e]; }
  __syncthreads();
  const double eta = smalls[o_sc + SC_ETA];
  const long long total = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e - (long long)i * n);
    double s1 = 0.0, s2 = 0.0;
    for (int p = 0; p < k; ++p) {
      const double vi = V[(size_t)p * ldv + i];
      double r1 = 0.0, r2 = 0.0;
      for (int q = 0; q < k; ++q) {
        const double vj = V[(size_t)q * ldv + j];
        r1 += S[p * k + q] * vj;
        r2 += Sc[p * k + q] * vj;
      }
      s1 += vi * r1;
      s2 += vi * r2;
    }
    const double xb = Xbar[e];
    X[e] = eta * xb + s1;
    Xbar[e] = eta * xb + s2;
  }
}

// Vn[:, :] <- Vn R^-1 (one CholQR pass), one thread per row
__global__ void rows_rinv_kernel(int n, int k, double* __restrict__ Vn, int ld,
                                 const double* __restrict__ Rinv, const int* skip) {
  if (skip && *skip) return;
  __shared__ double Ri[IPM_MAXK * IPM_MAXK];
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) Ri[e] = Rinv[e];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v[IPM_MAXK];
#pragma unroll
    for (int q = 0; q < IPM_MAXK; ++q) v[q] = (q < k) ? Vn[(size_t)q * ld + i] : 0.0;
#pragma unroll
    for (int c = 0; c < IPM_MAXK; ++c) {
      if (c < k) {
        double s = 0.0;
#pragma unroll
        for (int p = 0; p < IPM_MAXK; ++p)
          if (p <= c && p < k) s += v[p] * Ri[p * k + c];
        Vn[(size_t)c * ld + i] = s;
      }
    }
  }
}

// copy `cols` columns of a float/double matrix into a double matrix
template <typename VT>
__global__ void copy_cols_kernel(int n, int cols, const VT* __restrict__ src, int lds,
                                 double* __restrict__ dst, int ldd, const int* skip) {
  if (skip && *skip) return;
  const long long total = (long long)n * cols;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(e / n), i = (int)(e - (long long)c * n);
    dst[(size_t)c * ldd + i] = (double)src[(size_t)c * lds + i];
  }
}

template <typename VT>
__global__ void to_vt_kernel(int n, const double* __restrict__ src, VT* __restrict__ dst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    dst[i] = (VT)src[i];
}

// ---------------------------------------------------------------- scalar step

struct PostArgs {
  double* smalls;
  int o_sc, o_GR, kc;
  const double* alpha;       // Lanczos Ritz values (ascending)
  int refined;               // use the FP64 Rayleigh quotients in smalls[o_GR] instead
  double trace_ub, trace_factor, beta, scale_c, scale_x, bnorm;
  double* trace;             // TR_NUM doubles per iteration (optional)
  int trace_capacity;
  int t;                     // < 0: the iteration counter in smalls (a replayed graph)
  const int* skip;
};

// Candidate dual value, lower bound test, serious/null step and the gaps
// (solver/usbs.py:584, 599-604, 623-625, 637, 643-652).
__global__ void post_kernel(PostArgs a) {
  if (a.skip && *a.skip) return;
  if (threadIdx.x != 0) return;
  double* sc = a.smalls + a.o_sc;
  const int t = a.t >= 0 ? a.t : (int)sc[SC_T];
  double lam0 = -a.alpha[0];
  if (a.refined) lam0 = -a.smalls[a.o_GR];
  const double eta = sc[SC_ETA];
  const double trXb = sc[SC_TRXBAR], bpo = sc[SC_BPO];
  const double trX_n = eta * trXb + sc[SC_TRS];
  const double primal_n = eta * bpo + sc[SC_PFULL];
  const double trXb_n = eta * trXb + sc[SC_SUMLAMC];
  const double bpo_n = eta * bpo + sc[SC_PCUR];
  const double byc = sc[SC_BYC];
  const double cand_pen = byc + a.trace_ub * fmax(lam0, 0.0);
  double ub = byc + (a.trace_ub / a.trace_factor) * fmax(lam0, 0.0);
  const double ub_old = sc[SC_OBJUB];
  ub = (isnan(ub) || isnan(ub_old)) ? __longlong_as_double(0x7ff8000000000000ll)
                                     : (ub < ub_old ? ub : ub_old);
  const double lb = sc[SC_LB];
  const double pen = sc[SC_PEN];
  const bool descent = a.beta * (pen - lb) <= pen - cand_pen;
  const double pen_n = descent ? cand_pen : pen;
  const double scx = a.scale_c * a.scale_x;
  double gap = fabs(ub - primal_n) / scx;
  gap /= 1.0 + fmax(fabs(primal_n), fabs(ub)) / scx;
  const double infgap = (sqrt(sc[SC_INFSQ]) / a.scale_x) / (1.0 + a.bnorm);
  const double maxinf = sc[SC_INFMAX] / a.scale_x;
  sc[SC_LAM0] = lam0;
  sc[SC_TRX] = trX_n;
  sc[SC_TRXBAR] = trXb_n;
  sc[SC_PRIMAL] = primal_n;
  sc[SC_BPO] = bpo_n;
  sc[SC_PEN] = pen_n;
  sc[SC_CANDPEN] = cand_pen;
  sc[SC_LBEST] = lb;
  sc[SC_OBJUB] = ub;
  sc[SC_OBJGAP] = gap;
  sc[SC_INFGAP] = infgap;
  sc[SC_MAXINF] = maxinf;
  sc[SC_DESCENT] = descent ? 1.0 : 0.0;
  sc[SC_T] = t + 1;
  if (a.trace && t < a.trace_capacity) {
    double* r = a.trace + (size_t)t * TR_NUM;
    r[TR_T] = t; r[TR_PRIMAL] = primal_n; r[TR_OBJUB] = ub; r[TR_OBJGAP] = gap;
    r[TR_INFGAP] = infgap; r[TR_MAXINF] = maxinf; r[TR_PEN] = pen_n; r[TR_CANDPEN] = cand_pen;
    r[TR_LB] = lb; r[TR_LAM0] = lam0; r[TR_DESCENT] = descent ? 1.0 : 0.0; r[TR_ETA] = eta;
    r[TR_TRS] = sc[SC_TRS]; r[TR_TRX] = trX_n; r[TR_QITERS] = sc[SC_QITERS];
    r[TR_LITERS] = sc[SC_LITERS]; r[TR_BPO] = bpo_n; r[TR_TRXBAR] = trXb_n;
    r[TR_BY] = descent ? byc : sc[SC_BY];
  }
}

// Rayleigh quotients theta_j = v_j^T Op v_j / v_j^T v_j from two Grams
__global__ void rayleigh_kernel(double* smalls, int o_G1, int o_G2, int o_out, int kc,
                                const int* skip) {
  if (skip && *skip) return;
  const int j = threadIdx.x;
  if (j < kc) smalls[o_out + j] = smalls[o_G1 + j * kc + j] / smalls[o_G2 + j * kc + j];
}

// ---------------------------------------------------------------- host driver

static size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

struct Arena {
  char* base;
  size_t off = 0, cap;
  template <typename T> T* take(size_t count) {
    T* p = (T*)(base ? base + off : nullptr);
    off += a256(count * sizeof(T));
    return p;
  }
};

struct Layout {
  int n, m, k, kc, kp, s, ssk, ld, mL, vt, grid_red, grid_gram;
  // smalls offsets
  int o_QB, o_GC, o_GYmC, o_GZ, o_GB, o_GYC, o_GW, o_VtO, o_Sout, o_Ssub, o_W, o_Splus, o_Scplus,
      o_Wpast, o_M, o_Mc, o_G, o_Rinv, o_GR1, o_GR2, o_GR, o_sc, n_smalls;
  // buffers
  double *smalls, *CV, *CV2, *Vn, *op64, *op64b, *bmu, *AF, *AFc, *ycand, *zbar, *ups, *Pm,
      *gpart, *gpart2, *mpart, *Pbar, *Xbar, *alpha, *beta;
  void *opL, *Q, *lz_work, *q0L;
  int* row_con;     // n + 4: constraint of each row, flag at [n] (diag_map_kernel)
  bool diag = false;   // every constraint one diagonal entry: one pass over V
  unsigned int* counters;
  int* status;
  int* ctl;
  int* skip;
};

static int plan(const usbs_problem* P, const usbs_params* Pa, const DeviceInfo& di, Arena& ar,
                Layout& L) {
  L.n = P->n; L.m = P->m;
  L.kc = Pa->k_curr; L.kp = Pa->k_past; L.k = L.kc + L.kp; L.s = L.k * (L.k + 1) / 2;
  L.ssk = (Pa->sketch_mode == 0) ? Pa->sketch_dim : 0;
  L.ld = (L.n + 31) & ~31;
  L.mL = Pa->lanczos_inner_iterations;
  L.vt = (Pa->precision == 64) ? 8 : 4;
  L.grid_red = di.sm_count * 2;
  L.grid_gram = di.sm_count * 2;
  int o = 0;
  auto take = [&](int cnt) { int r = o; o += (cnt + 3) & ~3; return r; };
  L.o_QB = take(L.s * L.s); L.o_GC = take(L.k * L.k); L.o_GYmC = take(L.k * L.k);
  L.o_GZ = take(L.k * L.k); L.o_GB = take(L.k * L.k); L.o_GYC = take(L.k * L.k);
  L.o_GW = take(L.s * 3);
  L.o_VtO = take(L.k * (L.ssk > 0 ? L.ssk : 1)); L.o_Sout = take(L.k * L.k);
  L.o_Ssub = take(L.k * L.k); L.o_W = take(L.k * L.k); L.o_Splus = take(L.k * L.k);
  L.o_Scplus = take(L.k * L.k); L.o_Wpast = take(L.k * L.k);
  L.o_M = take(L.k * (L.ssk > 0 ? L.ssk : 1)); L.o_Mc = take(L.k * (L.ssk > 0 ? L.ssk : 1));
  L.o_G = take(L.k * L.k); L.o_Rinv = take(L.k * L.k); L.o_GR1 = take(L.kc * L.kc);
  L.o_GR2 = take(L.kc * L.kc); L.o_GR = take(L.kc); L.o_sc = take(SC_NUM);
  L.n_smalls = o;
  L.smalls = ar.take<double>(L.n_smalls);
  L.CV = ar.take<double>((size_t)L.ld * L.k);
  L.CV2 = ar.take<double>((size_t)L.ld * L.k);
  L.Vn = ar.take<double>((size_t)L.ld * L.k);
  L.op64 = ar.take<double>((size_t)(P->nnz > 0 ? P->nnz : 1));
  L.op64b = ar.take<double>((size_t)(P->nnz > 0 ? P->nnz : 1));
  L.opL = (Pa->precision == 64) ? (void*)L.op64 : (void*)ar.take<float>((size_t)(P->nnz > 0 ? P->nnz : 1));
  L.bmu = ar.take<double>(L.m); L.AF = ar.take<double>(L.m); L.AFc = ar.take<double>(L.m);
  L.ycand = ar.take<double>(L.m); L.zbar = ar.take<double>(L.m); L.ups = ar.take<double>(L.m);
  L.Pm = ar.take<double>((size_t)L.m * (L.s + 3));   // Pm, then the 3 weight columns
  L.gpart = ar.take<double>((size_t)L.grid_gram * L.s * L.s);
  L.gpart2 = ar.take<double>((size_t)L.grid_gram * L.k * L.k);
  L.mpart = ar.take<double>((size_t)L.grid_red * 8);
  L.Pbar = (Pa->sketch_mode == 0) ? ar.take<double>((size_t)L.ld * L.ssk)
           : (Pa->sketch_mode == 2) ? ar.take<double>(L.ld) : nullptr;
  L.Xbar = (Pa->sketch_mode == 1) ? ar.take<double>((size_t)L.n * L.n) : nullptr;
  L.alpha = ar.take<double>(2 * MAXM);
  L.beta = L.alpha ? L.alpha + MAXM : nullptr;
  L.Q = ar.take<char>((size_t)L.ld * (L.mL + 1) * L.vt);
  L.q0L = ar.take<char>((size_t)L.ld * L.vt);
  L.counters = ar.take<unsigned int>(64);
  L.status = ar.take<int>(32);
  L.ctl = L.status + 16;
  L.skip = ar.take<int>(4);
  L.row_con = ar.take<int>((size_t)L.n + 4);
  const bool stream = Pa->lanczos_path == 2;
  const int nct = lanczos_team_size(di, L.n, Pa->precision, stream);
  L.lz_work = ar.take<char>(
      lanczos_workspace_bytes(L.n, P->nnz, L.ld, L.mL, Pa->precision, nct, stream));
  return 0;
}

#define CK(x)                                  \
  do {                                         \
    int _rc = (x);                             \
    if (_rc) return _rc;                       \
  } while (0)

static int kerr(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_error("%s: %s", what, cudaGetErrorString(e)); return -5; }
  return 0;
}

struct Solver {
  const usbs_problem* P;
  const usbs_params* Pa;
  usbs_state* S;
  DeviceInfo di;
  Layout L;
  cudaStream_t st;
  int lanes;
  unsigned int* ctr_gram;
  unsigned int* ctr_gram2;
  unsigned int* ctr_m;
  int gram_ctr_next = 0;

  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_l0 = nullptr, ev_l1 = nullptr;
  bool lz_pending = false;
  long long launches = 0;
  // CUDA graph of one outer iteration (captured at the first one, replayed)
  bool use_graph = false, capturing = false;
  cudaStream_t gst = nullptr;        // capture origin (the caller's stream may be the legacy one)
  cudaGraphExec_t gexec = nullptr;
  long long graph_body_launches = 0;
  // event record on the main stream; while capturing, a graph node of its own
  void record(cudaEvent_t e) {
    if (capturing) cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
    else cudaEventRecord(e, st);
  }
  // algorithmic bytes of one Lanczos launch from its counters (ctl[2], [4], [13], [14])
  double lanczos_bytes(const int* c) const {
    const double b = (double)L.vt, n = L.n, nnz = (double)P->nnz;
    const double steps = c[4], sum_nv = c[13], restarts = c[2], sum_kn = c[14];
    const double spmv = (4.0 + b) * nnz + 4.0 * (n + 1) + 2.0 * b * n;   // CSR + x + y
    const double cgs = 3.0 * b * n * sum_nv + 6.0 * b * n * steps;        // 3 Q passes + vectors
    const double rot = restarts * b * n * L.mL + b * n * (sum_kn + 2.0 * restarts);
    return steps * spmv + cgs + rot;
  }
  int gram(const double* X, int ldx, int kx, const double* Y, int ldy, int ky, int n, double* out,
           int side = 0) {
    GramArgs a;
    a.n = n; a.kx = kx; a.ky = ky; a.ldx = ldx; a.ldy = ldy; a.X = X; a.Y = Y;
    a.partial = side ? L.gpart2 : L.gpart;
    a.counter = side ? ctr_gram2 : ctr_gram;
    a.out = out; a.skip = nullptr;
    cudaStream_t st = side ? st2 : this->st;
    ++launches;
    // blocks by work, about 16k FMAs each (few blocks keep the final sum of
    // the per-block partials short), at most grid_gram
    const long long work = (long long)n * kx * ky;
    int blocks = (int)((work + 16383) / 16384);
    const int tiles = (n + GR_ROWS - 1) / GR_ROWS;
    if (blocks > tiles) blocks = tiles;
    if (blocks > L.grid_gram) blocks = L.grid_gram;
    if (blocks < 1) blocks = 1;
    if (X == Y && kx == ky && ldx == ldy && kx * ky > 4 * RED_BLOCK) {
      constexpr int EPT_T = (IPM_MAXS * (IPM_MAXS + 1) / 2 + RED_BLOCK - 1) / RED_BLOCK;
      gram_sym_kernel<EPT_T><<<blocks, RED_BLOCK, 0, st>>>(a);
      ++launches;
      const int et = kx * (kx + 1) / 2;
      gram_sym_reduce_kernel<<<(et + 127) / 128, 128, 0, st>>>(a.partial, blocks, kx, out, nullptr);
      return kerr("gram");
    }
    if (kx * ky <= RED_BLOCK) gram_kernel<1><<<blocks, RED_BLOCK, 0, st>>>(a);
    else if (kx * ky <= 4 * RED_BLOCK) gram_kernel<4><<<blocks, RED_BLOCK, 0, st>>>(a);
    else gram_kernel<(IPM_MAXS * IPM_MAXS + RED_BLOCK - 1) / RED_BLOCK><<<blocks, RED_BLOCK, 0, st>>>(a);
    return kerr("gram");
  }
  int spmm(const double* val, const double* X, int k, double* Y, int side = 0) {
    cudaStream_t st = side ? st2 : this->st;
    ++launches;
    int blocks = (int)(((long long)L.n * lanes + 255) / 256);
    if (blocks > di.sm_count * 8) blocks = di.sm_count * 8;
    if (blocks < 1) blocks = 1;
    spmm_kernel<<<blocks, 256, 0, st>>>(L.n, P->rowptr, P->col, val, X, L.ld, k, Y, L.ld, lanes,
                                        nullptr);
    return kerr("spmm");
  }
  int assemble(double c_scale, const double* w, void* out, int prec, int side = 0) {
    ++launches;
    return assemble_operator((int)P->nnz, P->c_val, c_scale, P->slot_ptr, P->slot_tid, P->t_con,
                             P->t_a0, w, out, prec, side ? st2 : st);
  }
  // V^T (c_scale C + A*(w)) V -> smalls[o]   (side 1: second stream and its own scratch)
  int proj(double c_scale, const double* w, const double* V, int o, int side = 0) {
    const double* val = P->c_val;
    double* op = side ? L.op64b : L.op64;
    double* cv = side ? L.CV2 : L.CV;
    if (w || c_scale != 1.0) {
      CK(assemble(c_scale, w, op, 64, side));
      val = op;
    }
    CK(spmm(val, V, L.k, cv, side));
    return gram(V, L.ld, L.k, cv, L.ld, L.k, L.n, L.smalls + o, side);
  }
  // GYmC, GZ, GB from Pm (svec_project output) and GC: pack the weights, one
  // Gram Pm^T [y z_bar b-upsilon], unpack (this stream)
  int a_proj3() {
    double* W = L.Pm + (size_t)L.m * L.s;
    ++launches;
    pack3_kernel<<<mgrid(), RED_BLOCK, 0, st>>>(L.m, S->y, L.zbar, L.bmu, W);
    CK(kerr("pack3"));
    CK(gram(L.Pm, L.m, L.s, W, L.m, 3, L.m, L.smalls + L.o_GW));
    ++launches;
    unpack_proj_kernel<<<1, 128, 0, st>>>(L.k, L.smalls + L.o_GW, L.smalls + L.o_GC,
                                          L.smalls + L.o_GYmC, L.smalls + L.o_GZ,
                                          L.smalls + L.o_GB);
    return kerr("unpack_proj");
  }
  MvecArgs margs() {
    MvecArgs a;
    a.m = L.m; a.smalls = L.smalls; a.o_sc = L.o_sc; a.y = S->y; a.z = S->z; a.zbar = L.zbar;
    a.ups = L.ups; a.ycand = L.ycand; a.bmu = L.bmu; a.b = P->b; a.mask = P->b_ineq_mask;
    a.scale_a = P->scale_a; a.AF = L.AF; a.AFc = L.AFc; a.rho = Pa->rho; a.partial = L.mpart;
    a.counter = ctr_m; a.skip = nullptr;
    return a;
  }
  int mgrid() const {
    int b = (L.m + RED_BLOCK - 1) / RED_BLOCK;
    if (b > L.grid_red) b = L.grid_red;
    return b < 1 ? 1 : b;
  }
  RowsArgs rows_args(bool with_constraints) const {
    RowsArgs ra;
    const double* V = S->V;
    ra.n = L.n; ra.k = L.k; ra.kp = L.kp; ra.ssk = L.ssk; ra.mode = Pa->sketch_mode;
    ra.V = V; ra.ldv = L.ld; ra.P = S->P; ra.Pbar = L.Pbar; ra.ldp = L.ld; ra.smalls = L.smalls;
    ra.o_sc = L.o_sc; ra.o_M = L.o_M; ra.o_Mc = L.o_Mc; ra.o_Splus = L.o_Splus;
    ra.o_Scplus = L.o_Scplus; ra.o_Wpast = L.o_Wpast; ra.Vn = L.Vn; ra.ldvn = L.ld;
    ra.skip = nullptr;
    ra.row_con = with_constraints ? L.row_con : nullptr;
    ra.con_ptr = P->con_ptr; ra.t_a = P->t_a; ra.AF = L.AF; ra.AFc = L.AFc;
    return ra;
  }
  int rgrid() const {
    int b = (L.n + 255) / 256;
    if (b > di.sm_count * 8) b = di.sm_count * 8;
    return b < 1 ? 1 : b;
  }
  // eigsh on -C + A*(w): leaves num_desired vectors in Q and Ritz values in alpha
  int lanczos(const double* w, int num_desired, bool timed = false) {
    CK(assemble(-1.0, w, L.opL, Pa->precision));
    if (cudaMemcpyAsync(L.Q, L.q0L, (size_t)L.n * L.vt, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return kerr("q0 copy");
    if (timed) {
      record(ev_l0);
      const int rc = lanczos_launch(num_desired);
      record(ev_l1);
      lz_pending = true;
      return rc;
    }
    return lanczos_launch(num_desired);
  }
  int lanczos_launch(int num_desired) {
    LanczosProblem lp;
    lp.n = L.n; lp.ld = L.ld; lp.m = L.mL; lp.num_desired = num_desired;
    lp.max_restarts = Pa->lanczos_max_restarts; lp.nnz = P->nnz; lp.tol = Pa->subprob_eps;
    lp.rowptr = P->rowptr; lp.col = P->col; lp.val = L.opL; lp.Q = L.Q;
    lp.alpha = L.alpha; lp.beta = L.beta; lp.ctl = L.ctl; lp.status = L.status;
    lp.work = L.lz_work;
    lp.rows_per_cta = Pa->lanczos_rows_per_cta;
    lp.no_coop = Pa->lanczos_path == 2 ? 1 : 0;
    const int rc = lanczos_run(di, &lp, 1, Pa->precision, st);
    launches += lanczos_last_launches();
    return rc;
  }
  // after a host sync: fold the last timed launch into the state's counters
  int collect_lanczos() {
    if (!lz_pending) return 0;
    float ms = 0.f;
    int c[16];
    if (cudaEventElapsedTime(&ms, ev_l0, ev_l1) != cudaSuccess ||
        cudaMemcpy(c, L.ctl, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess)
      return kerr("lanczos timing");
    S->lanczos_ms += ms;
    S->lanczos_launches += 1;
    S->lanczos_bytes += lanczos_bytes(c);
    lz_pending = false;
    return 0;
  }
  int copy_q_cols(int cols, double* dst) {
    ++launches;
    int blocks = rgrid();
    if (Pa->precision == 64)
      copy_cols_kernel<double><<<blocks, 256, 0, st>>>(L.n, cols, (const double*)L.Q, L.ld, dst, L.ld, nullptr);
    else
      copy_cols_kernel<float><<<blocks, 256, 0, st>>>(L.n, cols, (const float*)L.Q, L.ld, dst, L.ld, nullptr);
    return kerr("copy cols");
  }
  IpmArgs ipm_args(int mode) {
    IpmArgs a;
    a.mode = mode; a.k = L.k; a.max_iters = Pa->subprob_max_iters; a.ipm_grid = Pa->subprob_max_iters;
    a.eps = Pa->subprob_eps; a.trace_ub = Pa->trace_ub; a.rho = Pa->rho; a.smalls = L.smalls;
    a.o_sc = L.o_sc; a.o_QB = L.o_QB; a.o_GZ = L.o_GZ; a.o_GYmC = L.o_GYmC; a.o_GB = L.o_GB;
    a.o_GYC = L.o_GYC; a.o_Ssub = L.o_Ssub; a.o_Sout = L.o_Sout; a.status = L.status;
    a.skip = nullptr;
    a.dbg = nullptr;
    a.prof = S->debug ? S->debug + 4096 + 8 * mode : nullptr;
    if (S->debug && cur_t == 0) a.dbg = S->debug + 1024 * mode;
    return a;
  }
  int cur_t = 0;
  int run_ipm(int mode) { ++launches; return launch_ipm(ipm_args(mode), st); }
  int read_scalars(double* out, int first, int count) {
    if (cudaMemcpyAsync(out, L.smalls + L.o_sc + first, count * sizeof(double),
                        cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return kerr("read scalars");
    if (cudaStreamSynchronize(st) != cudaSuccess) return kerr("sync");
    return 0;
  }
  int set_scalar(int slot, double v) {
    if (cudaMemcpyAsync(L.smalls + L.o_sc + slot, &v, sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
      return kerr("set scalar");
    return cudaStreamSynchronize(st) == cudaSuccess ? 0 : kerr("sync");
  }
};

static int body(Solver& X, int t) {
  X.cur_t = t;
  Layout& L = X.L;
  const usbs_problem* P = X.P;
  const usbs_params* Pa = X.Pa;
  usbs_state* S = X.S;
  cudaStream_t st = X.st;
  double* V = S->V;
  // ---- projections onto the bundle basis (solver/usbs.py:54-61) ----
  // V^T C V (C V, then the Gram); Pm[c, :] = svec(V^T A_c V) (create_Q_base's
  // rows) and, from the same Pm, the three A* projections: svec(V^T A*(w) V) =
  // Pm^T w for w = y, z_bar and b - upsilon, one Gram against the packed
  // weight columns.  All on this stream: a fork here costs concurrent solves
  // (several per GPU) more in queue waits than the overlap gains one solve.
  CK(X.proj(1.0, nullptr, V, L.o_GC));                // V^T C V
  {
    MvecArgs ma = X.margs();
    ++X.launches;
    mvec_pre_kernel<<<X.mgrid(), RED_BLOCK, 0, st>>>(ma, Pa->trace_ub, L.k, 1);
    CK(kerr("mvec_pre"));
  }
  {
    int blocks = (int)(((long long)L.m * 32 + 255) / 256);
    if (blocks > X.di.sm_count * 16) blocks = X.di.sm_count * 16;
    ++X.launches;
    svec_project_kernel<<<blocks, 256, 0, st>>>(L.m, P->con_ptr, P->t_row, P->t_col, P->t_a, V,
                                                L.ld, L.k, L.Pm, L.m, nullptr);
    CK(kerr("svec_project"));
    CK(X.gram(L.Pm, L.m, L.s, L.Pm, L.m, L.s, L.m, L.smalls + L.o_QB));   // create_Q_base
  }
  CK(X.a_proj3());
  if (L.ssk > 0) CK(X.gram(V, L.ld, L.k, S->Omega, L.ld, L.ssk, L.n, L.smalls + L.o_VtO));
  // alternating-minimisation initial point: S_init = trace_ub * 0.99 I / (k+1)
  ++X.launches;
  sinit_kernel<<<1, 128, 0, st>>>(L.k, Pa->trace_ub * (0.99 * (1.0 / (L.k + 1.0))),
                                  L.smalls + L.o_Ssub);
  CK(kerr("S init"));
  // ---- subproblem: IPM + alternating minimisation over upsilon (solver/usbs.py:359-433) ----
  EigSArgs ea;
  ea.k = L.k; ea.k_curr = L.kc; ea.ssk = L.ssk; ea.smalls = L.smalls; ea.o_sc = L.o_sc;
  ea.o_Sout = L.o_Sout; ea.o_GC = L.o_GC; ea.o_W = L.o_W; ea.o_Splus = L.o_Splus;
  ea.o_Scplus = L.o_Scplus; ea.o_Wpast = L.o_Wpast; ea.o_VtO = L.o_VtO; ea.o_M = L.o_M;
  ea.o_Mc = L.o_Mc; ea.status = L.status; ea.skip = nullptr;
  const int qblocks = X.mgrid();
  for (int pass = 0; pass < Pa->subprob_max_iters; ++pass) {
    CK(X.run_ipm(0));
    ++X.launches;
    CK(launch_eigS(ea, st));
    if (L.diag) {
      // constraint evaluation and the sketch / kept-direction updates in one
      // pass over V (nothing in between reads P, P_bar or the kept directions)
      RowsArgs ra = X.rows_args(true);
      ++X.launches;
      rows_update_kernel<<<X.rgrid(), 256, 0, st>>>(ra);
      CK(kerr("rows_update"));
    } else {
      ++X.launches;
      quadform_kernel<<<qblocks, 256, 0, st>>>(L.m, P->con_ptr, P->t_row, P->t_col, P->t_a, V,
                                               L.ld, L.k, L.smalls + L.o_Splus,
                                               L.smalls + L.o_Scplus, L.AF, L.AFc, nullptr);
      CK(kerr("quadform"));
    }
    if (!P->has_ineq) break;       // upsilon stays 0: the loop ends after one pass
    MvecArgs ma = X.margs();
    ++X.launches;
    mvec_upsilon_kernel<<<X.mgrid(), RED_BLOCK, 0, st>>>(ma);
    CK(kerr("upsilon"));
    double gap = 0.0;
    CK(X.read_scalars(&gap, SC_UPSGAP, 1));
    if (!(gap > Pa->subprob_eps)) break;
    // warm start the next pass from (eta, S) and refresh V^T A*(b - upsilon) V
    if (cudaMemcpyAsync(L.smalls + L.o_Ssub, L.smalls + L.o_Sout, (size_t)L.k * L.k * sizeof(double),
                        cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return kerr("S warm start");
    {
      MvecArgs mb = X.margs();
      ++X.launches;
      mvec_pre_kernel<<<X.mgrid(), RED_BLOCK, 0, st>>>(mb, Pa->trace_ub, L.k, 0);
      CK(kerr("mvec_pre"));
    }
    CK(X.a_proj3());                                  // V^T A*(b - upsilon) V refreshed
  }
  // ---- z, y_cand, infeasibility, z_bar (solver/usbs.py:582-583, 638-639, 648-652) ----
  {
    MvecArgs ma = X.margs();
    ++X.launches;
    mvec_update_kernel<<<X.mgrid(), RED_BLOCK, 0, st>>>(ma);
    CK(kerr("mvec_update"));
  }
  // ---- sketch / X updates and kept directions ----
  if (Pa->sketch_mode == 1) {
    ++X.launches;
    xmode_kernel<<<X.di.sm_count * 8, 256, 0, st>>>(L.n, L.k, V, L.ld, L.smalls, L.o_sc, L.o_Sout,
                                                    L.o_Scplus, S->X, L.Xbar, nullptr);
    CK(kerr("xmode"));
  }
  if (!L.diag) {
    RowsArgs ra = X.rows_args(false);
    ++X.launches;
    rows_update_kernel<<<X.rgrid(), 256, 0, st>>>(ra);
    CK(kerr("rows_update"));
  }
  // ---- lower bound (solver/usbs.py:606-621) on a second stream: it needs V and
  // y_cand only, so it overlaps the Lanczos call below ----
  if (cudaEventRecord(X.ev_fork, st) != cudaSuccess ||
      cudaStreamWaitEvent(X.st2, X.ev_fork, 0) != cudaSuccess)
    return kerr("fork");
  CK(X.proj(-1.0, L.ycand, V, L.o_GYC, 1));     // V^T (A*(y_cand) - C) V (solver/usbs.py:219-220)
  ++X.launches;
  CK(launch_ipm(X.ipm_args(1), X.st2));
  if (cudaEventRecord(X.ev_join, X.st2) != cudaSuccess) return kerr("join record");
  // ---- candidate eigenvectors at y_cand (solver/usbs.py:588-599) ----
  CK(X.lanczos(L.ycand, L.kc, true));
  CK(X.copy_q_cols(L.kc, L.Vn + (size_t)L.kp * L.ld));
  if (cudaStreamWaitEvent(st, X.ev_join, 0) != cudaSuccess) return kerr("join");
  int refined = 0;
  if (Pa->precision != 64) {
    // FP64 Rayleigh quotients of the FP32 Ritz vectors (op64b holds -C + A*(y_cand))
    double* Vc = L.Vn + (size_t)L.kp * L.ld;
    CK(X.spmm(L.op64b, Vc, L.kc, L.CV));
    CK(X.gram(Vc, L.ld, L.kc, L.CV, L.ld, L.kc, L.n, L.smalls + L.o_GR1));
    CK(X.gram(Vc, L.ld, L.kc, Vc, L.ld, L.kc, L.n, L.smalls + L.o_GR2));
    ++X.launches;
    rayleigh_kernel<<<1, 32, 0, st>>>(L.smalls, L.o_GR1, L.o_GR2, L.o_GR, L.kc, nullptr);
    CK(kerr("rayleigh"));
    refined = 1;
  }
  {
    PostArgs pa;
    pa.smalls = L.smalls; pa.o_sc = L.o_sc; pa.o_GR = L.o_GR; pa.kc = L.kc; pa.alpha = L.alpha;
    pa.refined = refined; pa.trace_ub = Pa->trace_ub; pa.trace_factor = Pa->trace_factor;
    pa.beta = Pa->beta; pa.scale_c = P->scale_c; pa.scale_x = P->scale_x; pa.bnorm = P->b_norm;
    pa.trace = S->trace;
    pa.trace_capacity = S->trace ? S->trace_capacity : 0;
    pa.t = t; pa.skip = nullptr;
    ++X.launches;
    post_kernel<<<1, 32, 0, st>>>(pa);
    CK(kerr("post"));
  }
  ++X.launches;
  descent_copy_kernel<<<X.mgrid(), 256, 0, st>>>(L.m, L.smalls, L.o_sc, S->y, L.ycand, nullptr);
  CK(kerr("descent"));
  // ---- next basis: shifted CholQR3 of [V W_past, cand_vecs] (solver/usbs.py:640-642) ----
  for (int pass = 0; pass < 3; ++pass) {
    CK(X.gram(L.Vn, L.ld, L.k, L.Vn, L.ld, L.k, L.n, L.smalls + L.o_G));
    CholQRArgs ca;
    ca.k = L.k; ca.n = L.n; ca.shifted = (pass == 0); ca.smalls = L.smalls; ca.o_G = L.o_G;
    ca.o_Rinv = L.o_Rinv; ca.status = L.status; ca.skip = nullptr;
    ++X.launches;
    CK(launch_cholqr(ca, st));
    ++X.launches;
    rows_rinv_kernel<<<X.rgrid(), 256, 0, st>>>(L.n, L.k, L.Vn, L.ld, L.smalls + L.o_Rinv, nullptr);
    CK(kerr("rinv"));
  }
  if (cudaMemcpyAsync(V, L.Vn, (size_t)L.ld * L.k * sizeof(double), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return kerr("V copy");
  return 0;
}

// One outer iteration.  Problems without inequality constraints (no host
// decision inside the body) whose Lanczos runs as one cluster replay a CUDA
// graph of the body: captured at the first iteration on a stream of the
// solver's own (capture is not possible on the legacy default stream), with
// the iteration number read on the device (post_kernel); each iteration is
// then one cudaGraphLaunch into the caller's stream and the host does not
// wait between iterations of a condition-check block.  If the capture fails
// the solve continues eagerly and graph_iterations holds -(the CUDA error).
static bool graph_wanted(const Solver& X) {
  const char* e = getenv("USBS_GRAPH");           // 0 runs every iteration eagerly
  if (e && atoi(e) == 0) return false;
  return !X.P->has_ineq && !X.S->debug &&
         lanczos_kernel_kind(X.L.n, X.Pa->lanczos_inner_iterations, X.Pa->precision) == 1;
}

static int step(Solver& X, int t) {
  if (!X.use_graph) return body(X, t);
  if (!X.gexec) {
    cudaGraph_t g = nullptr;
    const long long l0 = X.launches;
    cudaError_t e = cudaStreamCreateWithFlags(&X.gst, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(X.gst, cudaStreamCaptureModeRelaxed);
    int rc = -5;
    if (e == cudaSuccess) {
      const cudaStream_t user = X.st;
      X.st = X.gst;
      X.capturing = true;
      rc = body(X, -1);
      X.capturing = false;
      X.st = user;
      e = cudaStreamEndCapture(X.gst, &g);
      if (rc != 0 && e == cudaSuccess) e = cudaErrorUnknown;
    }
    if (e == cudaSuccess && g) e = cudaGraphInstantiate(&X.gexec, g, 0);
    if (g) cudaGraphDestroy(g);
    X.graph_body_launches = X.launches - l0;
    X.launches = l0;
    if (e != cudaSuccess || !X.gexec) {
      cudaGetLastError();                           // nothing was launched: run eagerly
      if (X.gexec) cudaGraphExecDestroy(X.gexec);
      X.gexec = nullptr;
      X.use_graph = false;
      X.lz_pending = false;
      X.S->graph_iterations = -(long long)(e != cudaSuccess ? e : cudaErrorUnknown);
      return body(X, t);
    }
  }
  X.launches += X.graph_body_launches;
  X.lz_pending = true;
  ++X.S->graph_iterations;
  return cudaGraphLaunch(X.gexec, X.st) == cudaSuccess ? 0 : kerr("graph launch");
}

// geometric schedule of condition checks (utils/loop.py:84-98)
static std::vector<long long> cond_schedule(long long maxiter, double base) {
  std::vector<long long> out;
  if (base <= 1.0) { out.assign((size_t)maxiter, 1); return out; }
  const double num = std::ceil(std::log((base - 1) * maxiter - 1) / std::log(base)) + 1;
  long long csum = 0, kept = 0;
  for (int i = 0; i < (int)num; ++i) {
    const long long s = (long long)std::pow(base, (double)i);
    csum += s;
    if (csum >= maxiter) continue;
    out.push_back(s);
    kept += s;
  }
  out.push_back(maxiter - kept);
  return out;
}

// ================================================================ CGAL
// cgal() (solver/cgal.py:21-243) on the device: per iteration one m-vector
// pass (projection onto the constraint set, the adjoint weights and the gap
// and infeasibility sums), eigsh(1) on -C + A*(adj), C v and A(v v^T), a
// second m-vector pass (the new z and the dual-step denominator, its last block
// forms every scalar of the iteration), the y step and the rank-one sketch (or
// dense X) update.  All reductions are fixed-order (per-block partials summed
// by the last block), so results are deterministic.

enum CgalSlot {
  CG_ADJZ = 0, CG_YDZ, CG_DZDZ, CG_INF2, CG_PB2, CG_INFMAX, CG_VCV, CG_VV, CG_ADJAV, CG_ZNPB,
  CG_PRIMAL, CG_TRX, CG_OBJGAP, CG_INFGAP, CG_MAXINF, CG_DSS, CG_EIG0, CG_NUM
};

struct CgalArgs {
  int m, t;
  double* sc;                       // CG_NUM scalars, then v^T Omega
  double *y, *z, *adj, *zn, *Av;
  const double *b, *mask, *scale_a;
  double scale_c, scale_x, beta, beta_next, eta, trace_ub, beta0;
  double* partial;
  unsigned int* counter;
  double* trace;
  int trace_capacity;
};

__device__ __forceinline__ MvecArgs cg_fin(const CgalArgs& a) {
  MvecArgs f;
  f.partial = a.partial;
  f.counter = a.counter;
  return f;
}

// proj_b, adj and the sums of solver/cgal.py:104-107 and 118-138 that use the
// current z
__global__ void __launch_bounds__(RED_BLOCK) cgal_pre_kernel(CgalArgs a) {
  __shared__ double red[RED_BLOCK / 32];
  double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.m; c += gridDim.x * blockDim.x) {
    const double y = a.y[c], z = a.z[c], b = a.b[c], mk = a.mask[c], sa = a.scale_a[c];
    const double pb = (1.0 - mk) * b + mk * fmin(z + (1.0 / a.beta) * y, b);
    const double dz = z - pb;
    const double adj = y + a.beta * dz;
    a.adj[c] = adj;
    v[0] += adj * z;
    v[1] += y * dz;
    v[2] += dz * dz;
    const double pb0 = (1.0 - mk) * b + mk * fmin(z, b);
    const double e = ((z - pb0) / sa) / a.scale_x;
    const double f = (pb0 / sa) / a.scale_x;
    v[3] += e * e;
    v[4] += f * f;
    v[5] = fmax(v[5], fabs((z - pb0) / sa));
  }
  const bool is_max[6] = {false, false, false, false, false, true};
  if (!mvec_finish<6>(cg_fin(a), v, is_max, red)) return;
  if (threadIdx.x == 0)
    for (int r = 0; r < 6; ++r) a.sc[CG_ADJZ + r] = red[r];
}

// v = Q[:, 0], or 0 when the smallest eigenvalue is >= 0 (solver/cgal.py:113-116)
template <typename VT>
__global__ void cgal_v_kernel(int n, const VT* __restrict__ Q, const double* alpha,
                              double* __restrict__ v, double* sc) {
  const bool zero = !(alpha[0] < 0.0);
  if (blockIdx.x == 0 && threadIdx.x == 0) sc[CG_EIG0] = alpha[0];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    v[i] = zero ? 0.0 : (double)Q[i];
}

// z_next and the dual-step denominator; the last block forms the iteration's
// scalars (solver/cgal.py:108-112, 139-170)
__global__ void __launch_bounds__(RED_BLOCK) cgal_post_kernel(CgalArgs a) {
  __shared__ double red[RED_BLOCK / 32];
  double v[2] = {0.0, 0.0};
  const double eta = a.eta, tr = a.trace_ub;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.m; c += gridDim.x * blockDim.x) {
    const double zn = (1.0 - eta) * a.z[c] + eta * tr * a.Av[c];
    a.zn[c] = zn;
    const double b = a.b[c], mk = a.mask[c];
    const double pbn = (1.0 - mk) * b + mk * fmin(zn + (1.0 / a.beta_next) * a.y[c], b);
    v[0] += a.adj[c] * a.Av[c];
    const double d = zn - pbn;
    v[1] += d * d;
  }
  const bool is_max[2] = {false, false};
  if (!mvec_finish<2>(cg_fin(a), v, is_max, red)) return;
  if (threadIdx.x != 0) return;
  double* sc = a.sc;
  sc[CG_ADJAV] = red[0];
  sc[CG_ZNPB] = red[1];
  const double primal = sc[CG_PRIMAL];
  const double scx = a.scale_c * a.scale_x;
  // v^T A*(adj) v = adj . A(v v^T)
  double sdg = tr * sc[CG_VCV] - primal;
  sdg += sc[CG_ADJZ];
  sdg -= tr * red[0];
  double og = sdg - sc[CG_YDZ];
  og -= 0.5 * a.beta * sc[CG_DZDZ];
  og = og / scx;
  og /= 1.0 + fabs(primal) / scx;
  const double ig = sqrt(sc[CG_INF2]) / (1.0 + sqrt(sc[CG_PB2]));
  const double mi = sc[CG_INFMAX] / a.scale_x;
  const double q = 4.0 * a.beta_next * eta * eta * tr * tr / red[1];
  const double dss = fmin(fmax(q, 0.0), a.beta0);
  const double primal_n = (1.0 - eta) * primal + eta * tr * sc[CG_VCV];
  const double trx_n = (1.0 - eta) * sc[CG_TRX] + eta * tr * sc[CG_VV];
  sc[CG_OBJGAP] = og;
  sc[CG_INFGAP] = ig;
  sc[CG_MAXINF] = mi;
  sc[CG_DSS] = dss;
  sc[CG_PRIMAL] = primal_n;
  sc[CG_TRX] = trx_n;
  if (a.trace && a.t < a.trace_capacity) {
    double* r = a.trace + (size_t)a.t * TR_NUM;
    r[0] = a.t; r[1] = sc[CG_EIG0]; r[2] = og; r[3] = ig; r[4] = mi; r[5] = primal_n;
    r[6] = trx_n; r[7] = dss;
  }
}

// y <- y + dss (z_next - proj_b), z <- z_next (solver/cgal.py:168-172)
__global__ void cgal_y_kernel(CgalArgs a) {
  const double dss = a.sc[CG_DSS];
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.m; c += gridDim.x * blockDim.x) {
    const double zn = a.zn[c], b = a.b[c], mk = a.mask[c], y = a.y[c];
    const double pbn = (1.0 - mk) * b + mk * fmin(zn + (1.0 / a.beta_next) * y, b);
    a.y[c] = y + dss * (zn - pbn);
    a.z[c] = zn;
  }
}

// P <- (1 - eta) P + eta tr v (v^T Omega)   (solver/cgal.py:155-158)
__global__ void cgal_sketch_kernel(int n, int ssk, const double* __restrict__ v,
                                   const double* __restrict__ vO, double* __restrict__ P, int ldp,
                                   double eta, double tr) {
  const long long total = (long long)n * ssk;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(e / n), i = (int)(e - (long long)c * n);
    const size_t o = (size_t)c * ldp + i;
    P[o] = (1.0 - eta) * P[o] + eta * tr * (v[i] * vO[c]);
  }
}

// X <- (1 - eta) X + eta tr v v^T   (row-major n x n, solver/cgal.py:153-154)
__global__ void cgal_dense_kernel(int n, const double* __restrict__ v, double* __restrict__ X,
                                  double eta, double tr) {
  const long long total = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / n), c = (int)(e - (long long)r * n);
    X[e] = (1.0 - eta) * X[e] + eta * tr * (v[r] * v[c]);
  }
}

struct CgalLayout {
  int n, m, ld, mL, vt, ssk, grid_red, grid_gram;
  double *sc, *adj, *zn, *Av, *v, *Cv, *mpart, *gpart, *alpha, *beta;
  void *opL, *Q, *q0L, *lz_work;
  unsigned int* counters;
  int *status, *ctl;
};

static void cgal_plan(const usbs_problem* P, const usbs_cgal_params* Pa, const DeviceInfo& di,
                      Arena& ar, CgalLayout& L) {
  L.n = P->n; L.m = P->m; L.ld = (L.n + 31) & ~31; L.mL = Pa->lanczos_inner_iterations;
  L.vt = (Pa->precision == 64) ? 8 : 4;
  L.ssk = (Pa->sketch_mode == 0) ? Pa->sketch_dim : 0;
  L.grid_red = di.sm_count * 2;
  L.grid_gram = di.sm_count * 2;
  L.sc = ar.take<double>(CG_NUM + 64);
  L.adj = ar.take<double>(L.m); L.zn = ar.take<double>(L.m); L.Av = ar.take<double>(L.m);
  L.v = ar.take<double>(L.ld); L.Cv = ar.take<double>(L.ld);
  L.mpart = ar.take<double>((size_t)L.grid_red * 8);
  L.gpart = ar.take<double>((size_t)L.grid_gram * 64);
  L.alpha = ar.take<double>(2 * MAXM);
  L.beta = L.alpha ? L.alpha + MAXM : nullptr;
  L.opL = ar.take<char>((size_t)(P->nnz > 0 ? P->nnz : 1) * L.vt);
  L.Q = ar.take<char>((size_t)L.ld * (L.mL + 1) * L.vt);
  L.q0L = ar.take<char>((size_t)L.ld * L.vt);
  L.counters = ar.take<unsigned int>(16);
  L.status = ar.take<int>(32);
  L.ctl = L.status + 16;
  const int nct = lanczos_team_size(di, L.n, Pa->precision);
  L.lz_work = ar.take<char>(lanczos_workspace_bytes(L.n, P->nnz, L.ld, L.mL, Pa->precision, nct));
}

}  // namespace usbs

using namespace usbs;

extern "C" {

size_t usbs_solve_workspace_bytes(const usbs_problem* P, const usbs_params* Pa) {
  DeviceInfo di;
  if (get_device_info(&di)) {
    di.sm_count = 152;
    di.lanczos_occ64 = di.lanczos_occ32 = 4;
    di.stream_occ64 = di.stream_occ32 = 8;
  }
  Arena ar{nullptr, 0, 0};
  Layout L;
  plan(P, Pa, di, ar, L);
  return ar.off + 4096;
}

int usbs_solve(const usbs_problem* P, const usbs_params* Pa, usbs_state* S, void* workspace,
               size_t workspace_bytes, usbs_cond_callback cb, void* cb_user, void* stream) {
  if (!P || !Pa || !S) { set_error("usbs_solve: null argument"); return -2; }
  const int k = Pa->k_curr + Pa->k_past;
  if (Pa->k_curr < 1 || Pa->k_past < 0 || k > IPM_MAXK) {
    set_error("usbs_solve: k_curr + k_past = %d must be in [1, %d]", k, IPM_MAXK);
    return -2;
  }
  if (Pa->lanczos_inner_iterations < Pa->k_curr || Pa->lanczos_inner_iterations > MAXM ||
      Pa->lanczos_inner_iterations < k) {
    set_error("usbs_solve: lanczos_inner_iterations must be in [k, %d]", MAXM);
    return -2;
  }
  if (Pa->precision != 64 && Pa->precision != 32) { set_error("precision must be 32 or 64"); return -2; }
  if (Pa->lanczos_path != 0 && Pa->lanczos_path != 2) {
    set_error("usbs_solve: lanczos_path must be 0 or 2");
    return -2;
  }
  if (Pa->lanczos_rows_per_cta != 0 && Pa->lanczos_rows_per_cta < 16) {
    set_error("usbs_solve: lanczos_rows_per_cta must be 0 or >= 16");
    return -2;
  }
  if (Pa->sketch_mode == 0 && (Pa->sketch_dim < 1 || Pa->sketch_dim > 64 || !S->Omega || !S->P)) {
    set_error("usbs_solve: sketch mode needs 1 <= sketch_dim <= 64, P and Omega");
    return -2;
  }
  if (Pa->sketch_mode == 1 && (!S->X || P->n > 46340)) { set_error("usbs_solve: dense-X mode needs X and n <= 46340"); return -2; }
  if (Pa->sketch_mode == 2 && !S->P) { set_error("usbs_solve: diagonal mode needs P"); return -2; }
  if (S->ld != ((P->n + 31) & ~31)) { set_error("usbs_solve: state ld must be n rounded up to 32"); return -2; }
  if (Pa->cond_exp_base < 1.0 || Pa->cond_exp_base > 2.0) { set_error("cond_exp_base must be in [1, 2]"); return -2; }
  Solver X;
  X.P = P; X.Pa = Pa; X.S = S; X.st = (cudaStream_t)stream;
  CK(get_device_info(&X.di));
  Arena ar{(char*)workspace, 0, workspace_bytes};
  plan(P, Pa, X.di, ar, X.L);
  if (!workspace || ar.off + 1024 > workspace_bytes) {
    set_error("usbs_solve: workspace of %zu bytes given, %zu needed", workspace_bytes, ar.off + 4096);
    return -2;
  }
  Layout& L = X.L;
  cudaStream_t st = X.st;
  X.lanes = lanczos_lanes(L.n, P->nnz);
  X.ctr_gram = L.counters;
  X.ctr_gram2 = L.counters + 8;
  X.ctr_m = L.counters + 16;
  if (cudaStreamCreateWithFlags(&X.st2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&X.ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&X.ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&X.ev_l0) != cudaSuccess || cudaEventCreate(&X.ev_l1) != cudaSuccess)
    return kerr("stream/event create");
  S->lanczos_launches = 0;
  S->lanczos_ms = 0.0;
  S->lanczos_bytes = 0.0;
  struct Cleanup {
    Solver* x;
    ~Cleanup() {
      if (x->st2) cudaStreamDestroy(x->st2);
      if (x->ev_fork) cudaEventDestroy(x->ev_fork);
      if (x->ev_join) cudaEventDestroy(x->ev_join);
      if (x->ev_l0) cudaEventDestroy(x->ev_l0);
      if (x->ev_l1) cudaEventDestroy(x->ev_l1);
      if (x->gexec) cudaGraphExecDestroy(x->gexec);
      if (x->gst) cudaStreamDestroy(x->gst);
    }
  } cleanup{&X};
  S->graph_iterations = 0;
  X.use_graph = graph_wanted(X);
  cudaMemsetAsync(L.counters, 0, 64 * sizeof(unsigned int), st);
  cudaMemsetAsync(L.status, 0, 32 * sizeof(int), st);
  cudaMemsetAsync(L.smalls, 0, (size_t)L.n_smalls * sizeof(double), st);
  cudaMemsetAsync(L.ups, 0, (size_t)L.m * sizeof(double), st);
  cudaMemcpyAsync(L.zbar, S->z, (size_t)L.m * sizeof(double), cudaMemcpyDeviceToDevice, st);
  if (Pa->sketch_mode == 0)
    cudaMemcpyAsync(L.Pbar, S->P, (size_t)L.ld * L.ssk * sizeof(double), cudaMemcpyDeviceToDevice, st);
  if (Pa->sketch_mode == 2)
    cudaMemcpyAsync(L.Pbar, S->P, (size_t)L.n * sizeof(double), cudaMemcpyDeviceToDevice, st);
  if (Pa->sketch_mode == 1)
    cudaMemcpyAsync(L.Xbar, S->X, (size_t)L.n * L.n * sizeof(double), cudaMemcpyDeviceToDevice, st);
  // Lanczos start vector in the Lanczos precision
  if (Pa->precision == 64)
    cudaMemcpyAsync(L.q0L, S->q0, (size_t)L.n * sizeof(double), cudaMemcpyDeviceToDevice, st);
  else
    to_vt_kernel<float><<<X.rgrid(), 256, 0, st>>>(L.n, S->q0, (float*)L.q0L);
  CK(kerr("init"));
  // ---- initial bundle: k smallest eigenvectors at y (solver/usbs.py:691-706) ----
  CK(X.lanczos(S->y, k));
  CK(X.copy_q_cols(k, S->V));
  if (Pa->precision != 64) {
    // orthonormalise the FP32 Ritz vectors in FP64 (shifted CholQR3)
    for (int pass = 0; pass < 3; ++pass) {
      CK(X.gram(S->V, L.ld, k, S->V, L.ld, k, L.n, L.smalls + L.o_G));
      CholQRArgs ca;
      ca.k = k; ca.n = L.n; ca.shifted = (pass == 0); ca.smalls = L.smalls; ca.o_G = L.o_G;
      ca.o_Rinv = L.o_Rinv; ca.status = L.status; ca.skip = nullptr;
      CK(launch_cholqr(ca, st));
      rows_rinv_kernel<<<X.rgrid(), 256, 0, st>>>(L.n, k, S->V, L.ld, L.smalls + L.o_Rinv, nullptr);
      CK(kerr("rinv"));
    }
  }
  // one pass over V for the constraints and the row updates when every
  // constraint is a single diagonal entry (USBS_FUSED_ROWS=0 keeps two passes)
  int diag_flag = 1;
  {
    const char* e = getenv("USBS_FUSED_ROWS");
    if (!P->has_ineq && L.m == L.n && !(e && atoi(e) == 0)) {
      cudaMemsetAsync(L.row_con, 0xff, (size_t)L.n * sizeof(int), st);
      cudaMemsetAsync(L.row_con + L.n, 0, sizeof(int), st);
      diag_map_kernel<<<X.mgrid(), 256, 0, st>>>(L.n, L.m, P->con_ptr, P->t_row, P->t_col,
                                                 L.row_con);
      CK(kerr("diag map"));
      if (cudaMemcpyAsync(&diag_flag, L.row_con + L.n, sizeof(int), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess)
        return kerr("diag map read");
    }
  }
  double alpha0 = 0.0;
  if (cudaMemcpyAsync(&alpha0, L.alpha, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return kerr("init eig");
  L.diag = (diag_flag == 0);
  double by0 = 0.0;
  {
    MvecArgs ma = X.margs();
    mvec_pre_kernel<<<X.mgrid(), RED_BLOCK, 0, st>>>(ma, Pa->trace_ub, k, 1);
    CK(kerr("mvec_pre"));
    CK(X.read_scalars(&by0, SC_BY, 1));
  }
  const double init_pen = by0 + Pa->trace_ub * std::fmax(-alpha0, 0.0);
  {
    double sc[SC_NUM];
    CK(X.read_scalars(sc, 0, SC_NUM));
    sc[SC_TRX] = S->tr_X; sc[SC_TRXBAR] = S->tr_X; sc[SC_PRIMAL] = S->primal_obj;
    sc[SC_BPO] = S->primal_obj; sc[SC_PEN] = init_pen; sc[SC_CANDPEN] = init_pen;
    sc[SC_LBEST] = 0.0; sc[SC_OBJUB] = INFINITY;
    sc[SC_OBJGAP] = 1.1 * Pa->obj_gap_eps; sc[SC_INFGAP] = 1.1 * Pa->infeas_gap_eps;
    sc[SC_MAXINF] = 1.1 * Pa->max_infeas_eps; sc[SC_T] = 0;
    if (cudaMemcpyAsync(L.smalls + L.o_sc, sc, sizeof(sc), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return kerr("init scalars");
  }
  // ---- outer loop (utils/loop.py:80-115 semantics, cond = solver/usbs.py:502-540) ----
  const auto t0 = std::chrono::steady_clock::now();
  auto elapsed = [&]() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  };
  double curr_time = 0.0;
  bool nonfinite = false;
  auto cond = [&](int t, bool* go) -> int {
    double sc[SC_NUM];
    CK(X.read_scalars(sc, 0, SC_NUM));
    double* r = S->cond;
    for (int f = 0; f < TR_NUM; ++f) r[f] = 0.0;
    r[TR_T] = t; r[TR_PRIMAL] = sc[SC_PRIMAL]; r[TR_OBJUB] = sc[SC_OBJUB];
    r[TR_OBJGAP] = sc[SC_OBJGAP]; r[TR_INFGAP] = sc[SC_INFGAP]; r[TR_MAXINF] = sc[SC_MAXINF];
    r[TR_PEN] = sc[SC_PEN]; r[TR_CANDPEN] = sc[SC_CANDPEN]; r[TR_LB] = sc[SC_LBEST];
    r[TR_LAM0] = sc[SC_LAM0]; r[TR_DESCENT] = t > 0 ? sc[SC_DESCENT] : 0.0;
    r[TR_ETA] = sc[SC_ETA]; r[TR_TRS] = sc[SC_TRS]; r[TR_TRX] = sc[SC_TRX];
    r[TR_QITERS] = sc[SC_QITERS]; r[TR_LITERS] = sc[SC_LITERS]; r[TR_BPO] = sc[SC_BPO];
    r[TR_TRXBAR] = sc[SC_TRXBAR];
    // b . y of the current y: y_cand after a descent step (the post kernel's rule)
    r[TR_BY] = (t > 0 && sc[SC_DESCENT] != 0.0) ? sc[SC_BYC] : sc[SC_BY];
    if (cb) cb(cb_user, t);
    // a NaN gap stops the loop as the reference's comparisons do (every one
    // is false); the status word says why
    if (t > 0 && !(std::isfinite(sc[SC_OBJGAP]) && std::isfinite(sc[SC_INFGAP]) &&
                   std::isfinite(sc[SC_MAXINF]) && std::isfinite(sc[SC_PRIMAL])))
      nonfinite = true;
    *go = (t == 0) || ((curr_time < Pa->max_time) &&
                       (sc[SC_OBJGAP] > Pa->obj_gap_eps || sc[SC_INFGAP] > Pa->infeas_gap_eps ||
                        sc[SC_MAXINF] > Pa->max_infeas_eps));
    return 0;
  };
  const std::vector<long long> sched = cond_schedule(Pa->max_iters, Pa->cond_exp_base);
  int t = 0;
  bool go = true;
  CK(cond(0, &go));
  for (size_t b = 0; b < sched.size() && go; ++b) {
    for (long long j = 0; j < sched[b]; ++j) {
      if (j > 0 && !X.use_graph) {   // eager: sync to collect the previous Lanczos timing
        if (cudaStreamSynchronize(st) != cudaSuccess) return kerr("iteration");
        CK(X.collect_lanczos());
      }
      CK(step(X, t));
      ++t;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return kerr("iteration");
    CK(X.collect_lanczos());
    curr_time = elapsed();
    CK(cond(t, &go));
  }
  // ---- outputs ----
  double sc[SC_NUM];
  CK(X.read_scalars(sc, 0, SC_NUM));
  int status[8];
  if (cudaMemcpy(status, L.status, sizeof(status), cudaMemcpyDeviceToHost) != cudaSuccess)
    return kerr("status");
  S->iterations = t;
  S->tr_X = sc[SC_TRX];
  S->primal_obj = sc[SC_PRIMAL];
  S->obj_gap = sc[SC_OBJGAP];
  S->infeas_gap = sc[SC_INFGAP];
  S->max_infeas = sc[SC_MAXINF];
  S->obj_ub = sc[SC_OBJUB];
  S->pen_dual_obj = sc[SC_PEN];
  S->status = status[0] | (nonfinite ? ST_NONFINITE : 0);
  S->elapsed = elapsed();
  S->kernel_launches = X.launches;
  return 0;
}

size_t usbs_cgal_workspace_bytes(const usbs_problem* P, const usbs_cgal_params* Pa) {
  DeviceInfo di;
  if (get_device_info(&di)) {
    di.sm_count = 152;
    di.lanczos_occ64 = di.lanczos_occ32 = 4;
    di.stream_occ64 = di.stream_occ32 = 8;
  }
  Arena ar{nullptr, 0, 0};
  CgalLayout L;
  cgal_plan(P, Pa, di, ar, L);
  return ar.off + 4096;
}

int usbs_cgal_solve(const usbs_problem* P, const usbs_cgal_params* Pa, usbs_state* S,
                    void* workspace, size_t workspace_bytes, usbs_cond_callback cb, void* cb_user,
                    void* stream) {
  if (!P || !Pa || !S) { set_error("usbs_cgal_solve: null argument"); return -2; }
  if (Pa->lanczos_inner_iterations < 1 || Pa->lanczos_inner_iterations > MAXM) {
    set_error("usbs_cgal_solve: lanczos_inner_iterations must be in [1, %d]", MAXM);
    return -2;
  }
  if (Pa->precision != 64 && Pa->precision != 32) { set_error("precision must be 32 or 64"); return -2; }
  if (Pa->sketch_mode == 0 && (Pa->sketch_dim < 1 || Pa->sketch_dim > 64 || !S->Omega || !S->P)) {
    set_error("usbs_cgal_solve: sketch mode needs 1 <= sketch_dim <= 64, P and Omega");
    return -2;
  }
  if (Pa->sketch_mode == 1 && (!S->X || P->n > 46340)) {
    set_error("usbs_cgal_solve: dense-X mode needs X and n <= 46340");
    return -2;
  }
  if (Pa->sketch_mode != 0 && Pa->sketch_mode != 1) { set_error("usbs_cgal_solve: sketch_mode must be 0 or 1"); return -2; }
  if (S->ld != ((P->n + 31) & ~31)) { set_error("usbs_cgal_solve: state ld must be n rounded up to 32"); return -2; }
  if (Pa->cond_exp_base < 1.0 || Pa->cond_exp_base > 2.0) { set_error("cond_exp_base must be in [1, 2]"); return -2; }
  DeviceInfo di;
  CK(get_device_info(&di));
  Arena ar{(char*)workspace, 0, workspace_bytes};
  CgalLayout L;
  cgal_plan(P, Pa, di, ar, L);
  if (!workspace || ar.off + 1024 > workspace_bytes) {
    set_error("usbs_cgal_solve: workspace of %zu bytes given, %zu needed", workspace_bytes, ar.off + 4096);
    return -2;
  }
  cudaStream_t st = (cudaStream_t)stream;
  long long launches = 0;
  const int lanes = lanczos_lanes(L.n, P->nnz);
  auto rgrid = [&](long long work) {
    long long b = (work + 255) / 256;
    if (b > (long long)di.sm_count * 8) b = (long long)di.sm_count * 8;
    return (int)(b < 1 ? 1 : b);
  };
  int mgrid = (L.m + RED_BLOCK - 1) / RED_BLOCK;
  if (mgrid > L.grid_red) mgrid = L.grid_red;
  if (mgrid < 1) mgrid = 1;
  auto gram1 = [&](const double* Y, int ky, double* out) -> int {
    GramArgs g;
    g.n = L.n; g.kx = 1; g.ky = ky; g.ldx = L.ld; g.ldy = L.ld; g.X = L.v; g.Y = Y;
    g.partial = L.gpart; g.counter = L.counters + 8; g.out = out; g.skip = nullptr;
    int blocks = (L.n + GR_ROWS - 1) / GR_ROWS;
    if (blocks > L.grid_gram) blocks = L.grid_gram;
    if (blocks < 1) blocks = 1;
    ++launches;
    gram_kernel<1><<<blocks, RED_BLOCK, 0, st>>>(g);
    return kerr("cgal gram");
  };
  cudaMemsetAsync(L.counters, 0, 16 * sizeof(unsigned int), st);
  cudaMemsetAsync(L.status, 0, 32 * sizeof(int), st);
  cudaMemsetAsync(L.sc, 0, (CG_NUM + 64) * sizeof(double), st);
  if (Pa->precision == 64)
    cudaMemcpyAsync(L.q0L, S->q0, (size_t)L.n * sizeof(double), cudaMemcpyDeviceToDevice, st);
  else
    to_vt_kernel<float><<<rgrid(L.n), 256, 0, st>>>(L.n, S->q0, (float*)L.q0L);
  {
    double init[2] = {S->primal_obj, S->tr_X};
    double g3[3] = {1.1 * Pa->obj_gap_eps, 1.1 * Pa->infeas_gap_eps, 1.1 * Pa->max_infeas_eps};
    if (cudaMemcpyAsync(L.sc + CG_PRIMAL, init, sizeof(init), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(L.sc + CG_OBJGAP, g3, sizeof(g3), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return kerr("cgal init");
  }
  CK(kerr("cgal init"));
  CgalArgs a;
  a.m = L.m; a.sc = L.sc; a.y = S->y; a.z = S->z; a.adj = L.adj; a.zn = L.zn; a.Av = L.Av;
  a.b = P->b; a.mask = P->b_ineq_mask; a.scale_a = P->scale_a; a.scale_c = P->scale_c;
  a.scale_x = P->scale_x; a.trace_ub = Pa->trace_ub; a.beta0 = Pa->beta0;
  a.partial = L.mpart; a.counter = L.counters; a.trace = S->trace;
  a.trace_capacity = S->trace ? S->trace_capacity : 0;
  auto body = [&](int t) -> int {
    a.t = t;
    a.beta = Pa->beta0 * std::sqrt((double)t + 1.0);
    a.beta_next = Pa->beta0 * std::sqrt((double)t + 2.0);
    a.eta = 2.0 / ((double)t + 2.0);
    ++launches;
    cgal_pre_kernel<<<mgrid, RED_BLOCK, 0, st>>>(a);
    CK(kerr("cgal pre"));
    // eigsh(1) of -C + A*(adj) (solver/cgal.py:108-112)
    ++launches;
    CK(assemble_operator((int)P->nnz, P->c_val, -1.0, P->slot_ptr, P->slot_tid, P->t_con, P->t_a0,
                         L.adj, L.opL, Pa->precision, st));
    if (cudaMemcpyAsync(L.Q, L.q0L, (size_t)L.n * L.vt, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return kerr("cgal q0");
    LanczosProblem lp;
    lp.n = L.n; lp.ld = L.ld; lp.m = L.mL; lp.num_desired = 1;
    lp.max_restarts = Pa->lanczos_max_restarts; lp.nnz = P->nnz; lp.tol = Pa->subprob_eps;
    lp.rowptr = P->rowptr; lp.col = P->col; lp.val = L.opL; lp.Q = L.Q;
    lp.alpha = L.alpha; lp.beta = L.beta; lp.ctl = L.ctl; lp.status = L.status; lp.work = L.lz_work;
    CK(lanczos_run(di, &lp, 1, Pa->precision, st));
    launches += lanczos_last_launches();
    ++launches;
    if (Pa->precision == 64)
      cgal_v_kernel<double><<<rgrid(L.n), 256, 0, st>>>(L.n, (const double*)L.Q, L.alpha, L.v, L.sc);
    else
      cgal_v_kernel<float><<<rgrid(L.n), 256, 0, st>>>(L.n, (const float*)L.Q, L.alpha, L.v, L.sc);
    CK(kerr("cgal v"));
    // C v and A(v v^T)
    ++launches;
    spmm_kernel<<<rgrid((long long)L.n * lanes), 256, 0, st>>>(L.n, P->rowptr, P->col, P->c_val, L.v,
                                                             L.ld, 1, L.Cv, L.ld, lanes, nullptr);
    CK(kerr("cgal Cv"));
    ++launches;
    CK(apply_A_operator(L.m, P->con_ptr, P->t_row, P->t_col, P->t_a, L.v, L.ld, 1, L.Av, st));
    CK(gram1(L.Cv, 1, L.sc + CG_VCV));
    CK(gram1(L.v, 1, L.sc + CG_VV));
    if (Pa->sketch_mode == 0) CK(gram1(S->Omega, L.ssk, L.sc + CG_NUM));
    ++launches;
    cgal_post_kernel<<<mgrid, RED_BLOCK, 0, st>>>(a);
    CK(kerr("cgal post"));
    ++launches;
    cgal_y_kernel<<<mgrid, RED_BLOCK, 0, st>>>(a);
    CK(kerr("cgal y"));
    ++launches;
    if (Pa->sketch_mode == 0)
      cgal_sketch_kernel<<<rgrid((long long)L.n * L.ssk), 256, 0, st>>>(L.n, L.ssk, L.v, L.sc + CG_NUM,
                                                                       S->P, S->ld, a.eta, Pa->trace_ub);
    else
      cgal_dense_kernel<<<rgrid((long long)L.n * L.n), 256, 0, st>>>(L.n, L.v, S->X, a.eta, Pa->trace_ub);
    return kerr("cgal update");
  };
  // loop with the reference's condition schedule (utils/loop.py:80-115,
  // cond = solver/cgal.py:76-97)
  const auto t0 = std::chrono::steady_clock::now();
  auto elapsed = [&]() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  };
  double curr_time = 0.0;
  auto read = [&](double* out, int first, int count) -> int {
    if (cudaMemcpyAsync(out, L.sc + first, count * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return kerr("cgal read");
    return 0;
  };
  auto cond = [&](int t, bool* go) -> int {
    double sc[CG_NUM];
    CK(read(sc, 0, CG_NUM));
    const double* g = sc + CG_OBJGAP;
    double* r = S->cond;
    for (int f = 0; f < TR_NUM; ++f) r[f] = 0.0;
    r[0] = t; r[1] = sc[CG_EIG0]; r[2] = sc[CG_OBJGAP]; r[3] = sc[CG_INFGAP];
    r[4] = sc[CG_MAXINF]; r[5] = sc[CG_PRIMAL]; r[6] = sc[CG_TRX]; r[7] = sc[CG_DSS];
    if (cb) cb(cb_user, t);
    *go = (t == 0) || ((curr_time < Pa->max_time) &&
                       (g[0] > Pa->obj_gap_eps || g[1] > Pa->infeas_gap_eps || g[2] > Pa->max_infeas_eps));
    return 0;
  };
  const std::vector<long long> sched = cond_schedule(Pa->max_iters, Pa->cond_exp_base);
  int t = 0;
  bool go = true;
  CK(cond(0, &go));
  for (size_t bk = 0; bk < sched.size() && go; ++bk) {
    for (long long j = 0; j < sched[bk]; ++j) {
      CK(body(t));
      ++t;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return kerr("cgal iteration");
    curr_time = elapsed();
    CK(cond(t, &go));
  }
  double sc[CG_NUM];
  CK(read(sc, 0, CG_NUM));
  int status[8];
  if (cudaMemcpy(status, L.status, sizeof(status), cudaMemcpyDeviceToHost) != cudaSuccess)
    return kerr("cgal status");
  S->iterations = t;
  S->tr_X = sc[CG_TRX];
  S->primal_obj = sc[CG_PRIMAL];
  S->obj_gap = sc[CG_OBJGAP];
  S->infeas_gap = sc[CG_INFGAP];
  S->max_infeas = sc[CG_MAXINF];
  S->status = status[0];
  S->elapsed = elapsed();
  S->kernel_launches = launches;
  return 0;
}

}  // extern "C"
