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

// 0.5 * [U (T (x) X + X (x) T) U^T]_{a, a2}
__device__ __forceinline__ double symkron(const double* T, const double* X, int k, int b, int c,
                                          int b2, int c2) {
  const int na = (b == c) ? 1 : 2, nb = (b2 == c2) ? 1 : 2;
  const double wa = (b == c) ? 1.0 : RSQ2, wb = (b2 == c2) ? 1.0 : RSQ2;
  double acc = 0.0;
  for (int u = 0; u < na; ++u) {
    const int i = u ? c : b, j = u ? b : c;
    for (int v = 0; v < nb; ++v) {
      const int i2 = v ? c2 : b2, j2 = v ? b2 : c2;
      acc += T[i * k + i2] * X[j * k + j2] + X[i * k + i2] * T[j * k + j2];
    }
  }
  return 0.5 * wa * wb * acc;
}

// Cholesky positive-definiteness test of A + s dA (k x k, lower triangle)
__device__ bool pd_test(const double* A, const double* dA, double s, int k) {
  double L[IPM_MAXS];
  for (int j = 0; j < k; ++j) {
    double d = A[j * k + j] + s * dA[j * k + j];
    for (int p = 0; p < j; ++p) d -= L[j * (j + 1) / 2 + p] * L[j * (j + 1) / 2 + p];
    if (!(d > 0.0)) return false;
    const double ljj = sqrt(d);
    L[j * (j + 1) / 2 + j] = ljj;
    for (int i = j + 1; i < k; ++i) {
      double v = A[i * k + j] + s * dA[i * k + j];
      for (int p = 0; p < j; ++p) v -= L[i * (i + 1) / 2 + p] * L[j * (j + 1) / 2 + p];
      L[i * (i + 1) / 2 + j] = v / ljj;
    }
  }
  return true;
}

__global__ void __launch_bounds__(IPM_BLOCK) ipm_kernel(const __grid_constant__ IpmArgs A) {
  extern __shared__ double dyn[];
  __shared__ IpmShared sh;
  __shared__ double s_red[IPM_BLOCK / 32];
  if (A.skip && *A.skip) return;
  const int k = A.k, s = k * (k + 1) / 2, tid = threadIdx.x;
  double* Q11 = dyn;            // s*s (mode 0)
  double* coeff = dyn + s * s;  // s*s
  double* sm = A.smalls;
  // svec index maps (np.tril_indices order)
  if (tid == 0) {
    int a = 0;
    for (int b = 0; b < k; ++b)
      for (int c = 0; c <= b; ++c) { sh.bi[a] = b; sh.ci[a] = c; ++a; }
  }
  __syncthreads();
  const double tr = A.trace_ub;
  const double tXb_raw = sm[A.o_sc + SC_TRXBAR];
  const double tX = (tXb_raw > 0.0) ? tXb_raw : tr;
  const double bpo = sm[A.o_sc + SC_BPO];
  double q22 = 0.0, h2 = 0.0;
  for (int a = tid; a < s; a += IPM_BLOCK) sh.sI[a] = (sh.bi[a] == sh.ci[a]) ? 1.0 : 0.0;
  if (A.mode == 0) {
    const double rho = A.rho;
    const double* QB = sm + A.o_QB;
    for (int e = tid; e < s * s; e += IPM_BLOCK) Q11[e] = (tr * tr / rho) * QB[e];
    const double* GZ = sm + A.o_GZ;
    const double* GYmC = sm + A.o_GYmC;
    const double* GB = sm + A.o_GB;
    for (int a = tid; a < s; a += IPM_BLOCK) {
      const int b = sh.bi[a], c = sh.ci[a];
      sh.q12[a] = (tr * tr / (rho * tX)) * svec_of(GZ, k, b, c);
      // svec(V^T (A*(y) - C - A*(b - ups)/rho) V)
      double gy = svec_of(GYmC, k, b, c);
      double gb = svec_of(GB, k, b, c);
      sh.h1[a] = tr * (gy - gb / rho);
    }
    q22 = (tr * tr / (rho * tX * tX)) * sm[A.o_sc + SC_ZZ];
    h2 = (tr / tX) * (sm[A.o_sc + SC_ZY] - bpo - sm[A.o_sc + SC_ZBMU] / rho);
  } else {
    const double* GYC = sm + A.o_GYC;  // V^T (A*(y_cand) - C) V
    for (int a = tid; a < s; a += IPM_BLOCK) {
      sh.h1[a] = tr * svec_of(GYC, k, sh.bi[a], sh.ci[a]);   // g_1
      sh.q12[a] = 0.0;
    }
    h2 = (tr / tX) * (sm[A.o_sc + SC_ZYC] - bpo);           // g_2
  }
  __syncthreads();
  // ---- initial point ----
  double eta;
  if (A.mode == 0) {
    eta = (tX / tr) * sm[A.o_sc + SC_ETA_SUB];
    const double* S0 = sm + A.o_Ssub;
    for (int e = tid; e < k * k; e += IPM_BLOCK) sh.S[e] = S0[e] / tr;
  } else {
    eta = (bpo == 0.0) ? 0.00001 : 0.99 * (1.0 / (k + 1.0));
    for (int e = tid; e < k * k; e += IPM_BLOCK) {
      const int r = e / k, c = e - r * k;
      sh.S[e] = (r == c) ? 0.99 * (1.0 / (k + 1.0)) : 0.0;
    }
  }
  __syncthreads();
  for (int a = tid; a < s; a += IPM_BLOCK) sh.sS[a] = svec_of(sh.S, k, sh.bi[a], sh.ci[a]);
  __syncthreads();
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
  __syncthreads();
  double zeta = (A.mode == 0) ? (dot_s(sh.q12, sh.sS, s) + eta * q22 + h2) : h2;
  svec_inv_to(sh.ord, k, s, sh.bi, sh.ci, sh.T);
  __syncthreads();
  double vmax = zeta, vmin = zeta;
  for (int b = 0; b < k; ++b) { vmax = fmax(vmax, sh.T[b * k + b]); vmin = fmin(vmin, sh.T[b * k + b]); }
  double width = vmax - vmin;
  width = (width < 100.0) ? 100.0 : width;
  double omega = -1.01 * vmin;
  omega = (omega < width) ? width : omega;
  __syncthreads();
  if (tid < k) sh.T[tid * k + tid] += omega;
  zeta += omega;
  __syncthreads();
  for (int a = tid; a < s; a += IPM_BLOCK) sh.sT[a] = svec_of(sh.T, k, sh.bi[a], sh.ci[a]);
  __syncthreads();
  double trS = 0.0;
  for (int b = 0; b < k; ++b) trS += sh.S[b * k + b];
  double mu = (dot_s(sh.sS, sh.sT, s) + eta * zeta + omega * (1 - trS - eta)) / (2 * k + 4.0);
  double step = 1.0;
  int it = 0;
  const int maxit = A.max_iters;
  const double eps = A.eps;
  while (it < maxit) {
    const bool cont = (A.mode == 0) ? (mu > eps && step > eps * eps) : (mu > eps);
    if (!cont) break;
    // ---- Newton system ----
    const double tIS = trS;
    const double k1 = (1 - tIS - eta) / omega;
    const double k2 = zeta / eta + q22;
    double F2 = 0.0;
    if (A.mode == 0) {
      for (int a = tid; a < s; a += IPM_BLOCK) {
        double v = 0.0;
        for (int b = 0; b < s; ++b) v += Q11[a * s + b] * sh.sS[b];
        double f = v + eta * sh.q12[a] + sh.h1[a];
        sh.F1[a] = f + (-sh.sT[a] + omega * sh.sI[a]);
      }
      F2 = dot_s(sh.q12, sh.sS, s) + eta * q22 + h2;
      F2 = F2 + (-zeta + omega);
    }
    // S^-1 by warp 0
    if (tid < 32) {
      for (int e = tid; e < k * k; e += 32) sh.wk[e] = sh.S[e];
      __syncwarp();
      bool ok = warp_inverse(sh.wk, k, k, sh.Si, k);
      if (!ok && tid == 0) atomicOr(A.status, ST_SMALL_DENSE_FAIL);
    }
    __syncthreads();
    for (int a = tid; a < s; a += IPM_BLOCK) sh.sSi[a] = svec_of(sh.Si, k, sh.bi[a], sh.ci[a]);
    const double den = k1 * k2 + 1;
    const double ze = zeta / eta;
    for (int e = tid; e < s * s; e += IPM_BLOCK) {
      const int a = e / s, a2 = e - a * s;
      double v = symkron(sh.T, sh.Si, k, sh.bi[a], sh.ci[a], sh.bi[a2], sh.ci[a2]);
      if (A.mode == 0) {
        v = Q11[e] + v;
        v -= (sh.q12[a] * (k1 * sh.q12[a2] + sh.sI[a2]) + sh.sI[a] * (sh.q12[a2] - k2 * sh.sI[a2])) / den;
      } else {
        v += (ze / (k1 * ze + 1)) * (sh.sI[a] * sh.sI[a2]);
      }
      coeff[e] = v;
    }
    __syncthreads();
    for (int a = tid; a < s; a += IPM_BLOCK) {
      double o;
      if (A.mode == 0) {
        o = -sh.F1[a] + mu * sh.sSi[a] - sh.sT[a];
        o += ((mu / omega + tIS + eta - 1 + k1 * (F2 - mu / eta + zeta)) / den) * sh.q12[a];
        o += ((F2 - mu / eta + zeta - k2 * (mu / omega + tIS + eta - 1)) / den) * sh.sI[a];
      } else {
        o = ze * (-k1 * (mu / eta - h2 - omega) + mu / omega + tIS + eta - 1) / (-k1 * ze - 1) * sh.sI[a];
        o += (h2 - mu / eta) * sh.sI[a] - sh.h1[a];
        o += mu * sh.sSi[a];
      }
      sh.ord[a] = o;
    }
    __syncthreads();
    if (!block_lu_solve(coeff, s, sh.ord, s, sh.redv, sh.redi)) {
      if (tid == 0) atomicOr(A.status, ST_SMALL_DENSE_FAIL);
    }
    // sh.ord now holds dsS
    double d_eta, d_omega, d_zeta;
    if (A.mode == 0) {
      double t1 = 0.0;
      for (int a = threadIdx.x & 31; a < s; a += 32) t1 += (k1 * sh.q12[a] + sh.sI[a]) * sh.ord[a];
      t1 = warp_sum(t1);
      d_eta = (-t1 - (mu / omega) - tIS - eta + 1 + k1 * (-F2 + mu / eta - zeta)) / den;
      double t2 = 0.0;
      for (int a = threadIdx.x & 31; a < s; a += 32) t2 += (sh.q12[a] - k2 * sh.sI[a]) * sh.ord[a];
      t2 = warp_sum(t2);
      d_omega = (-F2 + mu / eta - zeta + k2 * (mu / omega + tIS + eta - 1) - t2) / den;
      for (int a = tid; a < s; a += IPM_BLOCK) {
        double v = 0.0;
        for (int b = 0; b < s; ++b) v += Q11[a * s + b] * sh.ord[b];
        sh.dsT[a] = v + d_eta * sh.q12[a] + d_omega * sh.sI[a] + sh.F1[a];
      }
      d_zeta = dot_s(sh.q12, sh.ord, s) + d_eta * q22 + d_omega + F2;
    } else {
      const double tI = dot_s(sh.sI, sh.ord, s);
      d_eta = (tI - k1 * (mu / eta - h2 - omega) + mu / omega + tIS + eta - 1) / (-k1 * ze - 1);
      d_omega = -ze * d_eta + mu / eta;
      d_omega = d_omega + (-h2 - omega);
      for (int a = tid; a < s; a += IPM_BLOCK)
        sh.dsT[a] = d_omega * sh.sI[a] - sh.sT[a] + sh.h1[a] + omega * sh.sI[a];
      d_zeta = d_omega - zeta + h2 + omega;
    }
    __syncthreads();
    svec_inv_to(sh.ord, k, s, sh.bi, sh.ci, sh.dS);
    svec_inv_to(sh.dsT, k, s, sh.bi, sh.ci, sh.dT);
    __syncthreads();
    // ---- step size ----
    double r = nanmin2(nanmin2(d_eta / eta, d_zeta / zeta), d_omega / omega);
    double st = -1.0 / r;
    if (!isnan(st) && st > 1.0) st = 1.0;
    st = 0.99 * ((st <= 0.0) ? 1.0 : st);
    double cS = 0.0, cT = 0.0;
    for (int j = tid; j < A.ipm_grid; j += IPM_BLOCK) {
      const double a = pow(0.9, (double)j);
      if (pd_test(sh.S, sh.dS, a, k)) cS = fmax(cS, a);
      if (pd_test(sh.T, sh.dT, a, k)) cT = fmax(cT, a);
    }
    cS = block_max(cS, s_red);
    __syncthreads();
    cT = block_max(cT, s_red);
    const double cand = (cS < cT) ? cS : cT;
    st = (st < cand) ? st : cand;
    __syncthreads();
    // ---- update ----
    for (int e = tid; e < k * k; e += IPM_BLOCK) {
      sh.S[e] = sh.S[e] + st * sh.dS[e];
      sh.T[e] = sh.T[e] + st * sh.dT[e];
    }
    eta = eta + st * d_eta;
    zeta = zeta + st * d_zeta;
    omega = omega + st * d_omega;
    __syncthreads();
    for (int a = tid; a < s; a += IPM_BLOCK) {
      sh.sS[a] = svec_of(sh.S, k, sh.bi[a], sh.ci[a]);
      sh.sT[a] = svec_of(sh.T, k, sh.bi[a], sh.ci[a]);
    }
    __syncthreads();
    trS = 0.0;
    for (int b = 0; b < k; ++b) trS += sh.S[b * k + b];
    double mun = (dot_s(sh.sS, sh.sT, s) + eta * zeta + omega * (1 - trS - eta)) / (2 * k + 4.0);
    mun *= (st > 0.2) ? (0.5 - 0.4 * st * st) : 1.0;
    if (!(isnan(mun) || mun <= mu)) mun = mu;
    mu = mun;
    step = st;
    ++it;
    __syncthreads();
  }
  // ---- outputs ----
  if (A.mode == 0) {
    for (int e = tid; e < k * k; e += IPM_BLOCK) sm[A.o_Sout + e] = tr * sh.S[e];
    if (tid == 0) {
      sm[A.o_sc + SC_ETA] = (tr / tX) * eta;
      sm[A.o_sc + SC_QITERS] = it;
    }
  } else {
    const double g1S = dot_s(sh.h1, sh.sS, s);
    if (tid == 0) {
      sm[A.o_sc + SC_LB] = sm[A.o_sc + SC_BYC] - g1S - eta * h2;
      sm[A.o_sc + SC_LITERS] = it;
    }
  }
}

// eigh(S) and the quantities the outer iteration derives from it.  One warp.
__global__ void eigS_kernel(EigSArgs A) {
  if (A.skip && *A.skip) return;
  __shared__ double Sw[IPM_MAXK * (IPM_MAXK + 1)], Z[IPM_MAXK * (IPM_MAXK + 1)], lam[IPM_MAXK];
  __shared__ double GW[IPM_MAXK * IPM_MAXK];
  const int k = A.k, kc = A.k_curr, lane = threadIdx.x;
  double* sm = A.smalls;
  const double* S = sm + A.o_Sout;
  for (int e = lane; e < k * k; e += 32) Sw[(e / k) * (IPM_MAXK + 1) + e % k] = S[e];
  __syncwarp();
  bool ok = warp_syev(Sw, IPM_MAXK + 1, k, lam, Z, IPM_MAXK + 1);
  if (!ok && lane == 0) atomicOr(A.status, ST_SMALL_DENSE_FAIL);
  __syncwarp();
  if (lane < k) lam[lane] = fmax(lam[lane], 0.0);   // clip(eigvals, 0)
  __syncwarp();
  double* W = sm + A.o_W;
  double* Sp = sm + A.o_Splus;
  double* Scp = sm + A.o_Scplus;
  for (int e = lane; e < k * k; e += 32) {
    const int r = e / k, c = e - r * k;
    W[e] = Z[r * (IPM_MAXK + 1) + c];
    double a = 0.0, b = 0.0;
    for (int j = 0; j < k; ++j) {
      const double t = Z[r * (IPM_MAXK + 1) + j] * lam[j] * Z[c * (IPM_MAXK + 1) + j];
      a += t;
      if (j < kc) b += t;
    }
    Sp[e] = a;
    Scp[e] = b;
  }
  // trace(F^T C F) = sum_j lam_j (W^T G_C W)_jj
  const double* GC = sm + A.o_GC;
  for (int e = lane; e < k * k; e += 32) {
    const int r = e / k, j = e - r * k;
    double v = 0.0;
    for (int c = 0; c < k; ++c) v += GC[r * k + c] * Z[c * (IPM_MAXK + 1) + j];
    GW[e] = v;   // (G_C W)[r][j]
  }
  __syncwarp();
  double pj = 0.0;
  if (lane < k) {
    for (int r = 0; r < k; ++r) pj += Z[r * (IPM_MAXK + 1) + lane] * GW[r * k + lane];
    pj *= lam[lane];
  }
  double pall = warp_sum(pj);
  double pcur = warp_sum(lane < kc ? pj : 0.0);
  double lc = warp_sum(lane < kc ? lam[lane] : 0.0);
  if (lane == 0) {
    double trS = 0.0;
    for (int b = 0; b < k; ++b) trS += S[b * k + b];
    sm[A.o_sc + SC_TRS] = trS;
    sm[A.o_sc + SC_SUMLAMC] = lc;
    sm[A.o_sc + SC_PFULL] = pall;
    sm[A.o_sc + SC_PCUR] = pcur;
  }
  // W_past = W[:, kc:]
  const int kp = k - kc;
  for (int e = lane; e < k * kp; e += 32) {
    const int r = e / kp, c = e - r * kp;
    sm[A.o_Wpast + e] = Z[r * (IPM_MAXK + 1) + kc + c];
  }
  // M = S+ (V^T Omega), Mc = Sc+ (V^T Omega)    (k x ssk)
  if (A.ssk > 0) {
    const double* VtO = sm + A.o_VtO;
    __syncwarp();
    for (int e = lane; e < k * A.ssk; e += 32) {
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

// One pass of (shifted) Cholesky QR: R^T R = G (+ shift I), output R^-1 (upper).
__global__ void cholqr_kernel(CholQRArgs A) {
  if (A.skip && *A.skip) return;
  __shared__ double R[IPM_MAXK * IPM_MAXK], Ri[IPM_MAXK * IPM_MAXK];
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
  if (lane == 0) {
    bool ok = true;
    for (int j = 0; j < k; ++j) {
      double d = G[j * k + j] + shift;
      for (int p = 0; p < j; ++p) d -= R[p * k + j] * R[p * k + j];
      if (!(d > 0.0)) { ok = false; d = 1.0; }
      const double rjj = sqrt(d);
      R[j * k + j] = rjj;
      for (int i = j + 1; i < k; ++i) {
        double v = G[j * k + i];
        for (int p = 0; p < j; ++p) v -= R[p * k + j] * R[p * k + i];
        R[j * k + i] = v / rjj;
      }
      for (int i = 0; i < j; ++i) R[j * k + i] = 0.0;
    }
    // R^-1 (upper triangular) by back substitution, column by column
    for (int c = 0; c < k; ++c) {
      for (int r = k - 1; r >= 0; --r) {
        double v = (r == c) ? 1.0 : 0.0;
        for (int p = r + 1; p < k; ++p) v -= R[r * k + p] * Ri[p * k + c];
        Ri[r * k + c] = (r > c) ? 0.0 : v / R[r * k + r];
      }
    }
    if (!ok) atomicOr(A.status, ST_SMALL_DENSE_FAIL);
  }
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
  eigS_kernel<<<1, 32, 0, st>>>(a);
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
