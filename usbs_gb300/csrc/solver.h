// Structures shared by the USBS outer-iteration kernels (ipm.cu, usbs_solver.cu).
#pragma once
#include <cuda_runtime.h>

namespace usbs {

constexpr int IPM_MAXK = 12;                                // k = k_curr + k_past
constexpr int IPM_MAXS = IPM_MAXK * (IPM_MAXK + 1) / 2;     // svec dimension
constexpr int IPM_BLOCK = 256;

// Scalar slots of the per-instance "smalls" buffer (offset o_sc).
enum ScalarSlot {
  SC_ETA = 0,      // eta returned by the quadratic subproblem (unscaled)
  SC_QITERS,       // IPM iterations (quadratic subproblem)
  SC_LITERS,       // IPM iterations (lower bound)
  SC_LB,           // lb_spec_est
  SC_TRS,          // trace(S)
  SC_SUMLAMC,      // sum of the k_curr smallest clipped eigenvalues of S
  SC_PFULL,        // trace(F^T C F)
  SC_PCUR,         // trace(F_c^T C F_c)
  SC_ZZ,           // z_bar . z_bar
  SC_ZY,           // z_bar . y
  SC_ZBMU,         // z_bar . (b - upsilon)
  SC_BY,           // b . y
  SC_BYC,          // b . y_cand
  SC_ZYC,          // z_bar(old) . y_cand
  SC_INFSQ,        // sum (infeas / SCALE_A)^2
  SC_INFMAX,       // max |infeas| / SCALE_A
  SC_LAM0,         // largest eigenvalue of C - A*(y_cand)  (= -alpha_0)
  SC_TRX,          // state: tr_X
  SC_TRXBAR,       // state: tr_X_bar
  SC_PRIMAL,       // state: primal_obj
  SC_BPO,          // state: bar_primal_obj
  SC_PEN,          // state: pen_dual_obj
  SC_CANDPEN,      // state: cand_pen_dual_obj
  SC_LBEST,        // state: lb_spec_est
  SC_OBJUB,        // state: obj_ub
  SC_OBJGAP,       // state: obj_gap
  SC_INFGAP,       // state: infeas_gap
  SC_MAXINF,       // state: max_infeas
  SC_ETA_SUB,      // alternating-minimisation warm start eta
  SC_UPSGAP,       // upsilon_gap
  SC_DESCENT,      // 1 if the last step was a descent (serious) step
  SC_T,            // iteration counter
  SC_NUM
};

// Per-iteration trace record (doubles), written by the post kernel.
enum TraceField {
  TR_T = 0, TR_PRIMAL, TR_OBJUB, TR_OBJGAP, TR_INFGAP, TR_MAXINF, TR_PEN, TR_CANDPEN, TR_LB,
  TR_LAM0, TR_DESCENT, TR_ETA, TR_TRS, TR_TRX, TR_QITERS, TR_LITERS, TR_BPO, TR_TRXBAR,
  TR_BY,           // b . y after the iteration (the reference's printed dual_obj)
  TR_NUM = 20
};

struct IpmArgs {
  int mode;            // 0 quadratic subproblem, 1 lower bound
  int k, max_iters, ipm_grid;
  double eps, trace_ub, rho;
  double* smalls;
  int o_sc, o_QB, o_GZ, o_GYmC, o_GB, o_GYC, o_Ssub, o_Sout;
  int* status;
  const int* skip;     // non-zero: instance inactive, kernel returns
  double* dbg;         // optional: per-iteration history, 8 doubles per IPM iteration
  double* prof;        // optional: clock64 cycles per phase (4 doubles, accumulated)
};

struct EigSArgs {
  int k, k_curr, ssk;
  double* smalls;
  int o_sc, o_Sout, o_GC, o_W, o_Splus, o_Scplus, o_Wpast, o_VtO, o_M, o_Mc;
  int* status;
  const int* skip;
};

struct CholQRArgs {
  int k, n, shifted;
  double* smalls;
  int o_G, o_Rinv;
  int* status;
  const int* skip;
};

int launch_ipm(const IpmArgs& a, cudaStream_t st);
int launch_eigS(const EigSArgs& a, cudaStream_t st);
int launch_cholqr(const CholQRArgs& a, cudaStream_t st);

}  // namespace usbs
