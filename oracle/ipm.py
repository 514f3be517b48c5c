"""k x k bundle subproblems solved by primal-dual interior point (oracle, FP64).

Restates ``solver/usbs.py``:
  * ``solve_quad_subprob_ipm``   solver/usbs.py:25-192
  * ``compute_lb_spec_est_ipm``  solver/usbs.py:195-356

The n-sized inputs are passed already projected onto the bundle basis V:
``Q_base`` = create_Q_base (solver/usbs.py:54), and the k x k matrices
``G_C`` = V^T C V, ``G_w`` = V^T A*(w) V for the vectors w the reference uses
(solver/usbs.py:55-61, 219-220).  The line search keeps the reference's grid of
0.9**j step sizes and its "smallest eigenvalue > 0" test (solver/usbs.py:134-154).
"""
from collections import namedtuple

import numpy as np

from .loop import while_loop
from .operators import svec, svec_inv


IPMState = namedtuple("IPMState", ["i", "S", "eta", "T", "zeta", "omega", "mu", "step_size"])


def _line_search(S, dS, T, dT, ipm_max_iters):
    steps = 0.9 ** np.arange(ipm_max_iters)
    minS = np.linalg.eigvalsh(S[None] + steps[:, None, None] * dS[None])[:, 0]
    minT = np.linalg.eigvalsh(T[None] + steps[:, None, None] * dT[None])[:, 0]
    cS = np.max(steps * (minS > 0))
    cT = np.max(steps * (minT > 0))
    return cS if cS < cT else cT


def _sym_kron(U, T, S_inv):
    return 0.5 * U @ (np.kron(T, S_inv) + np.kron(S_inv, T)) @ U.T


def _step_and_mu(st, dS, d_eta, dT, d_zeta, d_omega, k, ipm_max_iters, svec_I, U, hist=None):
    numers = np.array([st.eta, st.zeta, st.omega])
    denoms = np.array([d_eta, d_zeta, d_omega])
    with np.errstate(divide="ignore", invalid="ignore"):
        step = min(-1.0 / np.min(denoms / numers), 1.0)
    step = 0.99 * (1.0 if step <= 0.0 else step)
    cand = _line_search(st.S, dS, st.T, dT, ipm_max_iters)
    step = step if step < cand else cand
    S_n = st.S + step * dS
    eta_n = st.eta + step * d_eta
    T_n = st.T + step * dT
    zeta_n = st.zeta + step * d_zeta
    omega_n = st.omega + step * d_omega
    mu_n = (svec(U, S_n) @ svec(U, T_n) + eta_n * zeta_n
            + omega_n * (1 - svec_I @ svec(U, S_n) - eta_n)) / (2 * k + 4.0)
    mu_n *= (0.5 - 0.4 * step ** 2) if step > 0.2 else 1.0
    mu_n = min(mu_n, st.mu)
    if hist is not None:
        hist.append((mu_n, step, eta_n, zeta_n, omega_n, d_eta, d_omega, np.trace(S_n)))
    return IPMState(st.i + 1, S_n, eta_n, T_n, zeta_n, omega_n, mu_n, step)


def _init_dual(U, k, S_init, eta_init, T_svec, zeta_init, svec_I):
    T_init = svec_inv(U, T_svec, k)
    vals = np.append(np.diag(T_init), zeta_init)
    width = max(np.max(vals) - np.min(vals), 100.0)
    omega = max(-1.01 * np.min(vals), width)
    T_init = T_init + omega * np.eye(k)
    zeta_init = zeta_init + omega
    mu = (svec(U, S_init) @ svec(U, T_init) + eta_init * zeta_init
          + omega * (1 - svec_I @ svec(U, S_init) - eta_init)) / (2 * k + 4.0)
    return T_init, zeta_init, omega, mu


def quad_constants(U, k, trace_ub, rho, Q_base, G_C, G_y, G_bmu, G_zbar, zbar_zbar, zbar_y,
                   zbar_bmu, bar_primal_obj, tr_X_bar):
    """Problem constants of solve_quad_subprob_ipm (solver/usbs.py:53-61)."""
    tr_X_bar = tr_X_bar if tr_X_bar > 0.0 else trace_ub
    Q_11 = (trace_ub ** 2 / rho) * Q_base
    q_12 = (trace_ub ** 2 / (rho * tr_X_bar)) * svec(U, G_zbar)
    q_22 = (trace_ub ** 2 / (rho * tr_X_bar ** 2)) * zbar_zbar
    h_1 = trace_ub * svec(U, G_y - G_C - G_bmu / rho)
    h_2 = (trace_ub / tr_X_bar) * (zbar_y - bar_primal_obj - zbar_bmu / rho)
    return tr_X_bar, Q_11, q_12, q_22, h_1, h_2


def solve_quad_subprob_ipm(U, k, trace_ub, consts, eta_init, S_init, ipm_eps, ipm_max_iters,
                           info=None):
    tr_X_bar, Q_11, q_12, q_22, h_1, h_2 = consts
    svec_I = svec(U, np.eye(k))
    eta0 = (tr_X_bar / trace_ub) * eta_init
    S0 = S_init / trace_ub
    T_svec = Q_11 @ svec(U, S0) + eta0 * q_12 + h_1
    zeta0 = q_12 @ svec(U, S0) + eta0 * q_22 + h_2
    T0, zeta0, omega0, mu0 = _init_dual(U, k, S0, eta0, T_svec, zeta0, svec_I)

    def body(st):
        sS = svec(U, st.S)
        tI_S = svec_I @ sS
        k1 = (1 - tI_S - st.eta) / st.omega
        k2 = (st.zeta / st.eta) + q_22
        F_1 = Q_11 @ sS + st.eta * q_12 + h_1
        F_1 = F_1 + (-svec(U, st.T) + st.omega * svec_I)
        F_2 = q_12 @ sS + st.eta * q_22 + h_2
        F_2 = F_2 + (-st.zeta + st.omega)
        S_inv = np.linalg.inv(st.S)
        coeff = Q_11 + _sym_kron(U, st.T, S_inv)
        den = k1 * k2 + 1
        coeff = coeff - (np.outer(q_12, k1 * q_12 + svec_I)
                         + np.outer(svec_I, q_12 - k2 * svec_I)) / den
        ordv = -F_1 + st.mu * svec(U, S_inv) - svec(U, st.T)
        ordv = ordv + ((st.mu / st.omega + tI_S + st.eta - 1
                        + k1 * (F_2 - st.mu / st.eta + st.zeta)) / den) * q_12
        ordv = ordv + ((F_2 - st.mu / st.eta + st.zeta
                        - k2 * (st.mu / st.omega + tI_S + st.eta - 1)) / den) * svec_I
        dsS = np.linalg.solve(coeff, ordv)
        d_eta = (-(k1 * q_12 + svec_I) @ dsS - (st.mu / st.omega) - tI_S - st.eta + 1
                 + k1 * (-F_2 + st.mu / st.eta - st.zeta)) / den
        d_omega = (-F_2 + st.mu / st.eta - st.zeta
                   + k2 * (st.mu / st.omega + tI_S + st.eta - 1)
                   - (q_12 - k2 * svec_I) @ dsS) / den
        dsT = Q_11 @ dsS + d_eta * q_12 + d_omega * svec_I + F_1
        d_zeta = q_12 @ dsS + d_eta * q_22 + d_omega + F_2
        return _step_and_mu(st, svec_inv(U, dsS, k), d_eta, svec_inv(U, dsT, k), d_zeta, d_omega,
                            k, ipm_max_iters, svec_I, U, None if info is None else info.get("qhist"))

    init = IPMState(0, S0, eta0, T0, zeta0, omega0, mu0, 1.0)
    fin = while_loop(lambda s: (s.mu > ipm_eps) and (s.step_size > ipm_eps ** 2), body, init,
                     ipm_max_iters)
    if info is not None:
        info["quad_iters"] = fin.i
    return (trace_ub / tr_X_bar) * fin.eta, trace_ub * fin.S


def compute_lb_spec_est_ipm(U, k, trace_ub, b_y, G_C, G_y, zbar_y, bar_primal_obj, tr_X_bar,
                            ipm_eps, ipm_max_iters, info=None):
    tr_X_bar = tr_X_bar if tr_X_bar > 0.0 else trace_ub
    g_1 = trace_ub * svec(U, G_y - G_C)
    g_2 = (trace_ub / tr_X_bar) * (zbar_y - bar_primal_obj)
    svec_I = svec(U, np.eye(k))
    S0 = 0.99 * (np.eye(k) / (k + 1.0))
    eta0 = 0.00001 if bar_primal_obj == 0.0 else 0.99 * (1.0 / (k + 1.0))
    T0, zeta0, omega0, mu0 = _init_dual(U, k, S0, eta0, g_1, g_2, svec_I)

    def body(st):
        sS = svec(U, st.S)
        tI_S = svec_I @ sS
        k1 = (1 - tI_S - st.eta) / st.omega
        S_inv = np.linalg.inv(st.S)
        coeff = _sym_kron(U, st.T, S_inv)
        ze = st.zeta / st.eta
        coeff = coeff + (ze / (k1 * ze + 1)) * np.outer(svec_I, svec_I)
        ordv = ze * (-k1 * (st.mu / st.eta - g_2 - st.omega) + st.mu / st.omega + tI_S
                     + st.eta - 1) / (-k1 * ze - 1) * svec_I
        ordv = ordv + (g_2 - st.mu / st.eta) * svec_I - g_1
        ordv = ordv + st.mu * svec(U, S_inv)
        dsS = np.linalg.solve(coeff, ordv)
        d_eta = (svec_I @ dsS - k1 * (st.mu / st.eta - g_2 - st.omega) + st.mu / st.omega + tI_S
                 + st.eta - 1) / (-k1 * ze - 1)
        d_omega = -ze * d_eta + st.mu / st.eta
        d_omega = d_omega + (-g_2 - st.omega)
        dsT = d_omega * svec_I - svec(U, st.T) + g_1 + st.omega * svec_I
        d_zeta = d_omega - st.zeta + g_2 + st.omega
        return _step_and_mu(st, svec_inv(U, dsS, k), d_eta, svec_inv(U, dsT, k), d_zeta, d_omega,
                            k, ipm_max_iters, svec_I, U)

    init = IPMState(0, S0, eta0, T0, zeta0, omega0, mu0, 1.0)
    fin = while_loop(lambda s: s.mu > ipm_eps, body, init, ipm_max_iters)
    if info is not None:
        info["lb_iters"] = fin.i
    return b_y - g_1 @ svec(U, fin.S) - fin.eta * g_2
