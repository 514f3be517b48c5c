"""USBS outer loop (oracle, FP64).

Restates ``solver/usbs.py:359-789``: ``solve_step_subprob`` (359-433) and
``usbs`` (436-789) with its ``cond_func`` (502-540) and ``body_func`` (543-688).

Differences that are not arithmetic:
  * ``q0`` is an input (default :func:`oracle.rng.default_q0`) because
    ``jax.random.normal(PRNGKey(0))`` (solver/usbs.py:691) needs JAX;
  * ``create_Q_base`` and the V-projections are computed once per outer
    iteration; the reference recomputes the same values inside every
    alternating-minimisation pass;
  * a per-iteration trace (list of dicts) can be collected for parity tests;
  * ``max_time`` uses ``time.time()`` as the reference's io_callback does.
"""
import time

import numpy as np

from .common import SDPState
from .ipm import compute_lb_spec_est_ipm, quad_constants, solve_quad_subprob_ipm
from .lanczos import eigsh_smallest
from .loop import while_loop
from .operators import (adjoint_gram, apply_A_operator_batched, create_Q_base,
                        create_svec_matrix)
from .rng import default_q0


def solve_step_subprob(C, A_data, A_indices, U, b, b_ineq_mask, upsilon, trace_ub, rho,
                       bar_primal_obj, z_bar, tr_X_bar, y, V, n, m, k, subprob_eps,
                       subprob_max_iters, CV=None, info=None):
    """solver/usbs.py:359-433."""
    Q_base = create_Q_base(m, k, U, A_data, A_indices, V)
    if CV is None:
        CV = C @ V
    G_C = V.T @ CV
    G_y = adjoint_gram(A_data, A_indices, y, V)
    G_zbar = adjoint_gram(A_data, A_indices, z_bar, V)

    tr_X_bar_eff = tr_X_bar if tr_X_bar > 0.0 else trace_ub
    S_init = 0.99 * (np.eye(k) / (k + 1.0))
    eta_init = 0.00001 if bar_primal_obj == 0.0 else 0.99 * (1.0 / (k + 1.0))
    eta_init = (trace_ub / tr_X_bar_eff) * eta_init
    S_init = trace_ub * S_init

    def body(st):
        ups = st["upsilon"]
        bmu = b - ups
        consts = quad_constants(U, k, trace_ub, rho, Q_base, G_C, G_y,
                                adjoint_gram(A_data, A_indices, bmu, V), G_zbar,
                                z_bar @ z_bar, z_bar @ y, z_bar @ bmu, bar_primal_obj, tr_X_bar)
        eta_n, S_n = solve_quad_subprob_ipm(U, k, trace_ub, consts, st["eta"], st["S"],
                                            subprob_eps, subprob_max_iters, info)
        lam, W = np.linalg.eigh(S_n)
        lam = np.clip(lam, 0, None)
        F = (V @ W) * np.sqrt(lam)[None, :]
        z_n = eta_n * z_bar + apply_A_operator_batched(m, A_data, A_indices, F)
        ups_n = b_ineq_mask * np.clip(b - z_n - rho * y, 0.0, None)
        gap = np.max(np.abs(ups - ups_n))
        return dict(i=st["i"] + 1, eta=eta_n, S=S_n, upsilon=ups_n, gap=gap)

    init = dict(i=0, eta=eta_init, S=S_init, upsilon=upsilon, gap=1.0)
    fin = while_loop(lambda s: s["gap"] > subprob_eps, body, init, subprob_max_iters)
    if info is not None:
        info["subprob_iters"] = fin["i"]
        info["upsilon_gap"] = fin["gap"]
    return fin["eta"], fin["S"], fin["upsilon"], G_C


def usbs(sdp_state, n, m, trace_ub, trace_factor, rho, beta, k_curr, k_past, max_iters, max_time,
         obj_gap_eps, infeas_gap_eps, max_infeas_eps, lanczos_inner_iterations,
         lanczos_max_restarts, subprob_eps, subprob_max_iters, cond_exp_base=1.0,
         callback_fn=None, callback_static_args=None, callback_nonstatic_args=None, q0=None,
         trace=None):
    """solver/usbs.py:436-789.  Returns the final SDPState."""
    k = k_curr + k_past
    U = create_svec_matrix(k)
    SCALE_C, SCALE_X, SCALE_A = sdp_state.SCALE_C, sdp_state.SCALE_X, sdp_state.SCALE_A
    C = sdp_state.C.tocsr()
    negC = (-C).tocsr()
    A_data, A_idx = sdp_state.A_data, sdp_state.A_indices
    b, mask = sdp_state.b, sdp_state.b_ineq_mask
    if q0 is None:
        q0 = default_q0(n)

    def cond(st):
        if st["Omega"] is not None and callback_fn is not None:
            st["callback_val"] = callback_fn(st["P"], st["Omega"], callback_static_args,
                                             callback_nonstatic_args)
        return (st["t"] == 0) or ((st["curr_time"] - st["start_time"] < max_time) and (
            st["obj_gap"] > obj_gap_eps or st["infeas_gap"] > infeas_gap_eps
            or st["max_infeas"] > max_infeas_eps))

    def body(st):
        info = {"qhist": []}
        V = st["V"]
        CV = C @ V
        eta, S, ups_n, G_C = solve_step_subprob(
            C, A_data, A_idx, U, b, mask, st["upsilon"], trace_ub, rho, st["bar_primal_obj"],
            st["z_bar"], st["tr_X_bar"], st["y"], V, n, m, k, subprob_eps, subprob_max_iters,
            CV=CV, info=info)
        lam, W = np.linalg.eigh(S)
        lam = np.clip(lam, 0, None)
        F = (V @ W) * np.sqrt(lam)[None, :]
        AF = apply_A_operator_batched(m, A_data, A_idx, F)
        X_n = P_n = None
        if st["Omega"] is None and st["X"] is None:
            P_n = eta * st["P_bar"] + np.sum(F * F, axis=1)
        elif st["X_bar"] is not None:
            X_n = eta * st["X_bar"] + V @ S @ V.T
        else:
            P_n = eta * st["P_bar"] + F @ (F.T @ st["Omega"])
        tr_X_n = eta * st["tr_X_bar"] + np.trace(S)
        z_n = eta * st["z_bar"] + AF
        y_cand = st["y"] - (1.0 / rho) * (b - z_n - ups_n)
        primal_n = eta * st["bar_primal_obj"] + np.trace(F.T @ (C @ F))

        cand_vals, cand_vecs, _ = eigsh_smallest(n, negC, A_data, A_idx, y_cand, q0, k_curr,
                                                 lanczos_inner_iterations, lanczos_max_restarts,
                                                 subprob_eps)
        cand_vals = -cand_vals
        cand_pen = b @ y_cand + trace_ub * max(cand_vals[0], 0.0)
        obj_ub = min(b @ y_cand + (trace_ub / trace_factor) * max(cand_vals[0], 0.0),
                     st["obj_ub"])
        G_ycand = adjoint_gram(A_data, A_idx, y_cand, V)
        lb = compute_lb_spec_est_ipm(U, k, trace_ub, b @ y_cand, G_C, G_ycand,
                                     st["z_bar"] @ y_cand, st["bar_primal_obj"], st["tr_X_bar"],
                                     subprob_eps, subprob_max_iters, info)
        descent = beta * (st["pen_dual_obj"] - lb) <= st["pen_dual_obj"] - cand_pen
        y_n = y_cand if descent else st["y"]
        pen_n = cand_pen if descent else st["pen_dual_obj"]

        Fc = (V @ W[:, :k_curr]) * np.sqrt(lam[:k_curr])[None, :]
        X_bar_n = P_bar_n = None
        if st["Omega"] is None and st["X"] is None:
            P_bar_n = eta * st["P_bar"] + np.sum(Fc * Fc, axis=1)
        elif st["X_bar"] is not None:
            X_bar_n = eta * st["X_bar"] + Fc @ Fc.T
        else:
            P_bar_n = eta * st["P_bar"] + Fc @ (Fc.T @ st["Omega"])
        tr_X_bar_n = eta * st["tr_X_bar"] + np.sum(lam[:k_curr])
        z_bar_n = eta * st["z_bar"] + apply_A_operator_batched(m, A_data, A_idx, Fc)
        V_n, _ = np.linalg.qr(np.concatenate([V @ W[:, k_curr:], cand_vecs], axis=1))
        bar_primal_n = eta * st["bar_primal_obj"] + np.trace(Fc.T @ (C @ Fc))

        obj_gap = abs(obj_ub - primal_n) / (SCALE_C * SCALE_X)
        obj_gap /= 1.0 + max(abs(primal_n), abs(obj_ub)) / (SCALE_C * SCALE_X)
        infeas = np.clip(z_n - b, 0.0, None) + (1.0 - mask) * np.clip(b - z_n, 0.0, None)
        infeas_gap = np.linalg.norm(infeas / SCALE_A) / SCALE_X
        infeas_gap /= 1.0 + np.linalg.norm((b / SCALE_A) / SCALE_X)
        max_infeas = np.max(np.abs(infeas) / SCALE_A) / SCALE_X

        new = dict(st)
        new.update(t=st["t"] + 1, upsilon=ups_n, X=X_n, tr_X=tr_X_n, X_bar=X_bar_n,
                   tr_X_bar=tr_X_bar_n, P=P_n, P_bar=P_bar_n, z=z_n, z_bar=z_bar_n, y=y_n, V=V_n,
                   curr_time=time.time(), obj_gap=obj_gap, infeas_gap=infeas_gap,
                   max_infeas=max_infeas, primal_obj=primal_n, bar_primal_obj=bar_primal_n,
                   pen_dual_obj=pen_n, cand_pen_dual_obj=cand_pen, lb_spec_est=lb, obj_ub=obj_ub)
        if trace is not None:
            trace.append(dict(t=st["t"], eta=eta, trS=np.trace(S), lam=lam.copy(),
                              primal_obj=primal_n, bar_primal_obj=bar_primal_n, obj_ub=obj_ub,
                              cand_eig0=cand_vals[0], cand_eigvals=cand_vals.copy(),
                              cand_pen_dual_obj=cand_pen, lb_spec_est=lb, descent=bool(descent),
                              pen_dual_obj=pen_n, obj_gap=obj_gap, infeas_gap=infeas_gap,
                              max_infeas=max_infeas, tr_X=tr_X_n, tr_X_bar=tr_X_bar_n,
                              y_sum=float(np.sum(y_n)), z_sum=float(np.sum(z_n)), **info))
        return new

    init_vals, init_vecs, _ = eigsh_smallest(n, negC, A_data, A_idx, sdp_state.y, q0, k,
                                             lanczos_inner_iterations, lanczos_max_restarts,
                                             subprob_eps)
    init_vals = -init_vals
    init_pen = b @ sdp_state.y + trace_ub * max(init_vals[0], 0.0)
    t0 = time.time()
    st = dict(t=0, upsilon=np.zeros(m), Omega=sdp_state.Omega, X=sdp_state.X, tr_X=sdp_state.tr_X,
              X_bar=sdp_state.X, tr_X_bar=sdp_state.tr_X, P=sdp_state.P, P_bar=sdp_state.P,
              z=sdp_state.z, z_bar=sdp_state.z, y=sdp_state.y, V=init_vecs, start_time=t0,
              curr_time=t0, obj_gap=1.1 * obj_gap_eps, infeas_gap=1.1 * infeas_gap_eps,
              max_infeas=1.1 * max_infeas_eps, primal_obj=sdp_state.primal_obj,
              bar_primal_obj=sdp_state.primal_obj, pen_dual_obj=init_pen,
              cand_pen_dual_obj=init_pen, lb_spec_est=0.0, obj_ub=np.inf)
    fin = while_loop(cond, body, st, max_iters, cond_exp_base)
    out = SDPState(C=sdp_state.C, A_indices=A_idx, A_data=A_data, b=b, b_ineq_mask=mask,
                   X=fin["X"], P=fin["P"], Omega=sdp_state.Omega, y=fin["y"], z=fin["z"],
                   tr_X=fin["tr_X"], primal_obj=fin["primal_obj"], SCALE_C=SCALE_C,
                   SCALE_X=SCALE_X, SCALE_A=SCALE_A)
    return out, fin
