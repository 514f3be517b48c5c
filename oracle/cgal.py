"""CGAL baseline solver (oracle, FP64).  Restates ``solver/cgal.py:21-243``.

``q0`` is an input (default :func:`oracle.rng.default_q0`), standing in for the
``PRNGKey(0)`` draw the reference repeats every iteration (solver/cgal.py:108-109).
"""
import time

import numpy as np

from .common import SDPState
from .lanczos import eigsh_smallest
from .loop import while_loop
from .operators import apply_A_adjoint_slim, apply_A_operator_slim
from .rng import default_q0


def cgal(sdp_state, n, m, trace_ub, beta0, max_iters, max_time, obj_gap_eps, infeas_gap_eps,
         max_infeas_eps, lanczos_inner_iterations, lanczos_max_restarts, subprob_eps,
         cond_exp_base=1.0, callback_fn=None, callback_static_args=None,
         callback_nonstatic_args=None, q0=None, trace=None):
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
        t, y, z = st["t"], st["y"], st["z"]
        beta = beta0 * np.sqrt(t + 1)
        proj_b = (1 - mask) * b + mask * np.minimum(z + (1.0 / beta) * y, b)
        adj = y + beta * (z - proj_b)
        vals, vecs, _ = eigsh_smallest(n, negC, A_data, A_idx, adj, q0, 1,
                                       lanczos_inner_iterations, lanczos_max_restarts,
                                       subprob_eps)
        if vals[0] >= 0:
            vecs = 0.0 * vecs
        v = vecs[:, 0]
        Cv = C @ v
        sdg = trace_ub * (v @ Cv) - st["primal_obj"]
        sdg += adj @ z
        sdg -= trace_ub * (v @ apply_A_adjoint_slim(n, A_data, A_idx, adj, v))
        obj_gap = sdg - y @ (z - proj_b)
        obj_gap -= 0.5 * beta * np.linalg.norm(z - proj_b) ** 2
        obj_gap = obj_gap / (SCALE_C * SCALE_X)
        obj_gap /= 1.0 + (abs(st["primal_obj"]) / (SCALE_C * SCALE_X))

        proj_b = (1 - mask) * b + mask * np.minimum(z, b)
        infeas_gap = np.linalg.norm(((z - proj_b) / SCALE_A) / SCALE_X)
        infeas_gap /= 1.0 + np.linalg.norm((proj_b / SCALE_A) / SCALE_X)
        max_infeas = np.max(np.abs((z - proj_b) / SCALE_A)) / SCALE_X

        eta = 2.0 / (t + 2.0)
        X_n = P_n = None
        if st["Omega"] is None:
            X_n = (1 - eta) * st["X"] + eta * trace_ub * np.outer(v, v)
        else:
            P_n = (1 - eta) * st["P"] + eta * trace_ub * np.outer(v, v @ st["Omega"])
        tr_X_n = (1 - eta) * st["tr_X"] + eta * trace_ub * np.linalg.norm(v) ** 2
        z_n = (1 - eta) * z + eta * trace_ub * apply_A_operator_slim(m, A_data, A_idx, v)

        beta = beta0 * np.sqrt(t + 2)
        proj_b = (1 - mask) * b + mask * np.minimum(z_n + (1.0 / beta) * y, b)
        with np.errstate(divide="ignore"):
            dss = np.clip(4 * beta * eta ** 2 * trace_ub ** 2 / np.sum(np.square(z_n - proj_b)),
                          0.0, beta0)
        y_n = y + dss * (z_n - proj_b)
        primal_n = (1 - eta) * st["primal_obj"] + eta * trace_ub * (v @ Cv)

        new = dict(st)
        new.update(t=t + 1, X=X_n, P=P_n, y=y_n, z=z_n, tr_X=tr_X_n, curr_time=time.time(),
                   obj_gap=obj_gap, infeas_gap=infeas_gap, max_infeas=max_infeas,
                   primal_obj=primal_n)
        if trace is not None:
            trace.append(dict(t=t, eig0=vals[0], obj_gap=obj_gap, infeas_gap=infeas_gap,
                              max_infeas=max_infeas, primal_obj=primal_n, tr_X=tr_X_n,
                              dual_step=dss))
        return new

    t0 = time.time()
    st = dict(t=0, Omega=sdp_state.Omega, X=sdp_state.X, P=sdp_state.P, y=sdp_state.y,
              z=sdp_state.z, tr_X=sdp_state.tr_X, start_time=t0, curr_time=t0,
              obj_gap=1.1 * obj_gap_eps, infeas_gap=1.1 * infeas_gap_eps,
              max_infeas=1.1 * max_infeas_eps, primal_obj=sdp_state.primal_obj)
    fin = while_loop(cond, body, st, max_iters, cond_exp_base)
    out = SDPState(C=sdp_state.C, A_indices=A_idx, A_data=A_data, b=b, b_ineq_mask=mask,
                   X=fin["X"], P=fin["P"], Omega=sdp_state.Omega, y=fin["y"], z=fin["z"],
                   tr_X=fin["tr_X"], primal_obj=fin["primal_obj"], SCALE_C=SCALE_C,
                   SCALE_X=SCALE_X, SCALE_A=SCALE_A)
    return out, fin
