"""Thick-restart Lanczos for the smallest eigenpairs (oracle, FP64).

Restates ``solver/lanczos.py`` line by line:
  * ``_iterative_classical_gram_schmidt``  solver/lanczos.py:59-77 (CGS2)
  * ``_lanczos_restart``                   solver/lanczos.py:80-125
  * ``_build_arrowhead_matrix``            solver/lanczos.py:128-135
  * ``_pick_saved_ritz_values``            solver/lanczos.py:138-168
  * ``_thick_restart_lanczos``             solver/lanczos.py:177-236
  * ``eigsh_smallest``                     solver/lanczos.py:239-284

JAX gathers clamp out-of-range indices (``lambda_[num_converged]`` with
num_converged == m, ``lambda_[kr]`` with kr >= m); the clamps are explicit here.
The breakdown vector for step i is ``hash_normal(i + 1, n)`` instead of
``jax.random.normal(PRNGKey(i + 1))``.
"""
import numpy as np

from .loop import while_loop
from .operators import apply_A_adjoint_slim
from .rng import hash_normal


def _cgs2(Q, x):
    q = x
    h = Q.T @ q
    q = q - Q @ h
    r = h
    h = Q.T @ q
    q = q - Q @ h
    r = r + h
    return r, q


def make_operator(negC, A_data, A_indices, w):
    """x -> (negC @ x) + A*(w) x, the map eigsh_smallest works on (solver/lanczos.py:86-87)."""
    n = negC.shape[0]

    def op(x):
        return negC @ x + apply_A_adjoint_slim(n, A_data, A_indices, w, x)
    return op


def lanczos_restart(n, op, k, m, Q, alpha, beta, trace=None):
    for i in range(k, m):
        q = op(Q[:, i])
        valid = (i >= np.arange(m + 1)).astype(np.float64)
        Qv = Q * valid[None, :]
        r, q = _cgs2(Qv, q)
        a = r[i]
        b = np.linalg.norm(q)
        if b < 1e-15:
            _, qq = _cgs2(Qv, hash_normal(i + 1, n))
            q = qq / np.linalg.norm(qq)
        else:
            q = q / b
        Q[:, i + 1] = q
        alpha[i] = a
        beta[i] = b
        if trace is not None:
            trace.append(("step", i, a, b))
    return Q, alpha, beta


def build_arrowhead_matrix(alpha, beta, k):
    m = alpha.size
    ar = np.arange(m)
    upper = np.outer(beta * (k > ar), (k == ar).astype(np.float64))
    upper = upper + np.diag(beta[:-1] * (k <= np.arange(m - 1)), k=1)
    return upper + upper.T + np.diag(alpha)


def pick_saved_ritz_values(lam, num_converged, num_desired):
    m = lam.size
    delta = min(m - num_desired, 2 * (m - num_converged) // 5)
    kr = np.arange(m) + delta
    lam_t = lam[min(num_converged, m - 1)]
    with np.errstate(divide="ignore", invalid="ignore"):
        gamma = np.where(kr <= m, (lam - lam_t) / (lam[np.minimum(kr, m - 1)] - lam_t), 0.0)
    k_left = int(np.argmax(gamma))
    k_right = k_left + delta
    ar = np.arange(m)
    return (k_left >= ar) | (k_right < ar), gamma


def thick_restart_lanczos(n, op, q0, num_desired, inner_iterations, max_restarts, tolerance,
                          trace=None):
    m = inner_iterations
    Q = np.zeros((n, m + 1))
    Q[:, 0] = q0
    state = dict(Q=Q, alpha=np.zeros(m), beta=np.zeros(m), restart=0, k=0, nconv=0)

    def cond(s):
        return s["nconv"] < num_desired

    def body(s):
        Q, alpha, beta = lanczos_restart(n, op, s["k"], m, s["Q"].copy(), s["alpha"].copy(),
                                         s["beta"].copy(), trace)
        T = build_arrowhead_matrix(alpha, beta, s["k"])
        ritz, Y = np.linalg.eigh(T)
        resid = beta[-1] * np.abs(Y[-1, :])
        conv = resid < tolerance
        nconv = m if conv.all() else int(np.argmin(conv))
        saved, _ = pick_saved_ritz_values(ritz, nconv, num_desired)
        k_next = int(saved.sum())
        order = np.argsort(~saved, kind="stable")
        ritz = ritz[order]
        Y = Y[:, order]
        upd = k_next > np.arange(m)
        alpha_hat = np.where(upd, ritz, 0.0)
        beta_hat = np.where(upd, beta[-1] * Y[-1, :], 0.0)
        Qh = Q.copy()
        Qh[:, :-1] = np.where(upd[None, :], Q[:, :-1] @ Y, Q[:, :-1])
        Qh[:, k_next] = Q[:, -1]
        if trace is not None:
            trace.append(("restart", s["restart"], k_next, nconv, ritz.copy()))
        return dict(Q=Qh, alpha=alpha_hat, beta=beta_hat, restart=s["restart"] + 1, k=k_next,
                    nconv=nconv)

    return while_loop(cond, body, state, max_restarts)


def eigsh_smallest(n, C, A_data, A_indices, adjoint_left_vec, q0, num_desired, inner_iterations,
                   max_restarts, tolerance, trace=None):
    """Smallest ``num_desired`` eigenpairs of C + A*(adjoint_left_vec) (solver/lanczos.py:239).

    ``C`` is whatever matrix the caller passes (the solvers pass ``-state.C``)."""
    op = make_operator(C, A_data, A_indices, adjoint_left_vec)
    st = thick_restart_lanczos(n, op, q0, num_desired, inner_iterations, max_restarts, tolerance,
                               trace)
    return st["alpha"][:num_desired].copy(), st["Q"][:, :num_desired].copy(), st
