"""SDP state container, scaling and sketch reconstruction (oracle, FP64).

Restates ``utils/common.py:11-121``.  ``C`` is a SciPy sparse matrix (the
reference uses a JAX BCOO); everything else is a NumPy array or a float.
"""
from collections import namedtuple

import numpy as np
import scipy.sparse as sp

SDPState = namedtuple("SDPState", ["C", "A_indices", "A_data", "b", "b_ineq_mask", "X", "P",
                                   "Omega", "y", "z", "tr_X", "primal_obj", "SCALE_C",
                                   "SCALE_X", "SCALE_A"])


def scale_sdp_state(s):
    """utils/common.py:29-61."""
    return s._replace(
        C=(s.C * s.SCALE_C).tocsr(),
        A_data=s.A_data * s.SCALE_A[s.A_indices[:, 0]],
        b=s.b * s.SCALE_X * s.SCALE_A,
        X=None if s.X is None else s.X * s.SCALE_X,
        P=None if s.P is None else s.P * s.SCALE_X,
        z=s.z * s.SCALE_A * s.SCALE_X,
        tr_X=s.tr_X * s.SCALE_X,
        primal_obj=s.primal_obj * s.SCALE_X * s.SCALE_C)


def unscale_sdp_state(s):
    """utils/common.py:64-96."""
    return s._replace(
        C=(s.C / s.SCALE_C).tocsr(),
        A_data=s.A_data / s.SCALE_A[s.A_indices[:, 0]],
        b=(s.b / s.SCALE_A) / s.SCALE_X,
        X=None if s.X is None else s.X / s.SCALE_X,
        P=None if s.P is None else s.P / s.SCALE_X,
        z=(s.z / s.SCALE_A) / s.SCALE_X,
        tr_X=s.tr_X / s.SCALE_X,
        primal_obj=s.primal_obj / (s.SCALE_X * s.SCALE_C))


def reconstruct_from_sketch(Omega, P, approx_eps=1e-6):
    """Nystrom reconstruction from the sketch P = X Omega (utils/common.py:99-116)."""
    n = Omega.shape[0]
    rho = np.sqrt(n) * approx_eps * np.linalg.norm(P, ord=2)
    P_rho = P + rho * Omega
    B = Omega.T @ P_rho
    B = 0.5 * (B + B.T)
    try:
        L = np.linalg.cholesky(B)
    except np.linalg.LinAlgError:
        # jnp.linalg.cholesky returns NaNs for a matrix that is not positive
        # definite (a zero sketch, for one), and the NaNs flow through
        s = P.shape[1]
        return np.full((n, s), np.nan), np.full(s, np.nan)
    E, Rho, _ = np.linalg.svd(np.linalg.lstsq(L, P_rho.T, rcond=None)[0].T, full_matrices=False)
    Lam = np.clip(Rho ** 2 - rho, 0, np.inf)
    return E, Lam


def apply_A_operator_mx(n, m, A_data, A_indices, X):
    """A(X) for a dense X (utils/common.py:119-121)."""
    w = A_data * X[A_indices[:, 1], A_indices[:, 2]]
    return np.bincount(A_indices[:, 0], weights=w, minlength=m).astype(np.float64)


def to_csr(C):
    return sp.csr_matrix(C, dtype=np.float64)
