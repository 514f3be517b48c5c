"""MaxCut SDP instances (reference: utils/maxcut_helpers.py:26-92) and their
warm starts (implicit, explicit, dual-only: utils/maxcut_helpers.py:95-289).

maximise <C, X>  s.t.  diag(X) = 1,  tr(X) <= trace_ub,  X PSD,
with C = 1/4 (diag(W 1) - W) symmetrised.  The constraint tensor is the list of
(i, i, i) triples with value 1 and b = 1.  Set-up runs on the host.
"""
import numpy as np
import scipy.sparse as sp

from ..arrays import to_host
from ..rng import hash_normal_matrix
from ..state import SDPState, scale_sdp_state, unscale_sdp_state


def objective(W):
    """C = 1/4 sym(diag(W 1) - W) as CSR (utils/maxcut_helpers.py:38-41)."""
    W = sp.csr_matrix(W, dtype=np.float64)
    n = W.shape[0]
    deg = np.asarray(W @ np.ones(n)).ravel()
    C = sp.diags(deg) - W
    C = (0.25 * (0.5 * (C + C.T))).tocsr()
    C.sum_duplicates()
    C.sort_indices()
    return C


def problem_data(n):
    """diag(X) = 1 as (c, c, c) triples (utils/maxcut_helpers.py:26-33)."""
    idx = np.arange(n, dtype=np.int64)
    return np.ones(n), np.stack([idx, idx, idx], 1), np.ones(n), np.zeros(n)


def _iterate(n, sketch_dim, Omega):
    if sketch_dim == -1:
        return np.zeros((n, n)), None, None
    if sketch_dim > 0:
        Om = hash_normal_matrix(1, n, sketch_dim) if Omega is None else np.asarray(Omega, float)
        return None, np.zeros_like(Om), Om
    raise ValueError("Invalid value for sketch_dim")


def initialize_state(W, sketch_dim, Omega=None):
    """Cold start (utils/maxcut_helpers.py:36-92); SCALE_C = SCALE_X = 1."""
    C = objective(W)
    n = C.shape[0]
    A_data, A_idx, b, mask = problem_data(n)
    X, P, Om = _iterate(n, sketch_dim, Omega)
    st = SDPState(C=C, A_indices=A_idx, A_data=A_data, b=b, b_ineq_mask=mask, X=X, P=P,
                  Omega=Om, y=np.zeros(n), z=np.zeros(n), tr_X=0.0, primal_obj=0.0,
                  SCALE_C=1.0, SCALE_X=1.0, SCALE_A=np.ones(n))
    return scale_sdp_state(st)


def implicit_warm_start(old, W, sketch_dim, Omega_pad=None):
    """Grow a solved instance to the graph W (utils/maxcut_helpers.py:95-161):
    pad X / P with zero rows, extend Omega, carry y and z, correct the primal
    objective for the changed diagonal of C, rescale with SCALE_X = 1/n and
    SCALE_C = 1/||C||_F."""
    old = unscale_sdp_state(old)
    C = objective(W)
    n = C.shape[0]
    n_old = old.C.shape[0]
    A_data, A_idx, b, mask = problem_data(n)
    X, P, Om = old.X, old.P, old.Omega
    if old.X is not None:
        X = np.zeros((n, n))
        X[:n_old, :n_old] = np.asarray(old.X)
    if old.P is not None:
        P = np.zeros((n, sketch_dim))
        P[:n_old] = np.asarray(old.P)
        pad = hash_normal_matrix(n, n - n_old, sketch_dim) if Omega_pad is None else Omega_pad
        Om = np.concatenate([_host(old.Omega), pad], axis=0)
    m_old = np.asarray(old.b).shape[0]
    y = np.zeros(n); y[:m_old] = _host(old.y)
    z = np.zeros(n); z[:m_old] = np.asarray(old.z)
    primal = old.primal_obj - old.C.diagonal() @ np.asarray(old.z) + C.diagonal() @ z
    st = SDPState(C=C, A_indices=A_idx, A_data=A_data, b=b, b_ineq_mask=mask, X=X, P=P,
                  Omega=Om, y=y, z=z, tr_X=old.tr_X, primal_obj=primal,
                  SCALE_C=1.0 / np.linalg.norm(C.data), SCALE_X=1.0 / float(n),
                  SCALE_A=np.ones(n))
    return scale_sdp_state(st)


def explicit_warm_start(old, W, sketch_dim, Omega=None, device="cuda"):
    """Make the old iterate explicit on the graph W (utils/maxcut_helpers.py:
    164-229): a dense X is padded with zeros; a sketch is replaced by its
    Nystrom factors (reconstructed on the device), their trace corrected to
    tr_X, padded with zero rows and re-sketched by a fresh Omega (key n);
    z = diag(X), tr_X and the primal objective are recomputed."""
    old = unscale_sdp_state(old)
    C = objective(W)
    n = C.shape[0]
    n_old = old.C.shape[0]
    A_data, A_idx, b, mask = problem_data(n)
    X, P, Om = old.X, old.P, old.Omega
    if old.X is not None:
        X = np.zeros((n, n))
        X[:n_old, :n_old] = np.asarray(old.X)
        z = np.diagonal(X).copy()
        tr_X = float(np.trace(X))
        primal = float((C @ X).trace())
    if old.P is not None:
        from ..rounding import reconstruct_from_sketch
        Om = hash_normal_matrix(n, n, sketch_dim) if Omega is None else np.asarray(Omega, float)
        E, lam = reconstruct_from_sketch(_host(old.Omega), _host(old.P), device=device)
        E, lam = E.cpu().numpy(), lam.cpu().numpy()
        lam_c = lam + (old.tr_X - lam.sum()) / lam.shape[0]
        S = np.zeros((n, E.shape[1]))
        with np.errstate(invalid="ignore"):
            S[:n_old] = E * np.sqrt(lam_c)[None, :]
        P = S @ (S.T @ Om)
        z = np.einsum("ij,ij->i", S, S)          # A(S S^T) for the diag(X) = 1 rows
        tr_X = float(lam_c.sum())
        primal = float(np.einsum("ij,ij->", S, C @ S))
    y = np.zeros(n)
    y[:np.asarray(old.b).shape[0]] = _host(old.y)
    st = SDPState(C=C, A_indices=A_idx, A_data=A_data, b=b, b_ineq_mask=mask, X=X, P=P,
                  Omega=Om, y=y, z=z, tr_X=tr_X, primal_obj=primal,
                  SCALE_C=1.0 / np.linalg.norm(C.data), SCALE_X=1.0 / float(n),
                  SCALE_A=np.ones(n))
    return scale_sdp_state(st)


def _host(x):
    return np.asarray(to_host(x), float)


def dual_only_warm_start(old, W, sketch_dim, Omega=None):
    """Keep only the dual y (utils/maxcut_helpers.py:232-289)."""
    old = unscale_sdp_state(old)
    C = objective(W)
    n = C.shape[0]
    A_data, A_idx, b, mask = problem_data(n)
    X, P, Om = _iterate(n, sketch_dim, Omega)
    y = np.zeros(n); y[:np.asarray(old.b).shape[0]] = _host(old.y)
    st = SDPState(C=C, A_indices=A_idx, A_data=A_data, b=b, b_ineq_mask=mask, X=X, P=P,
                  Omega=Om, y=y, z=np.zeros(n), tr_X=0.0, primal_obj=0.0,
                  SCALE_C=1.0 / np.linalg.norm(C.data), SCALE_X=1.0 / float(n),
                  SCALE_A=np.ones(n))
    return scale_sdp_state(st)
