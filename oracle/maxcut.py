"""MaxCut SDP builder (oracle).  Restates ``utils/maxcut_helpers.py:26-92``, the
implicit / explicit / dual-only warm starts (``utils/maxcut_helpers.py:95-289``) and
the rounding callback ``compute_max_cut`` (``utils/maxcut_helpers.py:292-302``).

Input ``W`` is the (symmetric or not) weighted adjacency matrix, as the reference
reads it from a .mat file.  C = 1/4 (diag(W 1) - W), symmetrised; constraints
diag(X) = 1 as (i, i, i) triples.  ``Omega`` defaults to
``hash_normal_matrix(1, n, sketch_dim)`` in place of ``PRNGKey(0)``.
"""
import numpy as np
import scipy.sparse as sp

from .common import SDPState, reconstruct_from_sketch, scale_sdp_state, unscale_sdp_state
from .rng import hash_normal_matrix


def laplacian_objective(W):
    n = W.shape[0]
    W = sp.csc_matrix(W, dtype=np.float64)
    C = sp.spdiags((W @ np.ones((n, 1))).T, 0, n, n) - W
    C = 0.5 * (C + C.T)
    C = 0.25 * C
    C = sp.csr_matrix(C)
    C.sum_duplicates()
    C.sort_indices()
    return C


def get_all_problem_data(n):
    A_indices = np.repeat(np.arange(n)[:, None], 3, axis=1).astype(np.int64)
    A_data = np.ones(n)
    b = np.ones(n)
    b_ineq_mask = np.zeros(n)
    return A_data, A_indices, b, b_ineq_mask


def initialize_state(W, sketch_dim, Omega=None):
    C = laplacian_objective(W)
    n = C.shape[0]
    A_data, A_indices, b, mask = get_all_problem_data(n)
    m = n
    if sketch_dim == -1:
        X, Om, P = np.zeros((n, n)), None, None
    elif sketch_dim > 0:
        X = None
        Om = hash_normal_matrix(1, n, sketch_dim) if Omega is None else np.asarray(Omega)
        P = np.zeros_like(Om)
    else:
        raise ValueError("Invalid value for sketch_dim")
    st = SDPState(C=C, A_indices=A_indices, A_data=A_data, b=b, b_ineq_mask=mask, X=X, P=P,
                  Omega=Om, y=np.zeros(m), z=np.zeros(m), tr_X=0.0, primal_obj=0.0,
                  SCALE_C=1.0, SCALE_X=1.0, SCALE_A=np.ones(m))
    return scale_sdp_state(st)


def get_implicit_warm_start_state(old, W, sketch_dim, Omega_pad=None):
    """utils/maxcut_helpers.py:95-161 (sketch or dense-X state, rows padded with zeros)."""
    old = unscale_sdp_state(old)
    C = laplacian_objective(W)
    n = C.shape[0]
    n_old = old.C.shape[0]
    A_data, A_indices, b, mask = get_all_problem_data(n)
    m = n
    X, Om, P = old.X, old.Omega, old.P
    if old.X is not None:
        X = np.zeros((n, n))
        X[:n_old, :n_old] = old.X
    if old.P is not None:
        P = np.zeros((n, sketch_dim))
        P[:n_old] = old.P
        if Omega_pad is None:
            Omega_pad = hash_normal_matrix(n, n - n_old, sketch_dim)
        Om = np.concatenate([old.Omega, Omega_pad], axis=0)
    y = np.zeros(m)
    y[:old.b.shape[0]] = old.y
    z = np.zeros(m)
    z[:old.b.shape[0]] = old.z
    old_diag = old.C.diagonal()
    new_diag = C.diagonal()
    primal_obj = old.primal_obj - old_diag @ old.z + new_diag @ z
    st = SDPState(C=C, A_indices=A_indices, A_data=A_data, b=b, b_ineq_mask=mask, X=X, P=P,
                  Omega=Om, y=y, z=z, tr_X=old.tr_X, primal_obj=primal_obj,
                  SCALE_C=1.0 / np.linalg.norm(C.data), SCALE_X=1.0 / float(n),
                  SCALE_A=np.ones(m))
    return scale_sdp_state(st)


def get_explicit_warm_start_state(old, W, sketch_dim, Omega=None):
    """utils/maxcut_helpers.py:164-229: the old iterate made explicit: dense X
    padded with zeros, or the sketch's Nystrom factors with their trace
    corrected to tr_X (E padded with zero rows) re-sketched by a fresh Omega
    (key n, in place of PRNGKey(n)); z, tr_X and primal_obj recomputed."""
    from .common import apply_A_operator_mx
    from .operators import apply_A_operator_batched
    old = unscale_sdp_state(old)
    C = laplacian_objective(W)
    n = C.shape[0]
    n_old = old.C.shape[0]
    A_data, A_indices, b, mask = get_all_problem_data(n)
    m = n
    X, Om, P = old.X, old.Omega, old.P
    if old.X is not None:
        X = np.zeros((n, n))
        X[:n_old, :n_old] = old.X
        z = apply_A_operator_mx(n, m, A_data, A_indices, X)
        tr_X = float(np.trace(X))
        primal_obj = float((C @ X).trace())
    if old.P is not None:
        Om = hash_normal_matrix(n, n, sketch_dim) if Omega is None else np.asarray(Omega)
        E, Lam = reconstruct_from_sketch(old.Omega, old.P)
        tr_offset = (old.tr_X - np.sum(Lam)) / Lam.shape[0]
        Lam_c = Lam + tr_offset
        Ep = np.zeros((n, E.shape[1]))
        Ep[:n_old] = E
        with np.errstate(invalid="ignore"):
            S = Ep * np.sqrt(Lam_c)[None, :]
        P = S @ (S.T @ Om)
        z = apply_A_operator_batched(m, A_data, A_indices, S)
        tr_X = float(np.sum(Lam_c))
        primal_obj = float(np.trace(S.T @ (C @ S)))
    y = np.zeros(m)
    y[:old.b.shape[0]] = old.y
    st = SDPState(C=C, A_indices=A_indices, A_data=A_data, b=b, b_ineq_mask=mask, X=X, P=P,
                  Omega=Om, y=y, z=z, tr_X=tr_X, primal_obj=primal_obj,
                  SCALE_C=1.0 / np.linalg.norm(C.data), SCALE_X=1.0 / float(n),
                  SCALE_A=np.ones(m))
    return scale_sdp_state(st)


def get_dual_only_warm_start_state(old, W, sketch_dim, Omega=None):
    """utils/maxcut_helpers.py:232-289."""
    old = unscale_sdp_state(old)
    C = laplacian_objective(W)
    n = C.shape[0]
    A_data, A_indices, b, mask = get_all_problem_data(n)
    m = n
    if sketch_dim == -1:
        X, Om, P = np.zeros((n, n)), None, None
    elif sketch_dim > 0:
        X = None
        Om = hash_normal_matrix(1, n, sketch_dim) if Omega is None else np.asarray(Omega)
        P = np.zeros_like(Om)
    else:
        raise ValueError("Invalid value for sketch_dim")
    y = np.zeros(m)
    y[:old.b.shape[0]] = old.y
    st = SDPState(C=C, A_indices=A_indices, A_data=A_data, b=b, b_ineq_mask=mask, X=X, P=P,
                  Omega=Om, y=y, z=np.zeros(m), tr_X=0.0, primal_obj=0.0,
                  SCALE_C=1.0 / np.linalg.norm(C.data), SCALE_X=1.0 / float(n),
                  SCALE_A=np.ones(m))
    return scale_sdp_state(st)


def compute_max_cut(P, Omega, callback_static_args, callback_nonstatic_args):
    """Largest cut among the sign patterns of the sketch's reconstructed
    eigenvectors (utils/maxcut_helpers.py:292-302): callback_nonstatic_args is
    the unscaled C; returns max_j w_j^T C w_j over w_j = sign(E[:, j]) (+1 where
    E > 0, -1 elsewhere, NaN included)."""
    C = sp.csr_matrix(callback_nonstatic_args, dtype=np.float64)
    E, _ = reconstruct_from_sketch(np.asarray(Omega, float), np.asarray(P, float))
    with np.errstate(invalid="ignore"):
        W_bin = 2.0 * (E > 0).astype(float) - 1.0
    return float(np.max(np.einsum("ij,ij->j", W_bin, C @ W_bin)))
