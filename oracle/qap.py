"""QAP SDP relaxation builder (oracle).  Restates ``utils/qap_helpers.py:157-381``.

``build_objective_matrix`` (157-172): lifted (l^2+1) x (l^2+1) objective from the
Kronecker product of W (flow) and D (distance), shifted by one row/column.
``get_all_problem_data`` (175-318): X00 = 1, arrow constraints diag(Y) = Y_0.,
row and column sums, both partial traces, and Y >= 0 on the objective's upper
triangle (as -Y <= 0 inequality rows).  ``initialize_state`` (321-381): C = -C,
SCALE_X = 1/(l+1), SCALE_C = 1/||C||_F, SCALE_A from row norms and the ARPACK
spectral norm of the scaled constraint matrix (qap_helpers.py:335).
"""
import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import eigsh

from .common import SDPState, scale_sdp_state
from .rng import hash_normal_matrix


def build_objective_matrix(D, W):
    n = D.shape[0]
    dr, dc = np.nonzero(D)
    wr, wc = np.nonzero(W)
    d_data = D[dr, dc]
    w_data = W[wr, wc]
    rows = (dr[None, :] + n * wr[:, None]).reshape(-1) + 1
    cols = (dc[None, :] + n * wc[:, None]).reshape(-1) + 1
    data = (d_data[None, :] * w_data[:, None]).reshape(-1)
    return rows.astype(np.int64), cols.astype(np.int64), data, n * n + 1


def get_all_problem_data(C_rows, C_cols, N):
    n = N
    l = int(np.sqrt(n - 1))
    idx = [np.array([[0, 0, 0]])]
    dat = [np.array([1.0])]
    b = [np.array([1.0])]
    msk = [np.array([0.0])]
    mcount = 1
    # diag(Y) = Y_0. (arrow)
    ci = mcount + np.repeat(np.arange(n - 1), 3)
    j = np.arange(1, n)
    ca = (np.array([[1, 0, 1]]) * j[:, None]).reshape(-1)
    cb = (np.array([[0, 1, 1]]) * j[:, None]).reshape(-1)
    idx.append(np.stack([ci, ca, cb], 1))
    dat.append(np.tile(np.array([-1.0, -1.0, 2.0]), n - 1))
    b.append(np.zeros(n - 1))
    msk.append(np.zeros(n - 1))
    mcount += n - 1
    # row sums
    ci = mcount + np.repeat(np.arange(l), 2 * l)
    jj = np.arange(1, n).reshape(l, l).flatten()
    ca = (np.array([[1, 0]]) * jj[:, None]).reshape(-1)
    cb = (np.array([[0, 1]]) * jj[:, None]).reshape(-1)
    idx.append(np.stack([ci, ca, cb], 1))
    dat.append(np.ones(2 * (n - 1)))
    b.append(2.0 * np.ones(l))
    msk.append(np.zeros(l))
    mcount += l
    # column sums
    ci = mcount + np.repeat(np.arange(l), 2 * l)
    jj = np.arange(1, n).reshape(l, l).T.flatten()
    ca = (np.array([[1, 0]]) * jj[:, None]).reshape(-1)
    cb = (np.array([[0, 1]]) * jj[:, None]).reshape(-1)
    idx.append(np.stack([ci, ca, cb], 1))
    dat.append(np.ones(2 * (n - 1)))
    b.append(2.0 * np.ones(l))
    msk.append(np.zeros(l))
    mcount += l
    # partial trace 1
    ci = mcount + np.repeat(np.arange(n - 1), l)
    ca = 1 + np.tile(np.arange(l)[:, None, None] + l * np.arange(l)[None, None, :],
                     (1, l, 1)).reshape(-1)
    cb = 1 + np.tile(np.arange(l)[None, :, None] + l * np.arange(l)[None, None, :],
                     (l, 1, 1)).reshape(-1)
    idx.append(np.stack([ci, ca, cb], 1))
    idx.append(np.stack([ci, cb, ca], 1))
    dat.append(np.ones(2 * ca.size))
    b.append(2.0 * (ca == cb).reshape(l ** 2, l).T[0].astype(float))
    msk.append(np.zeros(n - 1))
    mcount += n - 1
    # partial trace 2
    ci = mcount + np.repeat(np.arange(n - 1), l)
    ca = 1 + np.tile(l * np.arange(l)[:, None, None] + np.arange(l)[None, None, :],
                     (1, l, 1)).reshape(-1)
    cb = 1 + np.tile(l * np.arange(l)[None, :, None] + np.arange(l)[None, None, :],
                     (l, 1, 1)).reshape(-1)
    idx.append(np.stack([ci, ca, cb], 1))
    idx.append(np.stack([ci, cb, ca], 1))
    dat.append(np.ones(2 * ca.size))
    b.append(2.0 * (ca == cb).reshape(l ** 2, l).T[0].astype(float))
    msk.append(np.zeros(n - 1))
    mcount += n - 1
    # Y >= 0 on the objective's upper triangle
    tri = C_rows <= C_cols
    nt = int(tri.sum())
    ci = mcount + np.arange(nt)
    trip = np.stack([ci, C_rows[tri], C_cols[tri]], 1)
    trip = np.concatenate([trip, trip[:, [0, 2, 1]]], 0)
    idx.append(trip)
    dat.append(np.full(trip.shape[0], -0.5))
    b.append(np.zeros(nt))
    msk.append(np.ones(nt))
    return (np.concatenate(dat), np.concatenate(idx).astype(np.int64), np.concatenate(b),
            np.concatenate(msk))


def _unscaled_problem(D, W):
    """C (= -W (x) D lifted), the constraints and the scales
    (utils/qap_helpers.py:321-370)."""
    r, c, v, N = build_objective_matrix(D, W)
    v = -v
    C = sp.csr_matrix((v, (r, c)), shape=(N, N))
    A_data, A_indices, b, mask = get_all_problem_data(r, c, N)
    n, m = N, b.shape[0]
    l = int(np.sqrt(n - 1))
    SCALE_X = 1.0 / float(l + 1)
    SCALE_C = 1.0 / np.linalg.norm(v)
    SCALE_A = 1.0 / np.sqrt(np.bincount(A_indices[:, 0], weights=A_data ** 2, minlength=m))
    A_mat = sp.coo_matrix((SCALE_A[A_indices[:, 0]] * A_data,
                           (A_indices[:, 0], A_indices[:, 1] * n + A_indices[:, 2])),
                          shape=(m, n * n)).tocsr()
    norm_A = np.sqrt(eigsh(A_mat @ A_mat.T, k=1, which="LM", return_eigenvectors=False,
                           maxiter=np.iinfo(np.int32).max)[0])
    SCALE_A = SCALE_A / norm_A
    return C, A_data, A_indices, b, mask, SCALE_C, SCALE_X, SCALE_A


def initialize_state(D, W, sketch_dim, Omega=None):
    C, A_data, A_indices, b, mask, SCALE_C, SCALE_X, SCALE_A = _unscaled_problem(D, W)
    n, m = C.shape[0], b.shape[0]
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
                  SCALE_C=SCALE_C, SCALE_X=SCALE_X, SCALE_A=SCALE_A)
    return scale_sdp_state(st)


def qap_round(P, Omega, callback_static_args, callback_nonstatic_args):
    """The QAP rounding callback (utils/qap_helpers.py:624-653): for every
    column of the reconstructed E (and its negative), an optimal assignment on
    the l x l cost max(c) - c with c = +-E[1:, i] reshaped row-major (row =
    facility, column = location), scored by trace(W P D P^T); returns the
    smaller of the two minima.  The reference's assignment solver is its own
    Munkres (utils/munkres.py:13-120); this restatement uses SciPy's
    linear_sum_assignment, which returns the same assignment whenever the
    optimum is unique (costs from a reconstructed sketch have no ties)."""
    import pickle
    from scipy.optimize import linear_sum_assignment
    from .common import reconstruct_from_sketch
    static = callback_static_args
    l = int(pickle.loads(static)["l"]) if isinstance(static, (bytes, bytearray)) else int(static)
    D = np.asarray(callback_nonstatic_args["D"], float)
    W = np.asarray(callback_nonstatic_args["W"], float)
    E, _ = reconstruct_from_sketch(np.asarray(Omega, float), np.asarray(P, float))
    if not np.all(np.isfinite(E)):
        return float("nan")

    def score(c):
        c = c.reshape(l, l)
        r, col = linear_sum_assignment(c.max() - c)
        perm = np.zeros((l, l))
        perm[r, col] = 1.0
        return float(np.trace(W @ perm @ D @ perm.T))

    cols = E.shape[1]
    min_pos = min(score(E[1:, i]) for i in range(min(l, cols)))
    min_neg = min(score(-E[1:, i]) for i in range(min(l, cols)))
    return min_pos if min_pos < min_neg else min_neg


# ---- warm starts (utils/qap_helpers.py:384-621) ----

def _index_map(a, l, num_drop):
    """utils/qap_helpers.py:412: a + num_drop * max((a - 1) // old_l, 0)."""
    a = np.asarray(a, np.int64)
    return a + num_drop * np.clip((a - 1) // (l - num_drop), 0, None)


def _fill_constraint_index_map(old_A_indices, new_A_indices, old_m):
    """utils/qap_helpers.py:384-392, stopping at the last old triple; old
    constraints never matched keep -1 (the reference leaves them unset)."""
    cmap = np.full(old_m, -1, np.int64)
    old_idx = 0
    for curr_idx in range(new_A_indices.shape[0]):
        if old_idx >= old_A_indices.shape[0]:
            break
        old_row, curr_row = old_A_indices[old_idx], new_A_indices[curr_idx]
        if curr_row[1] == old_row[1] and curr_row[2] == old_row[2]:
            cmap[old_row[0]] = curr_row[0]
            old_idx += 1
    return cmap


def _warm_common(old, D, W, sketch_dim):
    from .common import unscale_sdp_state
    old = unscale_sdp_state(old)
    prob = _unscaled_problem(np.asarray(D, float), np.asarray(W, float))
    C, A_data, A_indices, b = prob[:4]
    n, m = C.shape[0], b.shape[0]
    old_l = int(np.sqrt(old.C.shape[0] - 1))
    l = int(np.sqrt(n - 1))
    num_drop = l - old_l
    assert sketch_dim in (-1, l)
    old_idx = np.asarray(old.A_indices, np.int64).copy()
    old_idx[:, 1:] = _index_map(old_idx[:, 1:], l, num_drop)
    cmap = _fill_constraint_index_map(old_idx, A_indices, old.b.shape[0])

    def carry(v):
        out = np.zeros(m)
        ok = cmap >= 0
        out[cmap[ok]] = np.asarray(v)[ok]
        return out
    return old, prob, n, m, l, num_drop, carry


def _warm_state(prob, X, P, Om, y, z, tr_X, primal_obj):
    C, A_data, A_indices, b, mask, SCALE_C, SCALE_X, SCALE_A = prob
    return scale_sdp_state(SDPState(C=C, A_indices=A_indices, A_data=A_data, b=b,
                                    b_ineq_mask=mask, X=X, P=P, Omega=Om, y=y, z=z, tr_X=tr_X,
                                    primal_obj=primal_obj, SCALE_C=SCALE_C, SCALE_X=SCALE_X,
                                    SCALE_A=SCALE_A))


def get_implicit_warm_start_state(old, D, W, sketch_dim):
    """utils/qap_helpers.py:395-467 (PRNGKey(n) -> hash_normal_matrix key n)."""
    old, prob, n, m, l, num_drop, carry = _warm_common(old, D, W, sketch_dim)
    X, Om, P = old.X, old.Omega, old.P
    if old.X is not None:
        r, c = np.nonzero(old.X)
        X = np.zeros((n, n))
        X[_index_map(r, l, num_drop), _index_map(c, l, num_drop)] = old.X[r, c]
    if old.P is not None:
        rows = _index_map(np.arange(old.Omega.shape[0]), l, num_drop)
        Om = hash_normal_matrix(n, n, l)
        Om[rows] = old.Omega
        P = np.zeros_like(Om)
        P[rows] = old.P
    return _warm_state(prob, X, P, Om, carry(old.y), carry(old.z), old.tr_X, old.primal_obj)


def get_explicit_warm_start_state(old, D, W, sketch_dim):
    """utils/qap_helpers.py:469-553."""
    from .common import apply_A_operator_mx, reconstruct_from_sketch
    from .operators import apply_A_operator_batched
    old, prob, n, m, l, num_drop, carry = _warm_common(old, D, W, sketch_dim)
    C, A_data, A_indices = prob[:3]
    X, Om, P = old.X, old.Omega, old.P
    if old.X is not None:
        r, c = np.nonzero(old.X)
        X = np.zeros((n, n))
        X[_index_map(r, l, num_drop), _index_map(c, l, num_drop)] = old.X[r, c]
        z = apply_A_operator_mx(n, m, A_data, A_indices, X)
        tr_X = float(np.trace(X))
        primal_obj = float((C @ X).trace())
    if old.P is not None:
        Om = hash_normal_matrix(n, n, sketch_dim)
        E, Lam = reconstruct_from_sketch(old.Omega, old.P)
        tr_offset = (old.tr_X - np.sum(Lam)) / Lam.shape[0]
        Lam_c = Lam + tr_offset
        Ep = np.zeros_like(Om)
        Ep[_index_map(np.arange(E.shape[0]), l, num_drop)] = E
        with np.errstate(invalid="ignore"):
            S = Ep * np.sqrt(Lam_c)[None, :]
        P = S @ (S.T @ Om)
        z = apply_A_operator_batched(m, A_data, A_indices, S)
        tr_X = float(np.sum(Lam_c))
        primal_obj = float(np.trace(S.T @ (C @ S)))
    return _warm_state(prob, X, P, Om, carry(old.y), z, tr_X, primal_obj)


def get_dual_only_warm_start_state(old, D, W, sketch_dim):
    """utils/qap_helpers.py:556-621 (PRNGKey(0) -> key 1, as in the cold start)."""
    old, prob, n, m, l, num_drop, carry = _warm_common(old, D, W, sketch_dim)
    if sketch_dim == -1:
        X, Om, P = np.zeros((n, n)), None, None
    elif sketch_dim > 0:
        X = None
        Om = hash_normal_matrix(1, n, sketch_dim)
        P = np.zeros_like(Om)
    else:
        raise ValueError("Invalid value for sketch_dim")
    return _warm_state(prob, X, P, Om, carry(old.y), np.zeros(m), 0.0, 0.0)
