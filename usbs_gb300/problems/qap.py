"""QAP SDP relaxation instances (reference: utils/qap_helpers.py:157-381) and
their warm starts (implicit, explicit, dual-only: utils/qap_helpers.py:384-621).

The lifted variable Y is (l^2 + 1) x (l^2 + 1): row/column 0 is the homogenising
coordinate and index 1 + i + l j stands for "facility j at location i".  The
objective is the Kronecker product of the flow matrix W and the distance matrix
D, shifted by one (qap_helpers.py:157-172), and negated for minimisation.  The
constraints are grouped into families (qap_helpers.py:175-318):

* Y_00 = 1;
* the arrow constraints diag(Y) = Y_0. (2 Y_0j - Y_0j - Y_j0 = 0 written as three
  triples);
* row sums and column sums of the assignment (b = 2 with both triangles);
* the two partial traces (b = 2 on the diagonal blocks);
* Y >= 0 on the objective's upper-triangle pattern, as "<=" rows with -1/2 on
  both (i, j) and (j, i).

Scaling (qap_helpers.py:321-381): SCALE_X = 1/(l+1), SCALE_C = 1/||C||_F, and
SCALE_A = 1/row-norm divided by the spectral norm of the row-normalised
constraint matrix (ARPACK, as the reference does).  Set-up runs on the host.
"""
import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import eigsh

from ..arrays import to_host
from ..rng import hash_normal_matrix
from ..state import SDPState, scale_sdp_state


def objective_pattern(D, W):
    """(rows, cols, values, N) of the lifted objective W (x) D shifted by one."""
    l = D.shape[0]
    dr, dc = np.nonzero(D)
    wr, wc = np.nonzero(W)
    rows = 1 + (dr[None, :] + l * wr[:, None]).ravel()
    cols = 1 + (dc[None, :] + l * wc[:, None]).ravel()
    vals = (W[wr, wc][:, None] * D[dr, dc][None, :]).ravel()
    return rows.astype(np.int64), cols.astype(np.int64), vals, l * l + 1


def _family(first, con, i, j, a, b, mask):
    """Triples of one constraint family with constraint ids offset by `first`."""
    con = np.asarray(con, np.int64) + first
    trip = np.stack([con, np.asarray(i, np.int64), np.asarray(j, np.int64)], 1)
    return trip, np.asarray(a, float), np.asarray(b, float), np.asarray(mask, float)


def constraints(C_rows, C_cols, N):
    """(A_data, A_indices, b, b_ineq_mask) of the QAP relaxation."""
    l = int(round(np.sqrt(N - 1)))
    L2 = l * l
    fams = []
    m0 = 0

    def add(count, con, i, j, a, b, mask):
        nonlocal m0
        fams.append(_family(m0, con, i, j, a, b, mask))
        m0 += count

    # Y_00 = 1
    add(1, [0], [0], [0], [1.0], [1.0], [0.0])
    # arrow: 2 Y_jj - Y_0j - Y_j0 = 0, j = 1..L2 (one constraint per j, three triples)
    j = np.arange(1, L2 + 1)
    con = np.repeat(np.arange(L2), 3)
    ii = np.stack([j, np.zeros_like(j), j], 1).ravel()
    jj = np.stack([np.zeros_like(j), j, j], 1).ravel()
    add(L2, con, ii, jj, np.tile([-1.0, -1.0, 2.0], L2), np.zeros(L2), np.zeros(L2))
    # row sums (facility j over locations) and column sums, both triangles of row 0
    grid = 1 + np.arange(L2).reshape(l, l)          # grid[j, i] = 1 + i + l j
    for lines in (grid, grid.T):
        con = np.repeat(np.arange(l), 2 * l)
        members = lines.reshape(-1)
        ii = np.stack([members, np.zeros_like(members)], 1).ravel()
        jj = np.stack([np.zeros_like(members), members], 1).ravel()
        add(l, con, ii, jj, np.ones(2 * L2), 2.0 * np.ones(l), np.zeros(l))
    # partial traces: sum over the block index of Y[(a, p), (b, p)], both orders
    for first_major in (True, False):
        con, ii, jj, bb = [], [], [], []
        for a in range(l):
            for b in range(l):
                c = a * l + b
                p = np.arange(l)
                if first_major:
                    ra, rb = 1 + a + l * p, 1 + b + l * p
                else:
                    ra, rb = 1 + l * a + p, 1 + l * b + p
                con += [c] * (2 * l)
                ii += list(ra) + list(rb)
                jj += list(rb) + list(ra)
                bb.append(2.0 if a == b else 0.0)
        add(L2, con, ii, jj, np.ones(len(con)), bb, np.zeros(L2))
    # Y >= 0 on the objective's upper triangle: -Y_ij / 2 - Y_ji / 2 <= 0
    up = C_rows <= C_cols
    r, c = C_rows[up], C_cols[up]
    nt = r.size
    con = np.concatenate([np.arange(nt), np.arange(nt)])
    add(nt, con, np.concatenate([r, c]), np.concatenate([c, r]), np.full(2 * nt, -0.5),
        np.zeros(nt), np.ones(nt))
    trip = np.concatenate([f[0] for f in fams])
    return (np.concatenate([f[1] for f in fams]), trip, np.concatenate([f[2] for f in fams]),
            np.concatenate([f[3] for f in fams]))


def _problem(D, W):
    """(C, A_data, A_indices, b, mask, SCALE_C, SCALE_X, SCALE_A) of the
    relaxation, unscaled (utils/qap_helpers.py:321-370)."""
    D = np.asarray(D, float)
    W = np.asarray(W, float)
    r, c, v, N = objective_pattern(D, W)
    C = sp.csr_matrix((-v, (r, c)), shape=(N, N))
    A_data, A_idx, b, mask = constraints(r, c, N)
    m = b.shape[0]
    l = int(round(np.sqrt(N - 1)))
    scale_x = 1.0 / float(l + 1)
    scale_c = 1.0 / np.linalg.norm(v)
    rownorm = np.sqrt(np.bincount(A_idx[:, 0], weights=A_data ** 2, minlength=m))
    sa = 1.0 / rownorm
    A_mat = sp.csr_matrix((sa[A_idx[:, 0]] * A_data, (A_idx[:, 0], A_idx[:, 1] * N + A_idx[:, 2])),
                          shape=(m, N * N))
    # ||A||_2^2 by ARPACK as in the reference, from a fixed start vector: the
    # default random start makes the scaling, and with it every later bit of
    # the solve, differ between processes
    AAt = A_mat @ A_mat.T
    lam = eigsh(AAt, k=1, which="LM", return_eigenvectors=False, v0=np.ones(AAt.shape[0]),
                maxiter=np.iinfo(np.int32).max)[0]
    return C, A_data, A_idx, b, mask, scale_c, scale_x, sa / np.sqrt(lam)


def initialize_state(D, W, sketch_dim, Omega=None):
    """Scaled cold-start state of the QAP relaxation (utils/qap_helpers.py:321-381)."""
    C, A_data, A_idx, b, mask, scale_c, scale_x, sa = _problem(D, W)
    N, m = C.shape[0], b.shape[0]
    if sketch_dim == -1:
        X, P, Om = np.zeros((N, N)), None, None
    elif sketch_dim > 0:
        Om = hash_normal_matrix(1, N, sketch_dim) if Omega is None else np.asarray(Omega, float)
        X, P = None, np.zeros_like(Om)
    else:
        raise ValueError("Invalid value for sketch_dim")
    st = SDPState(C=C, A_indices=A_idx, A_data=A_data, b=b, b_ineq_mask=mask, X=X, P=P,
                  Omega=Om, y=np.zeros(m), z=np.zeros(m), tr_X=0.0, primal_obj=0.0,
                  SCALE_C=scale_c, SCALE_X=scale_x, SCALE_A=sa)
    return scale_sdp_state(st)


# ---------------------------------------------------------------- warm starts
# A solved instance with old_l facilities warm-starts one with l = old_l +
# num_drop (utils/qap_helpers.py:395-621): lifted index a = 1 + loc + old_l fac
# moves to a + num_drop * fac, and each old constraint to the new constraint
# whose triples its own match, found by walking both triple lists in order
# (utils/qap_helpers.py:384-392), here in (constraint, i, j) order.  The walk
# stops at the last old triple, and old constraints it never matches keep no
# dual (the reference leaves those map entries uninitialised).

def _host(x):
    return np.asarray(to_host(x), float)


def _index_map(a, l, num_drop):
    a = np.asarray(a, np.int64)
    return a + num_drop * np.clip((a - 1) // (l - num_drop), 0, None)


def _constraint_map(old_idx, new_idx, old_m):
    # both lists in (constraint, i, j) order: on the reference's listing this
    # gives its map, and it does not depend on how a state lists its triples
    old_idx = old_idx[np.lexsort((old_idx[:, 2], old_idx[:, 1], old_idx[:, 0]))]
    new_idx = np.asarray(new_idx)
    new_idx = new_idx[np.lexsort((new_idx[:, 2], new_idx[:, 1], new_idx[:, 0]))]
    cmap = np.full(old_m, -1, np.int64)
    o = 0
    for cur in range(new_idx.shape[0]):
        if o >= old_idx.shape[0]:
            break
        if new_idx[cur, 1] == old_idx[o, 1] and new_idx[cur, 2] == old_idx[o, 2]:
            cmap[old_idx[o, 0]] = new_idx[cur, 0]
            o += 1
    return cmap


def _carry(old, D, W, sketch_dim):
    # the QAP transforms move rows through the lifted index map on the host
    old = old._replace(y=_host(old.y), z=_host(old.z),
                       P=None if old.P is None else _host(old.P),
                       X=None if old.X is None else _host(old.X))
    from ..state import unscale_sdp_state
    old = unscale_sdp_state(old)
    C, A_data, A_idx, b, mask, scale_c, scale_x, sa = _problem(D, W)
    n, m = C.shape[0], b.shape[0]
    old_l = int(round(np.sqrt(old.C.shape[0] - 1)))
    l = int(round(np.sqrt(n - 1)))
    if sketch_dim not in (-1, l):
        raise ValueError(f"sketch_dim must be -1 or l = {l}")
    num_drop = l - old_l
    oidx = np.asarray(old.A_indices, np.int64).copy()
    oidx[:, 1:] = _index_map(oidx[:, 1:], l, num_drop)
    cmap = _constraint_map(oidx, A_idx, np.asarray(old.b).shape[0])
    keep = cmap >= 0

    def dual(v):
        out = np.zeros(m)
        out[cmap[keep]] = np.asarray(v, float)[keep]
        return out
    return old, (C, A_data, A_idx, b, mask, scale_c, scale_x, sa), l, num_drop, dual


def _state(prob, X, P, Om, y, z, tr_X, primal):
    C, A_data, A_idx, b, mask, scale_c, scale_x, sa = prob
    return scale_sdp_state(SDPState(C=C, A_indices=A_idx, A_data=A_data, b=b, b_ineq_mask=mask,
                                    X=X, P=P, Omega=Om, y=y, z=z, tr_X=tr_X, primal_obj=primal,
                                    SCALE_C=scale_c, SCALE_X=scale_x, SCALE_A=sa))


def implicit_warm_start(old, D, W, sketch_dim):
    """utils/qap_helpers.py:395-467: X, P and Omega's rows moved to the new
    lifted indices (new rows of Omega drawn fresh, key n), y and z carried by
    the constraint map, tr_X and primal_obj kept."""
    old, prob, l, num_drop, dual = _carry(old, D, W, sketch_dim)
    n = prob[0].shape[0]
    X, P, Om = None, None, None
    if old.X is not None:
        Xo = np.asarray(old.X, float)
        r, c = np.nonzero(Xo)
        X = np.zeros((n, n))
        X[_index_map(r, l, num_drop), _index_map(c, l, num_drop)] = Xo[r, c]
    if old.P is not None:
        rows = _index_map(np.arange(np.asarray(old.P).shape[0]), l, num_drop)
        Om = hash_normal_matrix(n, n, sketch_dim)
        Om[rows] = _host(old.Omega)
        P = np.zeros_like(Om)
        P[rows] = np.asarray(old.P, float)
    return _state(prob, X, P, Om, dual(old.y), dual(old.z), old.tr_X, old.primal_obj)


def explicit_warm_start(old, D, W, sketch_dim, device="cuda"):
    """utils/qap_helpers.py:469-553: the old iterate made explicit (dense X
    moved to the new indices, or the sketch's Nystrom factors reconstructed on
    the device, trace-corrected, moved and re-sketched by a fresh Omega, key
    n); z, tr_X and primal_obj recomputed; y carried by the constraint map."""
    old, prob, l, num_drop, dual = _carry(old, D, W, sketch_dim)
    C, A_data, A_idx = prob[0], prob[1], prob[2]
    n, m = C.shape[0], prob[3].shape[0]
    X, P, Om = None, None, None
    if old.X is not None:
        Xo = np.asarray(old.X, float)
        r, c = np.nonzero(Xo)
        X = np.zeros((n, n))
        X[_index_map(r, l, num_drop), _index_map(c, l, num_drop)] = Xo[r, c]
        z = np.bincount(A_idx[:, 0], weights=A_data * X[A_idx[:, 1], A_idx[:, 2]], minlength=m)
        tr_X = float(np.trace(X))
        primal = float((C @ X).trace())
    if old.P is not None:
        from ..rounding import reconstruct_from_sketch
        Om = hash_normal_matrix(n, n, sketch_dim)
        E, lam = reconstruct_from_sketch(_host(old.Omega), np.asarray(old.P, float), device=device)
        E, lam = E.cpu().numpy(), lam.cpu().numpy()
        lam_c = lam + (old.tr_X - lam.sum()) / lam.shape[0]
        S = np.zeros((n, E.shape[1]))
        with np.errstate(invalid="ignore"):
            S[_index_map(np.arange(E.shape[0]), l, num_drop)] = E * np.sqrt(lam_c)[None, :]
        P = S @ (S.T @ Om)
        prod = np.einsum("tj,tj->t", S[A_idx[:, 1]], S[A_idx[:, 2]])
        z = np.bincount(A_idx[:, 0], weights=A_data * prod, minlength=m)
        tr_X = float(lam_c.sum())
        primal = float(np.einsum("ij,ij->", S, C @ S))
    return _state(prob, X, P, Om, dual(old.y), z, tr_X, primal)


def dual_only_warm_start(old, D, W, sketch_dim):
    """utils/qap_helpers.py:556-621: only y, carried by the constraint map; a
    cold iterate (Omega as the cold start draws it)."""
    old, prob, l, num_drop, dual = _carry(old, D, W, sketch_dim)
    n, m = prob[0].shape[0], prob[3].shape[0]
    if sketch_dim == -1:
        X, P, Om = np.zeros((n, n)), None, None
    else:
        Om = hash_normal_matrix(1, n, sketch_dim)
        X, P = None, np.zeros_like(Om)
    return _state(prob, X, P, Om, dual(old.y), np.zeros(m), 0.0, 0.0)
