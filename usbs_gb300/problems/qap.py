"""QAP SDP relaxation instances (reference: utils/qap_helpers.py:157-381).

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


def initialize_state(D, W, sketch_dim, Omega=None):
    """Scaled cold-start state of the QAP relaxation (utils/qap_helpers.py:321-381)."""
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
    lam = eigsh(A_mat @ A_mat.T, k=1, which="LM", return_eigenvectors=False,
                maxiter=np.iinfo(np.int32).max)[0]
    sa = sa / np.sqrt(lam)
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
