"""Problem-data callbacks A(.), A*(.) and the svec/Q-base helpers (oracle, FP64).

Restates ``solver/utils.py:11-65``.  ``A_indices`` rows are (constraint, i, j)
triples and ``A_data`` their values, exactly as in the reference.  Scatter-adds
use ``np.bincount`` (sums in triple order).
"""
import numpy as np


def apply_A_operator_slim(m, A_data, A_indices, u):
    """A(u u^T): out[c] += a_t u[i_t] u[j_t]   (solver/utils.py:11-16)."""
    w = A_data * u[A_indices[:, 1]] * u[A_indices[:, 2]]
    return np.bincount(A_indices[:, 0], weights=w, minlength=m).astype(np.float64)


def apply_A_adjoint_slim(n, A_data, A_indices, z, u):
    """A*(z) u: out[i_t] += a_t z[c_t] u[j_t]   (solver/utils.py:19-24)."""
    w = A_data * z[A_indices[:, 0]] * u[A_indices[:, 2]]
    return np.bincount(A_indices[:, 1], weights=w, minlength=n).astype(np.float64)


def apply_A_operator_batched(m, A_data, A_indices, vecs):
    """sum_j A(v_j v_j^T) over the columns of vecs   (solver/utils.py:27-31)."""
    prod = np.einsum("tj,tj->t", vecs[A_indices[:, 1]], vecs[A_indices[:, 2]])
    return np.bincount(A_indices[:, 0], weights=A_data * prod, minlength=m).astype(np.float64)


def apply_A_adjoint_batched(n, A_data, A_indices, z, vecs):
    """[A*(z) v_j]_j for every column of vecs   (solver/utils.py:34-37)."""
    coef = A_data * z[A_indices[:, 0]]
    out = np.empty((n, vecs.shape[1]))
    for j in range(vecs.shape[1]):
        out[:, j] = np.bincount(A_indices[:, 1], weights=coef * vecs[A_indices[:, 2], j],
                                minlength=n)
    return out


def create_svec_matrix(k):
    """Dense svec isometry U (s x k^2), s = k(k+1)/2   (solver/utils.py:40-50).

    Row a follows np.tril_indices(k) order; diagonal entries map with weight 1,
    off-diagonal pairs with 1/sqrt(2) on both (b,c) and (c,b)."""
    s = k * (k + 1) // 2
    U = np.zeros((s, k * k))
    for a, (b, c) in enumerate(zip(*np.tril_indices(k))):
        if b == c:
            U[a, b * k + c] = 1.0
        else:
            U[a, b * k + c] = 1.0 / np.sqrt(2.0)
            U[a, c * k + b] = U[a, b * k + c]
    return U


def svec(U, M):
    return U @ M.reshape(-1)


def svec_inv(U, v, k):
    return (U.T @ v).reshape(k, k)


def create_Q_base(m, k, U, A_data, A_indices, V):
    """sum_c svec(B_c) svec(B_c)^T with B_c = sum_{t in c} a_t V[i_t] V[j_t]^T
    (solver/utils.py:53-65).  Computed per svec coordinate instead of through the
    m x k x k tensor (same sums, far less memory)."""
    rows, cols = np.tril_indices(k)
    Vi = V[A_indices[:, 1]]
    Vj = V[A_indices[:, 2]]
    s = len(rows)
    proj = np.empty((s, m))
    for a in range(s):
        b, c = rows[a], cols[a]
        if b == c:
            w = A_data * Vi[:, b] * Vj[:, b]
        else:
            w = A_data * (Vi[:, b] * Vj[:, c] + Vi[:, c] * Vj[:, b]) / np.sqrt(2.0)
        proj[a] = np.bincount(A_indices[:, 0], weights=w, minlength=m)
    return proj @ proj.T


def adjoint_gram(A_data, A_indices, z, V):
    """V^T A*(z) V  (the projection used at solver/usbs.py:56,58,219)."""
    coef = A_data * z[A_indices[:, 0]]
    return (V[A_indices[:, 1]] * coef[:, None]).T @ V[A_indices[:, 2]]
