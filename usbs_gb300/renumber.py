"""Node renumbering of an SDP instance for locality on the device.

The USBS iteration is invariant under a simultaneous permutation of the rows
and columns of X: solving the problem with C -> P^T C P, the triples' (i, j)
renumbered, and the rows of P, Omega, X and the Lanczos start vector permuted
gives the permuted iterates (the constraint-space vectors y, z, b are untouched),
equal up to the order of floating-point sums.  A reverse Cuthill-McKee order of
the operator's pattern (C and the triples' positions) puts each row's entries
near the diagonal: the Lanczos operator's gathers of x, random over all of HBM
and L2 in a random node order, then fall in a narrow band, so they reuse L1
and L2 lines.  The permutation is computed once per problem on the host
(SciPy's reverse_cuthill_mckee); there is no counterpart in the reference.

``perm[r]`` is the original index of row r of the renumbered problem.
"""
import numpy as np
import scipy.sparse as sp
from scipy.sparse.csgraph import reverse_cuthill_mckee

from .arrays import to_host


def _host(x):
    return np.asarray(to_host(x))


def rcm_permutation(C, A_indices, n):
    """RCM order of the symmetrised pattern of C and the triples' (i, j)."""
    C = sp.csr_matrix(C)
    idx = np.asarray(A_indices)
    T = sp.csr_matrix((np.ones(idx.shape[0]), (idx[:, 1], idx[:, 2])), shape=(n, n))
    pat = (abs(C) + T).tocsr()
    pat = (pat + pat.T).tocsr()
    pat.data[:] = 1.0
    return np.asarray(reverse_cuthill_mckee(pat, symmetric_mode=True), dtype=np.int64)


def inverse(perm):
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.shape[0])
    return inv


def permute_problem(C, A_indices, perm):
    """(P^T C P, triples with (i, j) renumbered) for perm (new -> old)."""
    inv = inverse(perm)
    Cp = sp.csr_matrix(C)[perm][:, perm].tocsr()
    Cp.sort_indices()
    idx = np.array(A_indices, dtype=np.int64, copy=True)
    idx[:, 1] = inv[idx[:, 1]]
    idx[:, 2] = inv[idx[:, 2]]
    return Cp, idx


def permute_state(st, perm):
    """The SDPState of the renumbered problem (rows of X, P, Omega permuted)."""
    Cp, idx = permute_problem(st.C, st.A_indices, perm)
    X = None if st.X is None else _host(st.X)[perm][:, perm]
    P = None if st.P is None else _host(st.P)[perm]
    Om = None if st.Omega is None else _host(st.Omega)[perm]
    return st._replace(C=Cp, A_indices=idx, X=X, P=P, Omega=Om)


def _take(M, inv, both=False):
    if hasattr(M, "index_select"):
        import torch
        t = torch.as_tensor(inv, device=M.device)
        M = M.index_select(0, t)
        return M.index_select(1, t) if both else M
    M = np.asarray(M)[inv]
    return M[:, inv] if both else M


def unpermute_rows(M, perm):
    """Rows of a renumbered n x ... array (NumPy or torch) in the original order."""
    return _take(M, inverse(perm))


def unpermute_state(st, orig, perm):
    """An output state of the renumbered problem back in the original numbering:
    rows of X, P and Omega (and X's columns) restored, C and the triples taken
    from the original state `orig`."""
    inv = inverse(perm)
    X = None if st.X is None else _take(st.X, inv, both=True)
    P = None if st.P is None else _take(st.P, inv)
    Om = None if st.Omega is None else _take(st.Omega, inv)
    return st._replace(C=orig.C, A_indices=orig.A_indices, X=X, P=P, Omega=Om)
