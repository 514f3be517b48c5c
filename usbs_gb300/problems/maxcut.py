"""MaxCut SDP instances (reference: utils/maxcut_helpers.py:26-92) and their
warm starts (implicit, explicit, dual-only: utils/maxcut_helpers.py:95-289).

maximise <C, X>  s.t.  diag(X) = 1,  tr(X) <= trace_ub,  X PSD,
with C = 1/4 (diag(W 1) - W) symmetrised.  The constraint tensor is the list of
(i, i, i) triples with value 1 and b = 1.  Set-up runs on the host.
"""
import numpy as np
import scipy.sparse as sp

from ..arrays import as_torch, to_device, to_host
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


def _device_of(*xs):
    """The device of the first device tensor among xs, else None (host)."""
    for x in xs:
        t = as_torch(x) if x is not None else None
        if t is not None and t.is_cuda:
            return t.device
    return None


def _padded(x, n, dev):
    """x with zero rows appended to n rows: a float64 tensor on `dev`, or a
    NumPy array when dev is None."""
    if dev is None:
        a = np.asarray(to_host(x), float)
        out = np.zeros((n,) + a.shape[1:])
        out[:a.shape[0]] = a
        return out
    import torch
    t = to_device(x, torch.float64, dev)
    out = torch.zeros((n,) + tuple(t.shape[1:]), dtype=torch.float64, device=dev)
    out[:t.shape[0]] = t
    return out


def implicit_warm_start(old, W, sketch_dim, Omega_pad=None):
    """Grow a solved instance to the graph W (utils/maxcut_helpers.py:95-161):
    pad X / P with zero rows, extend Omega, carry y and z, correct the primal
    objective for the changed diagonal of C, rescale with SCALE_X = 1/n and
    SCALE_C = 1/||C||_F.  When the old iterate is on the device (a finished
    solve's result), the new one is formed there, without a host round trip."""
    dev = _device_of(old.y, old.z, old.P, old.X)
    old = unscale_sdp_state(old)
    C = objective(W)
    n = C.shape[0]
    n_old = old.C.shape[0]
    A_data, A_idx, b, mask = problem_data(n)
    X, P, Om = old.X, old.P, old.Omega
    if old.X is not None:
        if dev is None:
            X = np.zeros((n, n))
            X[:n_old, :n_old] = np.asarray(old.X)
        else:
            import torch
            X = torch.zeros((n, n), dtype=torch.float64, device=dev)
            X[:n_old, :n_old] = to_device(old.X, X.dtype, dev)
    if old.P is not None:
        P = _padded(old.P, n, dev)
        pad = hash_normal_matrix(n, n - n_old, sketch_dim) if Omega_pad is None else Omega_pad
        Om = _padded(old.Omega, n, dev)
        Om[n_old:] = pad if dev is None else to_device(pad, Om.dtype, dev)
    m_old = np.asarray(old.b).shape[0]
    y = _padded(old.y, n, dev)
    z = _padded(old.z, n, dev)
    z_old = z[:m_old]
    dC_old = old.C.diagonal()
    dC = C.diagonal()
    if dev is None:
        corr = -dC_old @ z_old + dC @ z
    else:
        import torch
        corr = float(-(torch.as_tensor(dC_old, device=dev) @ z_old)
                     + torch.as_tensor(dC, device=dev) @ z)
    primal = old.primal_obj + corr
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
    """Keep only the dual y (utils/maxcut_helpers.py:232-289); a device y
    stays on the device."""
    dev = _device_of(old.y)
    old = unscale_sdp_state(old)
    C = objective(W)
    n = C.shape[0]
    A_data, A_idx, b, mask = problem_data(n)
    X, P, Om = _iterate(n, sketch_dim, Omega)
    y = _padded(old.y, n, dev)
    st = SDPState(C=C, A_indices=A_idx, A_data=A_data, b=b, b_ineq_mask=mask, X=X, P=P,
                  Omega=Om, y=y, z=np.zeros(n), tr_X=0.0, primal_obj=0.0,
                  SCALE_C=1.0 / np.linalg.norm(C.data), SCALE_X=1.0 / float(n),
                  SCALE_A=np.ones(n))
    return scale_sdp_state(st)
