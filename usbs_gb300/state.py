"""SDP state container and scaling (reference: utils/common.py:11-96).

``C`` is a SciPy sparse matrix on the host; the iterate fields (X, P, y, z) may
be NumPy arrays or CUDA torch tensors.  Scaling runs at set-up, as in the
reference: problem data on the host, device iterates on their device.
"""
from collections import namedtuple

import numpy as np

SDPState = namedtuple("SDPState", ["C", "A_indices", "A_data", "b", "b_ineq_mask", "X", "P",
                                   "Omega", "y", "z", "tr_X", "primal_obj", "SCALE_C",
                                   "SCALE_X", "SCALE_A"])


def _np(x):
    if x is None:
        return None
    if hasattr(x, "detach"):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def _scaled(x, f, SA=None, divide=False):
    """x * f (x / f with divide), elementwise times SA (over SA) if given.  A
    device tensor stays on its device; anything else becomes NumPy."""
    if x is None:
        return None
    if hasattr(x, "detach"):
        import torch
        out = x / f if divide else x * f
        if SA is not None:
            sa = torch.as_tensor(SA, dtype=x.dtype, device=x.device)
            out = out / sa if divide else out * sa
        return out
    out = _np(x) / f if divide else _np(x) * f
    if SA is not None:
        out = out / SA if divide else out * SA
    return out


def scale_sdp_state(s):
    """utils/common.py:29-61 (device iterates are scaled on their device)."""
    SA = _np(s.SCALE_A)
    return s._replace(
        C=(s.C * s.SCALE_C).tocsr(),
        A_data=_np(s.A_data) * SA[_np(s.A_indices)[:, 0]],
        b=_np(s.b) * s.SCALE_X * SA,
        X=_scaled(s.X, s.SCALE_X),
        P=_scaled(s.P, s.SCALE_X),
        z=_scaled(s.z, s.SCALE_X, SA),
        tr_X=s.tr_X * s.SCALE_X,
        primal_obj=s.primal_obj * s.SCALE_X * s.SCALE_C)


def unscale_sdp_state(s):
    """utils/common.py:64-96 (device iterates are unscaled on their device)."""
    SA = _np(s.SCALE_A)
    return s._replace(
        C=(s.C / s.SCALE_C).tocsr(),
        A_data=_np(s.A_data) / SA[_np(s.A_indices)[:, 0]],
        b=(_np(s.b) / SA) / s.SCALE_X,
        X=_scaled(s.X, s.SCALE_X, divide=True),
        P=_scaled(s.P, s.SCALE_X, divide=True),
        z=_scaled(s.z, s.SCALE_X, SA, divide=True),
        tr_X=s.tr_X / s.SCALE_X,
        primal_obj=s.primal_obj / (s.SCALE_X * s.SCALE_C))
