"""SDP state container and scaling (reference: utils/common.py:11-96).

``C`` is a SciPy sparse matrix on the host; the iterate fields (X, P, y, z) may
be NumPy arrays or CUDA torch tensors.  Scaling runs on the host at set-up, as
in the reference.
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


def scale_sdp_state(s):
    """utils/common.py:29-61."""
    SA = _np(s.SCALE_A)
    return s._replace(
        C=(s.C * s.SCALE_C).tocsr(),
        A_data=_np(s.A_data) * SA[_np(s.A_indices)[:, 0]],
        b=_np(s.b) * s.SCALE_X * SA,
        X=None if s.X is None else _np(s.X) * s.SCALE_X,
        P=None if s.P is None else _np(s.P) * s.SCALE_X,
        z=_np(s.z) * SA * s.SCALE_X,
        tr_X=s.tr_X * s.SCALE_X,
        primal_obj=s.primal_obj * s.SCALE_X * s.SCALE_C)


def unscale_sdp_state(s):
    """utils/common.py:64-96."""
    SA = _np(s.SCALE_A)
    return s._replace(
        C=(s.C / s.SCALE_C).tocsr(),
        A_data=_np(s.A_data) / SA[_np(s.A_indices)[:, 0]],
        b=(_np(s.b) / SA) / s.SCALE_X,
        X=None if s.X is None else _np(s.X) / s.SCALE_X,
        P=None if s.P is None else _np(s.P) / s.SCALE_X,
        z=(_np(s.z) / SA) / s.SCALE_X,
        tr_X=s.tr_X / s.SCALE_X,
        primal_obj=s.primal_obj / (s.SCALE_X * s.SCALE_C))
