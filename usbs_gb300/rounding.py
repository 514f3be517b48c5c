"""Rounding callbacks on the device.

* ``reconstruct_from_sketch(Omega, P, approx_eps)``: utils/common.py:99-116
* ``compute_max_cut(P, Omega, callback_static_args, callback_nonstatic_args)``:
  utils/maxcut_helpers.py:292-302, the reference's rounding callback, with its
  signature, so it plugs into ``usbs_gb300.solver.usbs(callback_fn=...)``.
* ``qap_round(P, Omega, callback_static_args, callback_nonstatic_args)``:
  utils/qap_helpers.py:624-653, the QAP rounding callback (static args: the
  pickled ``{"l": l}``; non-static: ``{"D": D, "W": W}``).

Both run through the C ABI (``usbs_reconstruct_from_sketch``,
``usbs_maxcut_round``): one pass over the sketch for its Gram matrices, the
s x s algebra in FP64 on one warp, one pass for the sign words and one CSR pass
for the cut values.  ``callback_nonstatic_args`` is the unscaled objective C as
the reference passes it (``sdp_state.C / sdp_state.SCALE_C``), a SciPy matrix
(copied to the device once and cached) or a :class:`DeviceCSR`.
"""
import ctypes

import numpy as np
import scipy.sparse as sp

from . import _lib


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("usbs_gb300.rounding needs a CUDA device (GB300); none is visible")
    return torch


class DeviceCSR:
    """A CSR matrix resident on the device (int32 indices, FP64 values)."""

    def __init__(self, C, device="cuda"):
        torch = _torch()
        C = sp.csr_matrix(C, dtype=np.float64)
        C.sum_duplicates()
        self.n = C.shape[0]
        self.rowptr = torch.as_tensor(C.indptr.astype(np.int32), device=device)
        self.col = torch.as_tensor(C.indices.astype(np.int32), device=device)
        self.val = torch.as_tensor(C.data, device=device)


_CSR_CACHE = []          # [(matrix object, DeviceCSR)], most recent last


def _device_csr(C, device):
    if isinstance(C, DeviceCSR):
        return C
    for obj, dc in _CSR_CACHE:
        if obj is C:
            return dc
    dc = DeviceCSR(C, device)
    _CSR_CACHE.append((C, dc))
    del _CSR_CACHE[:-4]
    return dc


def _operands(Omega, P, device):
    """Omega and P (n x s) as FP64 column-major device storage with one leading
    dimension: zero-copy for column views of the solver's sketch buffers."""
    torch = _torch()

    def dev(X):
        t = X if isinstance(X, torch.Tensor) else torch.as_tensor(np.asarray(X, np.float64))
        return t.to(device=device, dtype=torch.float64)

    o, p = dev(Omega), dev(P)
    if o.dim() != 2 or tuple(o.shape) != tuple(p.shape):
        raise ValueError(f"Omega {tuple(o.shape)} and P {tuple(p.shape)} must be equal n x s")
    n, s = o.shape
    if not (o.stride(0) == 1 and p.stride(0) == 1 and o.stride(1) == p.stride(1) >= n):
        o = o.t().contiguous().t()
        p = p.t().contiguous().t()
    return o, p, n, s, o.stride(1) if s > 1 else max(n, 1)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def reconstruct_from_sketch(Omega, P, approx_eps=1e-6, device=None):
    """(E, Lambda): E (n x s) and Lambda (s) as CUDA tensors, in the
    reference's column order (Rho descending); each column of E is fixed up to
    its sign, as an SVD's is."""
    torch = _torch()
    dev = torch.device(device) if device is not None else (
        P.device if isinstance(P, torch.Tensor) and P.is_cuda else torch.device("cuda"))
    o, p, n, s, ld = _operands(Omega, P, dev)
    lib = _lib.load()
    wsb = int(lib.usbs_round_workspace_bytes(n, s))
    if wsb == 0:
        raise ValueError(f"reconstruct_from_sketch: unsupported sizes n={n} s={s} (s <= 32)")
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    Et = torch.empty((s, n), dtype=torch.float64, device=dev)
    lam = torch.empty(s, dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    rc = lib.usbs_reconstruct_from_sketch(n, s, _ptr(o), _ptr(p), ld, float(approx_eps),
                                          _ptr(Et), n, _ptr(lam), _ptr(ws), wsb,
                                          ctypes.c_void_p(st))
    _lib.check(rc, "usbs_reconstruct_from_sketch")
    return Et.t(), lam


def max_cut_values(P, Omega, C, approx_eps=1e-6, device=None):
    """(value, column values, sign words) of compute_max_cut, as CUDA tensors."""
    torch = _torch()
    dev = torch.device(device) if device is not None else (
        P.device if isinstance(P, torch.Tensor) and P.is_cuda else torch.device("cuda"))
    o, p, n, s, ld = _operands(Omega, P, dev)
    dc = _device_csr(C, dev)
    if dc.n != n:
        raise ValueError(f"compute_max_cut: C has {dc.n} rows, the sketch {n}")
    lib = _lib.load()
    wsb = int(lib.usbs_round_workspace_bytes(n, s))
    if wsb == 0:
        raise ValueError(f"compute_max_cut: unsupported sizes n={n} s={s} (s <= 32)")
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    out = torch.empty(1 + s, dtype=torch.float64, device=dev)
    signs = torch.empty(n, dtype=torch.int32, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    rc = lib.usbs_maxcut_round(n, s, _ptr(o), _ptr(p), ld, _ptr(dc.rowptr), _ptr(dc.col),
                               _ptr(dc.val), float(approx_eps), _ptr(out),
                               ctypes.c_void_p(out.data_ptr() + 8), _ptr(signs), _ptr(ws), wsb,
                               ctypes.c_void_p(st))
    _lib.check(rc, "usbs_maxcut_round")
    return out[0], out[1:], signs


def compute_max_cut(P, Omega, callback_static_args, callback_nonstatic_args):
    """utils/maxcut_helpers.py:292-302: the largest cut w^T C w among the sign
    patterns w = sign(E[:, j]) of the reconstructed sketch (as a float)."""
    value, _, _ = max_cut_values(P, Omega, callback_nonstatic_args)
    return float(value.item())


_DENSE_CACHE = []        # [(matrix object, device tensor)], most recent last


def _device_dense(M, device):
    torch = _torch()
    if isinstance(M, torch.Tensor):
        return M.to(device=device, dtype=torch.float64).contiguous()
    for obj, t in _DENSE_CACHE:
        if obj is M:
            return t
    t = torch.as_tensor(np.ascontiguousarray(np.asarray(M, dtype=np.float64)), device=device)
    _DENSE_CACHE.append((M, t))
    del _DENSE_CACHE[:-4]
    return t


def qap_round_values(P, Omega, l, D, W, approx_eps=1e-6, device=None):
    """(value, candidate values, candidate permutations) of qap_round as CUDA
    tensors: the candidates are the first min(l, s) columns of E, then their
    negatives; a permutation gives each facility's location."""
    torch = _torch()
    dev = torch.device(device) if device is not None else (
        P.device if isinstance(P, torch.Tensor) and P.is_cuda else torch.device("cuda"))
    o, p, n, s, ld = _operands(Omega, P, dev)
    l = int(l)
    if n != l * l + 1:
        raise ValueError(f"qap_round: the sketch has {n} rows, l^2 + 1 = {l * l + 1} expected")
    Dt, Wt = _device_dense(D, dev), _device_dense(W, dev)
    if tuple(Dt.shape) != (l, l) or tuple(Wt.shape) != (l, l):
        raise ValueError("qap_round: D and W must be l x l")
    lib = _lib.load()
    wsb = int(lib.usbs_qap_round_workspace_bytes(l, s))
    if wsb == 0:
        raise ValueError(f"qap_round: unsupported sizes l={l} s={s} (l <= 64, s <= 32)")
    s2 = min(l, s)
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    out = torch.empty(1 + 2 * s2, dtype=torch.float64, device=dev)
    perms = torch.empty((2 * s2, l), dtype=torch.int32, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    rc = lib.usbs_qap_round(l, s, _ptr(o), _ptr(p), ld, _ptr(Wt), _ptr(Dt), float(approx_eps),
                            _ptr(out), ctypes.c_void_p(out.data_ptr() + 8), _ptr(perms), _ptr(ws),
                            wsb, ctypes.c_void_p(st))
    _lib.check(rc, "usbs_qap_round")
    return out[0], out[1:], perms


def qap_round(P, Omega, callback_static_args, callback_nonstatic_args):
    """utils/qap_helpers.py:624-653: the smallest QAP objective among the
    assignments read off the reconstructed sketch's columns (as a float)."""
    import pickle
    st = callback_static_args
    l = pickle.loads(st)["l"] if isinstance(st, (bytes, bytearray)) else (
        st["l"] if isinstance(st, dict) else int(st))
    value, _, _ = qap_round_values(P, Omega, l, callback_nonstatic_args["D"],
                                   callback_nonstatic_args["W"])
    return float(value.item())
