"""Reference-shaped entry points of the USBS hot path on the GB300.

Each function keeps the name, argument order and meaning of the reference
(rangell/usbs) and runs on the device through the C ABI of libusbs_gb300:

* ``apply_A_operator_slim/_batched``  solver/utils.py:11-16, 27-31
* ``apply_A_adjoint_slim/_batched``   solver/utils.py:19-24, 34-37
* ``eigsh_smallest``                  solver/lanczos.py:239-284
* ``usbs`` / ``cgal``                 solver/usbs.py:436, solver/cgal.py:21 (see solver.py)

Inputs may be NumPy / SciPy (copied to the device), CUDA torch tensors, or any
DLPack producer such as a JAX device array (used in place, no copy, when its
dtype matches); the outputs are CUDA torch tensors.  There is no CPU path:
without a CUDA device or without the built library every call raises.
"""
import collections
import ctypes
import hashlib

import numpy as np
import scipy.sparse as sp

from . import _lib
from .arrays import as_torch, shape_of, to_device
from .problem import DeviceProblem, layout


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("usbs_gb300 needs a CUDA device (GB300, sm_103a); none is visible")
    return torch


def _p(t):
    return ctypes.c_void_p(int(t.data_ptr())) if t is not None else ctypes.c_void_p(0)


def _stream():
    torch = _torch()
    return ctypes.c_void_p(int(torch.cuda.current_stream().cuda_stream))


def _dev(x, dtype, device):
    _torch()
    return to_device(x, dtype, device)


def _vt(precision):
    torch = _torch()
    if precision == 64:
        return torch.float64
    if precision == 32:
        return torch.float32
    raise ValueError("precision must be 64 or 32")


# Device layouts of recent reference-style calls (SciPy C, NumPy A_data and
# A_indices), keyed by the content of those arrays: a caller that passes the same
# problem every iteration, as the reference's solver loop does, gets the resident
# layout back instead of a host rebuild and a fresh upload.  A changed array
# (even in place) changes the key.
_LAYOUTS = collections.OrderedDict()
_LAYOUTS_MAX = 4


def _digest(*arrays):
    h = hashlib.blake2b(digest_size=16)
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str((a.dtype.str, a.shape)).encode())
        h.update(memoryview(a).cast("B"))
    return h.digest()


def _layout_key(C, A_data, A_indices, m, device):
    """Content key of host inputs, or None when any input is not a host array
    (device arrays are laid out afresh: hashing them would copy them back)."""
    if not sp.issparse(C) or not isinstance(A_data, np.ndarray) or \
            not isinstance(A_indices, np.ndarray):
        return None
    Cc = C.tocsr()
    return (int(m), str(device), Cc.shape, _digest(Cc.data, Cc.indices, Cc.indptr),
            _digest(A_data, A_indices))


def _problem_for(C, A_data, A_indices, m, device, *, make=None):
    if isinstance(C, DeviceProblem):
        return C
    make = make if make is not None else \
        (lambda: DeviceProblem(layout(C, A_data, A_indices, m=m), device=device))
    key = _layout_key(C, A_data, A_indices, m, device)
    if key is None:
        return make()
    prob = _LAYOUTS.get(key)
    if prob is None:
        prob = make()
        _LAYOUTS[key] = prob
        while len(_LAYOUTS) > _LAYOUTS_MAX:
            _LAYOUTS.popitem(last=False)
    else:
        _LAYOUTS.move_to_end(key)
    return prob


def _cols(U, n, device):
    """Column-major device copy of an (n,) or (n, k) array: returns (tensor[k, ld], ld, k)."""
    torch = _torch()
    Ut = _dev(U, torch.float64, device)
    if Ut.dim() == 1:
        Ut = Ut.reshape(n, 1)
    k = Ut.shape[1]
    return Ut.t().contiguous(), n, k


def apply_A_operator_batched(m, A_data, A_indices, vecs, *, problem=None, n=None, device="cuda"):
    """sum_j A(v_j v_j^T) over the columns of ``vecs`` -> (m,) float64."""
    torch = _torch()
    lib = _lib.load()
    if problem is None:
        nn = n if n is not None else int(shape_of(vecs)[0])
        problem = _problem_for(sp.csr_matrix((nn, nn)), A_data, A_indices, m, device)
    Ucm, ld, k = _cols(vecs, problem.n, problem.device)
    out = torch.empty(m, dtype=torch.float64, device=problem.device)
    _lib.check(lib.usbs_apply_A_operator(m, k, _p(problem.con_ptr), _p(problem.t_row),
                                         _p(problem.t_col), _p(problem.t_a), _p(Ucm), ld,
                                         _p(out), _stream()), "usbs_apply_A_operator")
    return out


def apply_A_operator_slim(m, A_data, A_indices, u, **kw):
    """A(u u^T) -> (m,) float64 (solver/utils.py:11-16)."""
    return apply_A_operator_batched(m, A_data, A_indices, u, **kw)


def apply_A_adjoint_batched(n, A_data, A_indices, z, vecs, *, problem=None, device="cuda"):
    """[A*(z) v_j]_j for the columns of ``vecs`` -> (n, k) float64."""
    torch = _torch()
    lib = _lib.load()
    zz = _dev(z, torch.float64, device if problem is None else problem.device)
    if problem is None:
        problem = _problem_for(sp.csr_matrix((n, n)), A_data, A_indices, zz.numel(), device)
    Ucm, ld, k = _cols(vecs, n, problem.device)
    out = torch.empty((k, n), dtype=torch.float64, device=problem.device)
    _lib.check(lib.usbs_apply_A_adjoint(n, k, _p(problem.row_ptr), _p(problem.r_con),
                                        _p(problem.r_col), _p(problem.r_a), _p(zz), _p(Ucm), ld,
                                        _p(out), n, _stream()), "usbs_apply_A_adjoint")
    return out.t()


def apply_A_adjoint_slim(n, A_data, A_indices, z, u, **kw):
    """A*(z) u -> (n,) float64 (solver/utils.py:19-24)."""
    return apply_A_adjoint_batched(n, A_data, A_indices, z, u, **kw)[:, 0]


def operator_apply(problem, c_scale, w, x, precision=64):
    """(c_scale * C + A*(w)) x on the device (the Lanczos operator, solver/lanczos.py:86-87)."""
    torch = _torch()
    lib = _lib.load()
    vt = _vt(precision)
    dev = problem.device
    op = torch.empty(max(problem.nnz, 1), dtype=vt, device=dev)
    wt = _dev(w, torch.float64, dev) if w is not None else None
    _lib.check(lib.usbs_assemble_operator(problem.nnz, _p(problem.c_val), float(c_scale),
                                          _p(problem.slot_ptr), _p(problem.slot_tid),
                                          _p(problem.t_con), _p(problem.t_a0), _p(wt), _p(op),
                                          precision, _stream()), "usbs_assemble_operator")
    xt = _dev(x, vt, dev)
    y = torch.empty(problem.n, dtype=vt, device=dev)
    _lib.check(lib.usbs_operator_apply(problem.n, problem.nnz, _p(problem.rowptr),
                                       _p(problem.col), _p(op), _p(xt), _p(y), precision,
                                       _stream()), "usbs_operator_apply")
    return y


class EigshInfo:
    def __init__(self, raw):
        self.k_saved, self.num_converged, self.restarts, self.breakdowns, self.matvecs, \
            self.status = (int(v) for v in raw[:6])
        self.restart_kcycles, self.total_kcycles = int(raw[6]), int(raw[7])
        self.phase_kcycles = [int(v) for v in raw[8:13]]
        self.sum_active_columns, self.sum_saved = int(raw[13]), int(raw[14])
        self.eig_kcycles = int(raw[15])

    def __repr__(self):
        return (f"EigshInfo(restarts={self.restarts}, converged={self.num_converged}, "
                f"matvecs={self.matvecs}, breakdowns={self.breakdowns}, status={self.status}, "
                f"restart_kcycles={self.restart_kcycles}, total_kcycles={self.total_kcycles}, "
                f"eig_kcycles={self.eig_kcycles}, bar/red/A/B/C={self.phase_kcycles})")


def eigsh_smallest(n, C, A_data, A_indices, adjoint_left_vec, q0, num_desired, inner_iterations,
                   max_restarts, tolerance, *, c_scale=1.0, precision=64, device="cuda",
                   return_info=False, workspace=None):
    """Smallest ``num_desired`` eigenpairs of c_scale*C + A*(adjoint_left_vec)
    (solver/lanczos.py:239-284).  ``C`` is a SciPy sparse matrix or a prepared
    :class:`DeviceProblem` (whose A data are then used).  Returns
    ``(eigenvalues[num_desired] float64, eigenvectors[n, num_desired])``."""
    torch = _torch()
    lib = _lib.load()
    w = as_torch(adjoint_left_vec)
    if w is None:
        w = np.asarray(adjoint_left_vec)
    prob = _problem_for(C, A_data, A_indices, int(w.shape[0]), device)
    dev = prob.device
    vt = _vt(precision)
    wt = _dev(w, torch.float64, dev)
    q0t = _dev(q0, vt, dev)
    ld = (n + 31) // 32 * 32
    Q = torch.empty((inner_iterations + 1, ld), dtype=vt, device=dev)
    evals = torch.empty(num_desired, dtype=torch.float64, device=dev)
    info = torch.zeros(16, dtype=torch.int32, device=dev)
    need = int(lib.usbs_eigsh_workspace_bytes(n, prob.nnz, inner_iterations, precision))
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(need, dtype=torch.uint8, device=dev)
    rc = lib.usbs_eigsh_smallest(n, prob.nnz, _p(prob.rowptr), _p(prob.col), _p(prob.c_val),
                                 float(c_scale), _p(prob.slot_ptr), _p(prob.slot_tid),
                                 _p(prob.t_con), _p(prob.t_a0), _p(wt), _p(q0t), num_desired,
                                 inner_iterations, max_restarts, float(tolerance), precision,
                                 _p(Q), ld, _p(evals), _p(info), _p(workspace), need, _stream())
    _lib.check(rc, "usbs_eigsh_smallest")
    vecs = Q[:num_desired, :n].t()
    if return_info:
        inf = EigshInfo(info.cpu().tolist())
        if inf.status & 1:
            raise RuntimeError("eigsh_smallest: a team barrier timed out on the device")
        return evals, vecs, inf
    return evals, vecs


class EigshProblem(ctypes.Structure):
    """usbs_eigsh_problem (include/usbs_gb300.h)."""
    _fields_ = [("n", ctypes.c_int), ("nnz", ctypes.c_longlong)] + \
        [(f, ctypes.c_void_p) for f in ("rowptr", "col", "c_val")] + [("c_scale", ctypes.c_double)] + \
        [(f, ctypes.c_void_p) for f in ("slot_ptr", "slot_tid", "t_con", "t_a",
                                         "adjoint_left_vec", "q0")] + \
        [("num_desired", ctypes.c_int), ("Q", ctypes.c_void_p), ("ldq", ctypes.c_int),
         ("eigenvalues", ctypes.c_void_p), ("info", ctypes.c_void_p),
         ("workspace", ctypes.c_void_p), ("workspace_bytes", ctypes.c_size_t)]


def _eigsh_batch(problems, num_desired, inner_iterations, precision, c_scale):
    """The usbs_eigsh_problem array of a batch with its output tensors (kept
    alive in the returned list)."""
    torch = _torch()
    lib = _lib.load()
    vt = _vt(precision)
    keep, out = [], []
    arr = (EigshProblem * max(len(problems), 1))()
    for i, (prob, w, q0) in enumerate(problems):
        dev = prob.device
        n = prob.n
        wt = _dev(w, torch.float64, dev)
        q0t = _dev(q0, vt, dev)
        ld = (n + 31) // 32 * 32
        Q = torch.empty((inner_iterations + 1, ld), dtype=vt, device=dev)
        evals = torch.empty(num_desired, dtype=torch.float64, device=dev)
        info = torch.zeros(16, dtype=torch.int32, device=dev)
        need = int(lib.usbs_eigsh_workspace_bytes(n, prob.nnz, inner_iterations, precision))
        ws = torch.empty(need, dtype=torch.uint8, device=dev)
        keep += [wt, q0t, Q, ws]
        a = arr[i]
        a.n, a.nnz = n, prob.nnz
        a.rowptr, a.col, a.c_val = prob.rowptr.data_ptr(), prob.col.data_ptr(), prob.c_val.data_ptr()
        a.c_scale = float(c_scale)
        a.slot_ptr, a.slot_tid = prob.slot_ptr.data_ptr(), prob.slot_tid.data_ptr()
        a.t_con, a.t_a = prob.t_con.data_ptr(), prob.t_a0.data_ptr()
        a.adjoint_left_vec, a.q0 = wt.data_ptr(), q0t.data_ptr()
        a.num_desired, a.Q, a.ldq = num_desired, Q.data_ptr(), ld
        a.eigenvalues, a.info = evals.data_ptr(), info.data_ptr()
        a.workspace, a.workspace_bytes = ws.data_ptr(), need
        out.append((evals, Q[:num_desired, :n].t(), info))
    return arr, keep, out


def _batch_results(out, return_info, what):
    if not return_info:
        return [(e, v) for e, v, _ in out]
    res = []
    for e, v, info in out:
        inf = EigshInfo(info.cpu().tolist())
        if inf.status & 1:
            raise RuntimeError(f"{what}: a team barrier timed out on the device")
        res.append((e, v, inf))
    return res


def eigsh_smallest_batched(problems, num_desired, inner_iterations, max_restarts, tolerance, *,
                           c_scale=1.0, precision=64, return_info=False):
    """eigsh_smallest for many independent problems in as few launches as the
    kernels allow (up to 48 per launch): ``problems`` is a list of
    ``(DeviceProblem, adjoint_left_vec, q0)`` on one device.  Returns a list of
    ``(eigenvalues, eigenvectors)`` (with an EigshInfo each if return_info)."""
    lib = _lib.load()
    fn = lib.usbs_eigsh_smallest_batched
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.POINTER(EigshProblem), ctypes.c_int, ctypes.c_int,
                   ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
    arr, keep, out = _eigsh_batch(problems, num_desired, inner_iterations, precision, c_scale)
    rc = fn(len(problems), arr, inner_iterations, max_restarts, float(tolerance), precision,
            _stream())
    _lib.check(rc, "usbs_eigsh_smallest_batched")
    del keep
    return _batch_results(out, return_info, "eigsh_smallest_batched")


TUNE_CANDIDATES = (64, 128, 256, 640, 1280)


def lanczos_autotune(problems, num_desired, inner_iterations, max_restarts, tolerance, *,
                     c_scale=1.0, precision=32):
    """Times the cluster-size candidates (rows per CTA) on a batch of at most
    48 ``(DeviceProblem, adjoint_left_vec, q0)`` and records the fastest for the
    batch's class (precision, log2 of the count, log2 of the largest n); later
    Lanczos launches of that class use it.  Returns ``{"rows_per_cta": best,
    "ms": {candidate: ms or None (same cluster size as the one before)}}``."""
    lib = _lib.load()
    fn = lib.usbs_lanczos_autotune
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.POINTER(EigshProblem), ctypes.c_int, ctypes.c_int,
                   ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                   ctypes.POINTER(ctypes.c_float)]
    arr, keep, _ = _eigsh_batch(problems, num_desired, inner_iterations, precision, c_scale)
    best = ctypes.c_int(0)
    ms = (ctypes.c_float * len(TUNE_CANDIDATES))()
    rc = fn(len(problems), arr, inner_iterations, max_restarts, float(tolerance), precision,
            _stream(), ctypes.byref(best), ms)
    _lib.check(rc, "usbs_lanczos_autotune")
    del keep
    return {"rows_per_cta": best.value,
            "ms": {c: (float(m) if m >= 0 else None) for c, m in zip(TUNE_CANDIDATES, ms)}}


def lanczos_tuning():
    """The process's tuned classes: a list of ``{"precision", "log2_count",
    "log2_max_n", "rows_per_cta"}`` (JSON-serialisable, for set_lanczos_tuning)."""
    lib = _lib.load()
    k = lib.usbs_lanczos_tuning_get(None, None, 0)
    keys = (ctypes.c_longlong * max(k, 1))()
    rows = (ctypes.c_int * max(k, 1))()
    k = lib.usbs_lanczos_tuning_get(ctypes.cast(keys, ctypes.c_void_p),
                                    ctypes.cast(rows, ctypes.c_void_p), k)
    return [{"precision": int(keys[i] >> 32), "log2_count": int((keys[i] >> 16) & 0xffff),
             "log2_max_n": int(keys[i] & 0xffff), "rows_per_cta": int(rows[i])}
            for i in range(k)]


def set_lanczos_tuning(entries, clear=False):
    """Loads entries of lanczos_tuning() (e.g. saved from another process)."""
    lib = _lib.load()
    if clear:
        lib.usbs_lanczos_tuning_clear()
    for e in entries:
        rc = lib.usbs_lanczos_tuning_put(int(e["precision"]), 1 << int(e["log2_count"]),
                                         1 << int(e["log2_max_n"]), int(e["rows_per_cta"]))
        _lib.check(rc, "usbs_lanczos_tuning_put")
