"""usbs() on the GB300: the reference's solver call surface over the C ABI.

``usbs(sdp_state, n, m, trace_ub, trace_factor, rho, beta, k_curr, k_past,
max_iters, max_time, obj_gap_eps, infeas_gap_eps, max_infeas_eps,
lanczos_inner_iterations, lanczos_max_restarts, subprob_eps, subprob_max_iters,
cond_exp_base, callback_fn, callback_static_args, callback_nonstatic_args)``
keeps the signature of solver/usbs.py:436-459 and returns an SDPState.  The
whole iteration runs on the device (libusbs_gb300 ``usbs_solve``); Python only
prepares the problem layout once and reads the result.

Extra keyword arguments: ``q0`` (Lanczos start vector; the reference draws it
from ``PRNGKey(0)``), ``precision`` (64 = FP64 parity path, 32 = FP32 Lanczos
with FP64 subproblems, gaps and Rayleigh refinement), ``device``,
``return_trace`` (per-iteration record), ``problem`` (a prepared
:class:`DeviceProblem`, to skip the host layout step).
"""
import ctypes
import time

import numpy as np
import scipy.sparse as sp

from . import _lib
from .arrays import as_torch, shape_of, to_device, to_host
from .problem import DeviceProblem, layout
from .rng import default_q0
from .state import SDPState

P = ctypes.c_void_p


class UsbsProblem(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("m", ctypes.c_int), ("nnz", ctypes.c_longlong),
                ("num_triples", ctypes.c_int)] + \
        [(f, P) for f in ("rowptr", "col", "c_val", "slot_ptr", "slot_tid", "t_con", "t_a0",
                          "con_ptr", "t_row", "t_col", "t_a", "row_ptr", "r_con", "r_col", "r_a",
                          "b", "b_ineq_mask", "scale_a")] + \
        [("scale_c", ctypes.c_double), ("scale_x", ctypes.c_double), ("b_norm", ctypes.c_double),
         ("has_ineq", ctypes.c_int)]


class UsbsParams(ctypes.Structure):
    _fields_ = [("trace_ub", ctypes.c_double), ("trace_factor", ctypes.c_double),
                ("rho", ctypes.c_double), ("beta", ctypes.c_double), ("k_curr", ctypes.c_int),
                ("k_past", ctypes.c_int), ("max_iters", ctypes.c_int),
                ("max_time", ctypes.c_double), ("obj_gap_eps", ctypes.c_double),
                ("infeas_gap_eps", ctypes.c_double), ("max_infeas_eps", ctypes.c_double),
                ("lanczos_inner_iterations", ctypes.c_int), ("lanczos_max_restarts", ctypes.c_int),
                ("subprob_eps", ctypes.c_double), ("subprob_max_iters", ctypes.c_int),
                ("cond_exp_base", ctypes.c_double), ("precision", ctypes.c_int),
                ("sketch_mode", ctypes.c_int), ("sketch_dim", ctypes.c_int),
                ("lanczos_rows_per_cta", ctypes.c_int), ("lanczos_path", ctypes.c_int)]


class UsbsState(ctypes.Structure):
    _fields_ = [("ld", ctypes.c_int)] + [(f, P) for f in ("y", "z", "V", "P", "Omega", "X", "q0",
                                                          "trace")] + \
        [("trace_capacity", ctypes.c_int), ("debug", P), ("tr_X", ctypes.c_double),
         ("primal_obj", ctypes.c_double), ("iterations", ctypes.c_int),
         ("obj_gap", ctypes.c_double), ("infeas_gap", ctypes.c_double),
         ("max_infeas", ctypes.c_double), ("obj_ub", ctypes.c_double),
         ("pen_dual_obj", ctypes.c_double), ("elapsed", ctypes.c_double),
         ("status", ctypes.c_int), ("lanczos_launches", ctypes.c_int),
         ("lanczos_ms", ctypes.c_double), ("lanczos_bytes", ctypes.c_double),
         ("kernel_launches", ctypes.c_longlong), ("cond", ctypes.c_double * 20),
         ("graph_iterations", ctypes.c_longlong)]


class CgalParams(ctypes.Structure):
    _fields_ = [("trace_ub", ctypes.c_double), ("beta0", ctypes.c_double),
                ("max_iters", ctypes.c_int), ("max_time", ctypes.c_double),
                ("obj_gap_eps", ctypes.c_double), ("infeas_gap_eps", ctypes.c_double),
                ("max_infeas_eps", ctypes.c_double), ("lanczos_inner_iterations", ctypes.c_int),
                ("lanczos_max_restarts", ctypes.c_int), ("subprob_eps", ctypes.c_double),
                ("cond_exp_base", ctypes.c_double), ("precision", ctypes.c_int),
                ("sketch_mode", ctypes.c_int), ("sketch_dim", ctypes.c_int)]


CALLBACK = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int)

TRACE_FIELDS = ["t", "primal_obj", "obj_ub", "obj_gap", "infeas_gap", "max_infeas",
                "pen_dual_obj", "cand_pen_dual_obj", "lb_spec_est", "cand_eig0", "descent", "eta",
                "trS", "tr_X", "quad_iters", "lb_iters", "bar_primal_obj", "tr_X_bar", "dual_obj"]


def log_line(rec, scale_c, scale_x, callback_val=None, curr_time=None):
    """The line solver/usbs.py:514-530 prints at every condition check (field
    names and order as the reference's), for the state record `rec` (trace
    field names) of that check; curr_time defaults to the wall clock now."""
    ct = time.time() if curr_time is None else curr_time
    return (f"t: {int(rec['t'])} - curr_time: {ct} - pen_dual_obj: {rec['pen_dual_obj']}"
            f" - cand_pen_dual_obj: {rec['cand_pen_dual_obj']} - lb_spec_est: {rec['lb_spec_est']}"
            f" - primal_obj: {rec['primal_obj'] / (scale_c * scale_x)} - dual_obj: {rec['dual_obj']}"
            f" - primal_obj_ub: {rec['obj_ub']} - obj_gap: {rec['obj_gap']}"
            f" - infeas_gap: {rec['infeas_gap']} - max_infeas: {rec['max_infeas']}"
            f" - callback_val: {callback_val}")


def cgal_log_line(rec, scale_c, scale_x, callback_val=None, curr_time=None):
    """The line solver/cgal.py:79-88 prints at every condition check."""
    ct = time.time() if curr_time is None else curr_time
    return (f"t: {int(rec['t'])} - curr_time: {ct} - primal_obj: "
            f"{rec['primal_obj'] / (scale_c * scale_x)} - obj_gap: {rec['obj_gap']}"
            f" - infeas_gap: {rec['infeas_gap']} - max_infeas: {rec['max_infeas']}"
            f" - callback_val: {callback_val}")
TRACE_WIDTH = 20


def _sigs(lib):
    lib.usbs_solve_workspace_bytes.restype = ctypes.c_size_t
    lib.usbs_solve_workspace_bytes.argtypes = [ctypes.POINTER(UsbsProblem),
                                               ctypes.POINTER(UsbsParams)]
    lib.usbs_solve.restype = ctypes.c_int
    lib.usbs_solve.argtypes = [ctypes.POINTER(UsbsProblem), ctypes.POINTER(UsbsParams),
                               ctypes.POINTER(UsbsState), P, ctypes.c_size_t, CALLBACK, P, P]
    lib.usbs_cgal_workspace_bytes.restype = ctypes.c_size_t
    lib.usbs_cgal_workspace_bytes.argtypes = [ctypes.POINTER(UsbsProblem),
                                              ctypes.POINTER(CgalParams)]
    lib.usbs_cgal_solve.restype = ctypes.c_int
    lib.usbs_cgal_solve.argtypes = [ctypes.POINTER(UsbsProblem), ctypes.POINTER(CgalParams),
                                    ctypes.POINTER(UsbsState), P, ctypes.c_size_t, CALLBACK, P,
                                    P]


def _ptr(t):
    return int(t.data_ptr()) if t is not None else None


def host_problem_layout(sdp_state):
    """The problem's device layout built on the host (no device memory)."""
    A_idx = np.asarray(_host(sdp_state.A_indices))
    b = np.asarray(_host(sdp_state.b))
    return layout(sp.csr_matrix(sdp_state.C), _host(sdp_state.A_data), A_idx, m=b.shape[0])


class DeviceInstance:
    """Problem layout + constraint vectors of one SDP, resident on one device."""

    def __init__(self, sdp_state, device, host_layout=None):
        import torch
        self.device = torch.device(device)
        b = np.asarray(_host(sdp_state.b), dtype=np.float64)
        if host_layout is None:
            host_layout = host_problem_layout(sdp_state)
        self.problem = DeviceProblem(host_layout, device)
        mask = np.asarray(_host(sdp_state.b_ineq_mask), dtype=np.float64)
        SA = np.broadcast_to(np.asarray(_host(sdp_state.SCALE_A), dtype=np.float64),
                             b.shape).copy()
        self.b = torch.as_tensor(b, device=self.device)
        self.mask = torch.as_tensor(mask, device=self.device)
        self.scale_a = torch.as_tensor(SA, device=self.device)
        self.scale_c = float(sdp_state.SCALE_C)
        self.scale_x = float(sdp_state.SCALE_X)
        self.b_norm = float(np.linalg.norm((b / SA) / self.scale_x))
        self.has_ineq = bool(np.any(mask != 0))

    def c_struct(self):
        p = self.problem
        s = UsbsProblem()
        s.n, s.m, s.nnz, s.num_triples = p.n, p.m, p.nnz, p.num_triples
        for f in ("rowptr", "col", "c_val", "slot_ptr", "slot_tid", "t_con", "t_a0", "con_ptr",
                  "t_row", "t_col", "t_a", "row_ptr", "r_con", "r_col", "r_a"):
            setattr(s, f, _ptr(getattr(p, f)))
        s.b, s.b_ineq_mask, s.scale_a = _ptr(self.b), _ptr(self.mask), _ptr(self.scale_a)
        s.scale_c, s.scale_x, s.b_norm, s.has_ineq = (self.scale_c, self.scale_x, self.b_norm,
                                                      int(self.has_ineq))
        return s


_host = to_host


def _to_dev(x, device):
    """float64 tensor on `device`; device arrays (torch or any DLPack producer)
    are not routed through the host."""
    import torch
    return to_device(x, torch.float64, device)


def _dev_cols(x, rows, ld, cols, device, dtype):
    """Column-major (cols x ld) device tensor from an (rows, cols) array."""
    import torch
    out = torch.zeros((cols, ld), dtype=dtype, device=device)
    if x is not None:
        xt = as_torch(x)
        if xt is None:
            xt = torch.as_tensor(np.asarray(x))
        out[:, :rows] = xt.to(device=device, dtype=dtype).reshape(rows, cols).t()
    return out


class _Renumbering:
    """The permutation a renumbered solve runs under (none by default): the
    callback's views of P and Omega and the returned state go back to the
    original numbering."""

    def __init__(self, orig=None, perm=None, dev=None):
        self.orig, self.perm, self.inv_t = orig, perm, None
        if perm is not None:
            import torch
            from .renumber import inverse
            self.inv_t = torch.as_tensor(inverse(perm), device=dev)

    def rows(self, *mats):
        if self.inv_t is None:
            return mats
        return tuple(M.index_select(0, self.inv_t) for M in mats)

    def restore(self, out, info):
        if self.perm is None:
            return out, info
        from .renumber import unpermute_rows, unpermute_state
        out = unpermute_state(out, self.orig, self.perm)
        if "V" in info:
            info["V"] = unpermute_rows(info["V"], self.perm)
        return out, info


def _renumbered(sdp_state, n, q0, flag, instance, dev):
    """(state to solve, its start vector, _Renumbering) for renumber=flag."""
    if not flag:
        return sdp_state, q0, _Renumbering()
    if instance is not None:
        raise ValueError("renumber=True builds its own device instance")
    from .renumber import permute_state, rcm_permutation
    perm = rcm_permutation(sdp_state.C, sdp_state.A_indices, n)
    q = default_q0(n) if q0 is None else _host(q0)
    return permute_state(sdp_state, perm), np.asarray(q)[perm], _Renumbering(sdp_state, perm, dev)


def usbs(sdp_state, n, m, trace_ub, trace_factor, rho, beta, k_curr, k_past, max_iters, max_time,
         obj_gap_eps, infeas_gap_eps, max_infeas_eps, lanczos_inner_iterations,
         lanczos_max_restarts, subprob_eps, subprob_max_iters, cond_exp_base=1.0,
         callback_fn=None, callback_static_args=None, callback_nonstatic_args=None, *, q0=None,
         precision=64, device="cuda", return_trace=False, return_info=False, instance=None,
         stream=None, debug=None, log=None, renumber=False, lanczos_rows_per_cta=0,
         lanczos_path=0):
    """``log``: True prints, a callable receives, the reference's per-check
    line (solver/usbs.py:514-530) at every condition check, t = 0 included.
    ``renumber``: solve the RCM-renumbered problem (locality for the device's
    sparse gathers) and return the result in the original numbering; the
    callback still sees P and Omega in the original numbering.
    ``lanczos_rows_per_cta``: rows per CTA of the cluster Lanczos (0: the
    library's choice; a solve service that shares the GPU packs tighter).
    ``lanczos_path``: 2 keeps every problem too large for one cluster on the
    stream path (no cooperative launch, so the solve can share the GPU)."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("usbs_gb300.usbs needs a CUDA device (GB300); none is visible")
    lib = _lib.load()
    _sigs(lib)
    dev = torch.device(device)
    sdp_state, q0, ren = _renumbered(sdp_state, n, q0, renumber, instance, dev)
    inst = instance if instance is not None else DeviceInstance(sdp_state, dev)
    k = k_curr + k_past
    ld = (n + 31) // 32 * 32
    f64 = torch.float64
    y = _to_dev(sdp_state.y, dev).clone()
    z = _to_dev(sdp_state.z, dev).clone()
    V = torch.zeros((k, ld), dtype=f64, device=dev)
    if sdp_state.X is not None:
        mode, sdim = 1, 0
        X = _to_dev(sdp_state.X, dev).clone()
        Pm = Om = None
    elif sdp_state.Omega is not None:
        mode = 0
        sdim = int(shape_of(sdp_state.Omega)[1])
        Om = _dev_cols(sdp_state.Omega, n, ld, sdim, dev, f64)
        Pm = _dev_cols(sdp_state.P, n, ld, sdim, dev, f64)
        X = None
    else:
        mode, sdim = 2, 0
        Pm = torch.zeros(ld, dtype=f64, device=dev)
        if sdp_state.P is not None:
            Pm[:n] = _to_dev(sdp_state.P, dev).reshape(-1)
        Om = X = None
    q0t = _to_dev(default_q0(n) if q0 is None else q0, dev)
    trace = torch.zeros((max(max_iters, 1), TRACE_WIDTH), dtype=f64, device=dev) \
        if return_trace else None
    log_fn = print if log is True else log

    prm = UsbsParams()
    prm.trace_ub, prm.trace_factor, prm.rho, prm.beta = trace_ub, trace_factor, rho, beta
    prm.k_curr, prm.k_past, prm.max_iters = k_curr, k_past, int(max_iters)
    prm.max_time = float(max_time)
    prm.obj_gap_eps, prm.infeas_gap_eps, prm.max_infeas_eps = (obj_gap_eps, infeas_gap_eps,
                                                               max_infeas_eps)
    prm.lanczos_inner_iterations = int(lanczos_inner_iterations)
    prm.lanczos_max_restarts = int(lanczos_max_restarts)
    prm.subprob_eps, prm.subprob_max_iters = subprob_eps, int(subprob_max_iters)
    prm.cond_exp_base = float(cond_exp_base)
    prm.precision, prm.sketch_mode, prm.sketch_dim = int(precision), mode, sdim
    prm.lanczos_rows_per_cta = int(lanczos_rows_per_cta)
    prm.lanczos_path = int(lanczos_path)
    pst = UsbsState()
    pst.ld = ld
    pst.y, pst.z, pst.V = _ptr(y), _ptr(z), _ptr(V)
    pst.P, pst.Omega, pst.X, pst.q0, pst.trace = _ptr(Pm), _ptr(Om), _ptr(X), _ptr(q0t), _ptr(trace)
    pst.trace_capacity = int(max_iters) if return_trace else 0
    pst.debug = _ptr(debug)
    pst.tr_X, pst.primal_obj = float(sdp_state.tr_X), float(sdp_state.primal_obj)
    prob = inst.c_struct()
    need = int(lib.usbs_solve_workspace_bytes(ctypes.byref(prob), ctypes.byref(prm)))
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    cb_val = {}

    def _cb(_user, t):
        if callback_fn is not None and Om is not None:
            cb_val[t] = callback_fn(*ren.rows(Pm[:, :n].t(), Om[:, :n].t()),
                                    callback_static_args, callback_nonstatic_args)
        if log_fn is not None:
            rec = {f: float(pst.cond[i]) for i, f in enumerate(TRACE_FIELDS)}
            log_fn(log_line(rec, float(sdp_state.SCALE_C), float(sdp_state.SCALE_X),
                            cb_val.get(t)))

    ccb = CALLBACK(_cb)
    st = stream if stream is not None else torch.cuda.current_stream(dev)
    rc = lib.usbs_solve(ctypes.byref(prob), ctypes.byref(prm), ctypes.byref(pst), _ptr(ws), need,
                        ccb, None, int(st.cuda_stream))
    _lib.check(rc, "usbs_solve")
    if pst.status & 1:
        raise RuntimeError("usbs_solve: a device barrier timed out")
    out = SDPState(C=sdp_state.C, A_indices=sdp_state.A_indices, A_data=sdp_state.A_data,
                   b=sdp_state.b, b_ineq_mask=sdp_state.b_ineq_mask,
                   X=X, P=(Pm[:, :n].t() if mode == 0 else (Pm[:n] if mode == 2 else None)),
                   Omega=sdp_state.Omega, y=y, z=z, tr_X=pst.tr_X, primal_obj=pst.primal_obj,
                   SCALE_C=sdp_state.SCALE_C, SCALE_X=sdp_state.SCALE_X,
                   SCALE_A=sdp_state.SCALE_A)
    info = dict(iterations=pst.iterations, obj_gap=pst.obj_gap, infeas_gap=pst.infeas_gap,
                max_infeas=pst.max_infeas, obj_ub=pst.obj_ub, pen_dual_obj=pst.pen_dual_obj,
                elapsed=pst.elapsed, status=pst.status, callback_vals=cb_val,
                V=V[:, :n].t(), lanczos_launches=pst.lanczos_launches,
                lanczos_ms=pst.lanczos_ms, lanczos_bytes=pst.lanczos_bytes,
                kernel_launches=pst.kernel_launches, graph_iterations=pst.graph_iterations)
    out, info = ren.restore(out, info)
    if return_trace:
        tr = trace[:pst.iterations].cpu().numpy()
        recs = [{f: float(r[i]) for i, f in enumerate(TRACE_FIELDS)} for r in tr]
        return out, recs, info
    if return_info:
        return out, info
    return out


CGAL_TRACE_FIELDS = ["t", "eig0", "obj_gap", "infeas_gap", "max_infeas", "primal_obj", "tr_X",
                     "dual_step"]


def cgal(sdp_state, n, m, trace_ub, beta0, max_iters, max_time, obj_gap_eps, infeas_gap_eps,
         max_infeas_eps, lanczos_inner_iterations, lanczos_max_restarts, subprob_eps,
         cond_exp_base=1.0, callback_fn=None, callback_static_args=None,
         callback_nonstatic_args=None, *, q0=None, precision=64, device="cuda",
         return_trace=False, return_info=False, instance=None, stream=None, log=None,
         renumber=False):
    """cgal() of solver/cgal.py:21-243 (same positional arguments), run by the
    device driver ``usbs_cgal_solve``.  Returns the updated SDPState; with
    ``return_trace`` also a list of per-iteration records, with
    ``return_info`` a dict of counters.  ``q0`` stands in for the reference's
    ``PRNGKey(0)`` Lanczos start vector (the same one every iteration)."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("usbs_gb300.cgal needs a CUDA device (GB300); none is visible")
    lib = _lib.load()
    _sigs(lib)
    dev = torch.device(device)
    sdp_state, q0, ren = _renumbered(sdp_state, n, q0, renumber, instance, dev)
    inst = instance if instance is not None else DeviceInstance(sdp_state, dev)
    ld = (n + 31) // 32 * 32
    f64 = torch.float64
    y = _to_dev(sdp_state.y, dev).clone()
    z = _to_dev(sdp_state.z, dev).clone()
    if sdp_state.Omega is not None:
        mode = 0
        sdim = int(shape_of(sdp_state.Omega)[1])
        Om = _dev_cols(sdp_state.Omega, n, ld, sdim, dev, f64)
        Pm = _dev_cols(sdp_state.P, n, ld, sdim, dev, f64)
        X = None
    elif sdp_state.X is not None:
        mode, sdim = 1, 0
        X = _to_dev(sdp_state.X, dev).clone()
        Pm = Om = None
    else:
        raise ValueError("cgal needs either Omega (sketch) or X (dense) in sdp_state")
    q0t = _to_dev(default_q0(n) if q0 is None else q0, dev)
    trace = torch.zeros((max(max_iters, 1), TRACE_WIDTH), dtype=f64, device=dev) \
        if return_trace else None
    prm = CgalParams()
    prm.trace_ub, prm.beta0, prm.max_iters = float(trace_ub), float(beta0), int(max_iters)
    prm.max_time = float(max_time)
    prm.obj_gap_eps, prm.infeas_gap_eps, prm.max_infeas_eps = (obj_gap_eps, infeas_gap_eps,
                                                               max_infeas_eps)
    prm.lanczos_inner_iterations = int(lanczos_inner_iterations)
    prm.lanczos_max_restarts = int(lanczos_max_restarts)
    prm.subprob_eps = float(subprob_eps)
    prm.cond_exp_base = float(cond_exp_base)
    prm.precision, prm.sketch_mode, prm.sketch_dim = int(precision), mode, sdim
    pst = UsbsState()
    pst.ld = ld
    pst.y, pst.z, pst.V = _ptr(y), _ptr(z), None
    pst.P, pst.Omega, pst.X, pst.q0, pst.trace = _ptr(Pm), _ptr(Om), _ptr(X), _ptr(q0t), _ptr(trace)
    pst.trace_capacity = int(max_iters) if return_trace else 0
    pst.debug = None
    pst.tr_X, pst.primal_obj = float(sdp_state.tr_X), float(sdp_state.primal_obj)
    prob = inst.c_struct()
    need = int(lib.usbs_cgal_workspace_bytes(ctypes.byref(prob), ctypes.byref(prm)))
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    cb_val = {}

    log_fn = print if log is True else log

    def _cb(_user, t):
        if callback_fn is not None and Om is not None:
            cb_val[t] = callback_fn(*ren.rows(Pm[:, :n].t(), Om[:, :n].t()),
                                    callback_static_args, callback_nonstatic_args)
        if log_fn is not None:
            rec = {f: float(pst.cond[i]) for i, f in enumerate(CGAL_TRACE_FIELDS)}
            log_fn(cgal_log_line(rec, float(sdp_state.SCALE_C), float(sdp_state.SCALE_X),
                                 cb_val.get(t)))

    ccb = CALLBACK(_cb)
    st = stream if stream is not None else torch.cuda.current_stream(dev)
    rc = lib.usbs_cgal_solve(ctypes.byref(prob), ctypes.byref(prm), ctypes.byref(pst), _ptr(ws),
                             need, ccb, None, int(st.cuda_stream))
    _lib.check(rc, "usbs_cgal_solve")
    if pst.status & 1:
        raise RuntimeError("usbs_cgal_solve: a device barrier timed out")
    out = SDPState(C=sdp_state.C, A_indices=sdp_state.A_indices, A_data=sdp_state.A_data,
                   b=sdp_state.b, b_ineq_mask=sdp_state.b_ineq_mask, X=X,
                   P=(Pm[:, :n].t() if mode == 0 else None), Omega=sdp_state.Omega, y=y, z=z,
                   tr_X=pst.tr_X, primal_obj=pst.primal_obj, SCALE_C=sdp_state.SCALE_C,
                   SCALE_X=sdp_state.SCALE_X, SCALE_A=sdp_state.SCALE_A)
    info = dict(iterations=pst.iterations, obj_gap=pst.obj_gap, infeas_gap=pst.infeas_gap,
                max_infeas=pst.max_infeas, elapsed=pst.elapsed, status=pst.status,
                callback_vals=cb_val, kernel_launches=pst.kernel_launches)
    out, info = ren.restore(out, info)
    if return_trace:
        tr = trace[:pst.iterations].cpu().numpy()
        recs = [{f: float(r[i]) for i, f in enumerate(CGAL_TRACE_FIELDS)} for r in tr]
        return out, recs, info
    if return_info:
        return out, info
    return out
