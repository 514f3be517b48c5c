"""Continuous-batching solve service: many SDP instances resident on one GPU.

Requests (an SDPState plus the usbs() arguments) are admitted as a slot and enough
HBM free up, so requests that arrive while others run start without waiting for the
batch to drain. Each admitted request runs ``usbs()`` to completion on its own CUDA
stream, driven by its own host thread. ctypes releases the GIL during the call, so
the solves' kernels overlap on the device.

A problem whose Lanczos basis fits in one thread-block cluster's shared memory
(``usbs_lanczos_kernel`` = 1) uses cluster-scheduled kernels only, and any number
of those run side by side; so does a problem on the stream path (kind 2, the
largest ones), whose kernels are ordinary launches that never wait on each
other. By default the service runs every larger problem on the stream path
(``lanczos_path=2``), so no request ever needs the GPU to itself. With
``lanczos_path=0`` a mid-size problem uses the cooperative team kernel (kind 0),
whose grid is sized for the whole GPU and must be co-resident; such a request
runs alone: it waits for the running solves to finish, and nothing else is
admitted until it is done.

Warm starts from resident state: a request may name an earlier request
(``warm_from``) and a transform (``warm_start(parent_result, cold_state) ->
SDPState``, e.g. the MaxCut implicit warm start). It is admitted once its
parent has finished; the transform then builds its initial state from the
parent's result, which is still on the device, without a host round trip.

Admission by memory: the service owns the HBM that was free when it started,
less ``reserve_bytes``. A request's device footprint (its state and its
``usbs_solve`` workspace) is computed exactly at submission. The request is
admitted only if that footprint plus the footprints of the running solves fits in
the budget. A request whose footprint alone exceeds the budget can never run: it
is rejected at submission (``wait()`` raises ``MemoryError``) instead of
waiting forever. A request that is still queued can be withdrawn with
``SolverService.cancel()`` (``wait()`` then raises ``RequestCancelled``); a
solve that has started runs to its end.

Concurrency on the device: every running solve uses two CUDA streams, and CUDA
maps streams onto CUDA_DEVICE_MAX_CONNECTIONS hardware queues (8 by default),
where a kernel waits behind whatever heads its queue. A process that runs many
slots should set CUDA_DEVICE_MAX_CONNECTIONS=32 before CUDA is initialised (the
library cannot change it afterwards). Measured on the 1,024-request serving
stream (n up to 50,000): 17.2 solves/s, p50 5.6 s, p99 7.5 s with 16 slots and
8 queues; 18.3 solves/s, p50 3.6 s, p99 4.9 s with 32 slots and 32 queues.

The reference has no serving layer. Each result is the same as a solve of that
request alone: the kernels are deterministic and share no state between solves.
"""
import collections
import ctypes
import threading
import time

from . import _lib, solver
from .arrays import shape_of

__all__ = ["SolveRequest", "SolverService", "Admission", "footprint_bytes", "RequestCancelled"]


class RequestCancelled(RuntimeError):
    """Raised by SolveRequest.wait() for a request withdrawn before it started."""


class Admission:
    """Slot and memory accounting of the service (host logic only)."""

    def __init__(self, budget_bytes, max_slots):
        self.budget = int(budget_bytes)
        self.free_slots = int(max_slots)
        self.running = 0
        self.running_bytes = 0
        self.exclusive = False

    def ever_fits(self, footprint):
        """False for a request that exceeds the whole budget (it would never start)."""
        return footprint <= self.budget

    def admissible(self, footprint, exclusive):
        if self.exclusive or self.free_slots == 0:
            return False
        if exclusive and self.running > 0:
            return False
        return self.running_bytes + footprint <= self.budget

    def start(self, footprint, exclusive):
        self.free_slots -= 1
        self.running += 1
        self.running_bytes += footprint
        self.exclusive = self.exclusive or exclusive

    def finish(self, footprint, exclusive):
        self.free_slots += 1
        self.running -= 1
        self.running_bytes -= footprint
        if exclusive:
            self.exclusive = False

    def pick(self, queue):
        """Index of the first admissible request in arrival order, or None.
        Entries are (footprint, exclusive) or (footprint, exclusive, ready); a
        request that is not ready (its warm-start parent still running) or
        does not fit does not block the ones behind it, except an exclusive
        one, which holds the line until the GPU drains."""
        for i, e in enumerate(queue):
            footprint, exclusive = e[0], e[1]
            if len(e) > 2 and not e[2]:
                continue
            if self.admissible(footprint, exclusive):
                return i
            if exclusive:
                return None
        return None


class SolveRequest:
    """One usbs() call.  ``kwargs`` are usbs()'s arguments after ``sdp_state``
    (n, m, trace_ub, ... as keywords); ``precision`` 32 or 64.  ``host_layout``
    (optional): the problem's layout prepared ahead (solver.host_problem_layout),
    so that submit() does no host work on it."""

    def __init__(self, sdp_state, precision=32, tag=None, warm_from=None, warm_start=None,
                 host_layout=None, **kwargs):
        self.sdp_state = sdp_state
        self.host_layout = host_layout
        self.warm_from = warm_from
        self.warm_start = warm_start
        self.warmed = False
        self.precision = int(precision)
        self.kwargs = kwargs
        self.tag = tag
        self.arrival = None
        self.start = None
        self.finish = None
        self.result = None
        self.info = None
        self.error = None
        self.done = threading.Event()
        self.footprint = None
        self.exclusive = False

    @property
    def latency(self):
        return None if self.finish is None else self.finish - self.arrival

    def wait(self, timeout=None):
        self.done.wait(timeout)
        if self.error is not None:
            raise self.error
        return self.result


def footprint_bytes(host_layout, k, sketch_dim, params_struct, lib):
    """Device bytes one solve holds: its problem layout, constraint vectors,
    iterate state and usbs_solve workspace."""
    n, m = host_layout.n, host_layout.m
    ld = (n + 31) // 32 * 32
    prob = solver.UsbsProblem()
    prob.n, prob.m, prob.nnz, prob.num_triples = n, m, host_layout.nnz, host_layout.num_triples
    ws = int(lib.usbs_solve_workspace_bytes(ctypes.byref(prob), ctypes.byref(params_struct)))
    lay = sum(getattr(host_layout, f).nbytes for f in solver.DeviceProblem.FIELDS)
    state = 8 * (3 * m + 2 * m + ld * k + 2 * ld * max(sketch_dim, 1) + ld)
    return ws + lay + state


class SolverService:
    """``submit()`` requests; ``max_slots`` solves run at once.
    ``lanczos_rows_per_cta``: the cluster Lanczos packing of requests that do
    not set their own (0: the library's single-solve choice)."""

    def __init__(self, device="cuda", max_slots=8, reserve_bytes=2 << 30, mem_info=None,
                 lanczos_rows_per_cta=0, lanczos_path=2):
        import torch
        self.device = torch.device(device)
        self.lanczos_path = int(lanczos_path)
        self.max_slots = int(max_slots)
        self.rows_per_cta = int(lanczos_rows_per_cta)
        self.reserve = int(reserve_bytes)
        mem_info = mem_info or (lambda: torch.cuda.mem_get_info(self.device))
        free, _total = mem_info()
        self._adm = Admission(free - self.reserve, self.max_slots)
        self._cv = threading.Condition()
        self._queue = collections.deque()
        self._stop = False
        self._streams = [torch.cuda.Stream(self.device) for _ in range(self.max_slots)]
        self._free_streams = list(range(self.max_slots))
        self._threads = [threading.Thread(target=self._worker, daemon=True)
                         for _ in range(self.max_slots)]
        for t in self._threads:
            t.start()

    # ------------------------------------------------------------ public
    def submit(self, req):
        lib = _lib.load()
        solver._sigs(lib)
        kw = req.kwargs
        host = req.host_layout if req.host_layout is not None else \
            solver.host_problem_layout(req.sdp_state)
        req._host_layout = host
        n = kw["n"]
        k = kw["k_curr"] + kw["k_past"]
        sdim = 0 if req.sdp_state.Omega is None else int(shape_of(req.sdp_state.Omega)[1])
        prm = solver.UsbsParams()
        prm.k_curr, prm.k_past = kw["k_curr"], kw["k_past"]
        prm.lanczos_inner_iterations = kw["lanczos_inner_iterations"]
        prm.precision = req.precision
        prm.sketch_mode = 0 if sdim else (1 if req.sdp_state.X is not None else 2)
        prm.sketch_dim = sdim
        prm.lanczos_path = self.lanczos_path
        req.footprint = footprint_bytes(host, k, sdim, prm, lib)
        # only the cooperative team kernel (kind 0) needs the GPU to itself
        req.exclusive = self.lanczos_path != 2 and lib.usbs_lanczos_kernel(
            n, kw["lanczos_inner_iterations"], req.precision) == 0
        req.arrival = time.perf_counter()
        if not self._adm.ever_fits(req.footprint):
            req.error = MemoryError(f"request needs {req.footprint} bytes of device memory; the "
                                    f"service budget is {self._adm.budget}")
            req.finish = req.arrival
            req._host_layout = None
            req.done.set()
            return req
        with self._cv:
            self._queue.append(req)
            self._cv.notify_all()
        return req

    def cancel(self, req):
        """Withdraw a queued request (True); False once it has started or ended."""
        with self._cv:
            try:
                self._queue.remove(req)
            except ValueError:
                return False
        req.error = RequestCancelled("request cancelled before it started")
        req.finish = time.perf_counter()
        req._host_layout = None
        req.done.set()
        return True

    def shutdown(self):
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.shutdown()

    # ------------------------------------------------------------ scheduling
    def _next(self):
        """Called with the lock held: pop the next admissible request."""
        i = self._adm.pick([(r.footprint, r.exclusive,
                             r.warm_from is None or r.warm_from.done.is_set())
                            for r in self._queue])
        if i is None:
            return None
        req = self._queue[i]
        del self._queue[i]
        return req

    def _worker(self):
        import torch
        while True:
            with self._cv:
                while True:
                    if self._stop and not self._queue:
                        return
                    req = self._next()
                    if req is not None:
                        break
                    self._cv.wait(0.05)
                sidx = self._free_streams.pop()
                self._adm.start(req.footprint, req.exclusive)
            stream = self._streams[sidx]
            req.start = time.perf_counter()
            try:
                with torch.cuda.stream(stream):
                    state, host_layout = req.sdp_state, req._host_layout
                    kw = dict(req.kwargs)
                    parent = req.warm_from
                    if parent is not None and parent.result is not None and req.warm_start:
                        # the parent's result is still on the device
                        state = req.warm_start(parent.result, req.sdp_state)
                        host_layout = None
                        req.warmed = True
                        kw["trace_ub"] = kw["trace_factor"] * kw["n"] * state.SCALE_X
                    inst = solver.DeviceInstance(state, self.device, host_layout=host_layout)
                    if self.rows_per_cta:
                        kw.setdefault("lanczos_rows_per_cta", self.rows_per_cta)
                    kw.setdefault("lanczos_path", self.lanczos_path)
                    out, info = solver.usbs(state, precision=req.precision,
                                            device=self.device, return_info=True,
                                            instance=inst, stream=stream, **kw)
                    stream.synchronize()
                    del inst
                req.result, req.info = out, info
            except Exception as exc:   # reported to the caller through wait()
                req.error = exc
            req.finish = time.perf_counter()
            with self._cv:
                self._adm.finish(req.footprint, req.exclusive)
                self._free_streams.append(sidx)
                self._cv.notify_all()
            req._host_layout = None
            req.done.set()
