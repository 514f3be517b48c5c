"""Failure detection on the device, without a GPU fault: bounded waits that run
out end in a status word, non-finite input is reported, and the service
rejects or withdraws requests instead of waiting on them forever.  After each
case the context stays usable (a normal eigsh call follows)."""
import ctypes

import numpy as np
import pytest

from oracle import maxcut as omaxcut
from usbs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

ST_BARRIER_TIMEOUT, ST_NONFINITE = 1, 2


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _small_problem(device):
    from usbs_gb300.problem import DeviceProblem, layout
    st = omaxcut.initialize_state(wl.er_graph(300, 3000, 3), 4)
    n = st.C.shape[0]
    return DeviceProblem(layout(st.C, st.A_data, st.A_indices, m=n), device), n


def _eigsh(device, y, precision=64, n_override=None):
    from usbs_gb300 import api
    from usbs_gb300.rng import default_q0
    prob, n = _small_problem(device)
    return api.eigsh_smallest(n, prob, None, None, y(n) if callable(y) else y, default_q0(n), 5,
                              32, 5, 1e-7, c_scale=-1.0, precision=precision, return_info=True)


def _context_still_usable(device):
    vals, _, info = _eigsh(device, lambda n: np.zeros(n))
    assert info.status == 0 and np.all(np.isfinite(vals.cpu().numpy()))


@pytest.mark.parametrize("which", [0, 1])      # 0: team barrier, 1: mbarrier
def test_bounded_wait_times_out_into_the_status_word(cuda, which):
    import torch
    from usbs_gb300 import _lib
    lib = _lib.load()
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    counters = torch.zeros(2, dtype=torch.int32, device=cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
    rc = lib.usbs_selftest_wait_limits(which, 4, 2_000_000, _ptr(counters), _ptr(status), stream)
    assert rc == 0, lib.usbs_last_error().decode()
    torch.cuda.synchronize(cuda)
    assert int(status.item()) == ST_BARRIER_TIMEOUT
    _context_still_usable(cuda)


def test_selftest_rejects_unbounded_limits(cuda):
    from usbs_gb300 import _lib
    lib = _lib.load()
    null = ctypes.c_void_p(0)
    assert lib.usbs_selftest_wait_limits(0, 4, 10 ** 12, null, null, null) == -2
    assert lib.usbs_selftest_wait_limits(2, 4, 10 ** 6, null, null, null) == -2


@pytest.mark.parametrize("precision", [64, 32])
def test_nan_in_the_dual_vector_is_reported(cuda, precision):
    def y(n):
        v = np.zeros(n)
        v[7] = np.nan
        return v
    vals, _, info = _eigsh(cuda, y, precision)
    assert info.status & ST_NONFINITE
    assert info.restarts == 1                   # the call ends at the first restart
    _context_still_usable(cuda)


def test_nan_in_the_solve_is_reported(cuda):
    from usbs_gb300 import solver
    st = omaxcut.initialize_state(wl.er_graph(200, 1500, 2), 4)
    n = st.C.shape[0]
    y = np.zeros(n)
    y[3] = np.nan
    st = st._replace(y=y)
    out, info = solver.usbs(st, n, n, 2.0 * n, 2.0, 0.01, 0.25, 4, 1, 20, np.inf, 1e-7, 1e-7, 1e-7,
                            32, 10, 1e-7, 100, precision=64, return_info=True)
    assert info["status"] & ST_NONFINITE
    assert info["iterations"] == 1              # NaN gaps stop the loop, as in the reference
    _context_still_usable(cuda)


def _request(n, e, seed, iters):
    from usbs_gb300.serving import SolveRequest
    st = omaxcut.initialize_state(wl.er_graph(n, e, seed), 4)
    return SolveRequest(st, precision=32, n=n, m=n, trace_ub=2.0 * n, trace_factor=2.0,
                        rho=0.01, beta=0.25, k_curr=4, k_past=1, max_iters=iters,
                        max_time=np.inf, obj_gap_eps=-1.0, infeas_gap_eps=-1.0,
                        max_infeas_eps=-1.0, lanczos_inner_iterations=32,
                        lanczos_max_restarts=10, subprob_eps=1e-7, subprob_max_iters=100)


def test_service_rejects_a_request_larger_than_its_budget(cuda):
    from usbs_gb300.serving import SolverService
    free = 4 << 20                              # the small request takes < 1 MB, the big ~7 MB
    with SolverService(max_slots=2, reserve_bytes=0, mem_info=lambda: (free, free)) as svc:
        small = svc.submit(_request(100, 600, 1, 2))
        big = svc.submit(_request(3000, 60000, 2, 2))
        assert big.done.is_set()
        with pytest.raises(MemoryError):
            big.wait(1)
        assert small.wait(600) is not None      # the small one still runs


def test_service_cancels_a_queued_request(cuda):
    from usbs_gb300.serving import RequestCancelled, SolverService
    with SolverService(max_slots=1, reserve_bytes=1 << 30) as svc:
        first = svc.submit(_request(400, 4000, 3, 40))
        second = svc.submit(_request(120, 800, 4, 2))
        assert svc.cancel(second)               # the only slot is taken by `first`
        with pytest.raises(RequestCancelled):
            second.wait(1)
        assert first.wait(600) is not None
        assert not svc.cancel(first)            # finished requests cannot be withdrawn
