"""The solve service: results in a concurrent mix equal the same solves alone."""
import numpy as np
import pytest

from oracle import maxcut as omaxcut
from usbs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

SET = dict(rho=0.01, beta=0.25, k_curr=4, k_past=1, max_iters=4, max_time=np.inf,
           obj_gap_eps=-1.0, infeas_gap_eps=-1.0, max_infeas_eps=-1.0,
           lanczos_inner_iterations=32, lanczos_max_restarts=20, subprob_eps=1e-7,
           subprob_max_iters=100)


def _requests():
    out = []
    for i, (n, e) in enumerate([(80, 500), (150, 1200), (230, 2000), (300, 2600), (120, 900),
                                (200, 1500)]):
        st = omaxcut.initialize_state(wl.er_graph(n, e, 10 + i), 4)
        out.append((st, dict(n=n, m=n, trace_ub=2.0 * n, trace_factor=2.0, **SET)))
    return out


@pytest.mark.parametrize("precision", [64, 32])
def test_results_alone_equal_results_in_the_mix(cuda, precision):
    from usbs_gb300 import solver
    from usbs_gb300.serving import SolveRequest, SolverService
    reqs = _requests()
    alone = [solver.usbs(st, precision=precision, **kw) for st, kw in reqs]
    with SolverService(max_slots=4, reserve_bytes=1 << 30) as svc:
        handles = [svc.submit(SolveRequest(st, precision=precision, **kw)) for st, kw in reqs]
        mixed = [h.wait(600) for h in handles]
    for a, b in zip(alone, mixed):
        np.testing.assert_allclose(b.y.cpu().numpy(), a.y.cpu().numpy(), rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(b.z.cpu().numpy(), a.z.cpu().numpy(), rtol=1e-12, atol=1e-14)
        assert abs(b.primal_obj - a.primal_obj) <= 1e-12 * max(1.0, abs(a.primal_obj))
    starts = sorted(h.start for h in handles)
    finishes = sorted(h.finish for h in handles)
    assert starts[1] < finishes[0]             # solves overlapped in time
