"""GPU parity of the device USBS iteration against the FP64 oracle."""
import numpy as np
import pytest

from oracle import maxcut as omaxcut
from oracle import rng as orng
from oracle import usbs as ousbs
from usbs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

S = wl.MAXCUT_SETTINGS
KEYS = ["primal_obj", "obj_ub", "lb_spec_est", "pen_dual_obj", "cand_pen_dual_obj", "eta",
        "obj_gap", "infeas_gap", "max_infeas", "tr_X"]


def _run_both(W, iters, precision, sketch_dim=10, k_curr=10, k_past=1):
    from usbs_gb300 import solver
    st = omaxcut.initialize_state(W, sketch_dim)
    n = st.C.shape[0]
    q0 = orng.default_q0(n)
    mL = min(n, 32)
    otr = []
    oout, ofin = ousbs.usbs(st, n, n, 2.0 * n, 2.0, S["rho"], S["beta"], k_curr, k_past, iters,
                            np.inf, -1.0, -1.0, -1.0, mL, S["lanczos_max_restarts"],
                            S["subprob_eps"], S["subprob_max_iters"], q0=q0, trace=otr)
    gout, gtr, info = solver.usbs(st, n, n, 2.0 * n, 2.0, S["rho"], S["beta"], k_curr, k_past,
                                  iters, np.inf, -1.0, -1.0, -1.0, mL,
                                  S["lanczos_max_restarts"], S["subprob_eps"],
                                  S["subprob_max_iters"], 1.0, None, None, None, q0=q0,
                                  precision=precision, return_trace=True)
    return st, oout, ofin, otr, gout, gtr, info


def _rel(a, b):
    return abs(a - b) / max(1.0, abs(a), abs(b))


def test_usbs_fp64_trace_matches_oracle(cuda):
    W = wl.er_graph(300, 4000, 7)
    st, oout, ofin, otr, gout, gtr, info = _run_both(W, 8, 64)
    assert info["status"] == 0 and info["iterations"] == 8
    for a, b in zip(otr, gtr):
        assert bool(a["descent"]) == bool(b["descent"]), a["t"]
        for key in KEYS:
            assert _rel(a[key], b[key]) < 1e-8, (a["t"], key, a[key], b[key])
    np.testing.assert_allclose(gout.y.cpu().numpy(), oout.y, rtol=1e-7, atol=1e-7)
    np.testing.assert_allclose(gout.z.cpu().numpy(), oout.z, rtol=1e-7, atol=1e-7)
    np.testing.assert_allclose(gout.P.cpu().numpy(), oout.P, rtol=1e-6, atol=1e-7)
    assert _rel(gout.primal_obj, oout.primal_obj) < 1e-8


def test_usbs_fp32_mixed_close_to_fp64_oracle(cuda):
    W = wl.torus_graph(30, 1)
    st, oout, ofin, otr, gout, gtr, info = _run_both(W, 12, 32)
    assert info["status"] == 0
    for a, b in zip(otr, gtr):
        assert _rel(a["primal_obj"], b["primal_obj"]) < 1e-4, (a["t"], a["primal_obj"],
                                                                b["primal_obj"])


def test_usbs_dense_X_mode(cuda):
    W = wl.er_graph(120, 900, 9)
    st, oout, ofin, otr, gout, gtr, info = _run_both(W, 5, 64, sketch_dim=-1, k_curr=4, k_past=1)
    for a, b in zip(otr, gtr):
        assert _rel(a["primal_obj"], b["primal_obj"]) < 1e-8
    np.testing.assert_allclose(gout.X.cpu().numpy(), oout.X, rtol=1e-7, atol=1e-8)


def test_usbs_stops_on_gap(cuda):
    """cond_func (solver/usbs.py:533-540): stops as soon as all three gaps are below eps."""
    from usbs_gb300 import solver
    W = wl.er_graph(60, 500, 2)
    st = omaxcut.initialize_state(W, 4)
    n = 60
    out, info = solver.usbs(st, n, n, 2.0 * n, 2.0, 0.01, 0.25, 3, 1, 400, np.inf, 1e-2, 1e-2,
                            1e-2, 32, 10, 1e-7, 100, 1.0, None, None, None, return_info=True)
    assert info["obj_gap"] <= 1e-2 and info["infeas_gap"] <= 1e-2 and info["max_infeas"] <= 1e-2
    assert info["iterations"] < 400
