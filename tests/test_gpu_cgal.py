"""GPU parity of the device CGAL iteration (solver/cgal.py:21-243) against the
FP64 oracle."""
import numpy as np
import pytest

from oracle import cgal as ocgal
from oracle import maxcut as omaxcut
from oracle import rng as orng
from usbs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

KEYS = ["obj_gap", "infeas_gap", "max_infeas", "primal_obj", "tr_X", "dual_step"]


def _rel(a, b):
    return abs(a - b) / max(1.0, abs(a), abs(b))


def _run_both(W, iters, precision, sketch_dim=4, restarts=200, tol=1e-10):
    from usbs_gb300 import solver
    st = omaxcut.initialize_state(W, sketch_dim)
    n = st.C.shape[0]
    q0 = orng.default_q0(n)
    tr = 1.0 * n * st.SCALE_X
    otr = []
    oout, ofin = ocgal.cgal(st, n, n, tr, 1.0, iters, np.inf, -1.0, -1.0, -1.0, min(n, 32),
                            restarts, tol, q0=q0, trace=otr)
    gout, gtr, info = solver.cgal(st, n, n, tr, 1.0, iters, np.inf, -1.0, -1.0, -1.0, min(n, 32),
                                  restarts, tol, 1.0, None, None, None, q0=q0,
                                  precision=precision, return_trace=True)
    return oout, otr, gout, gtr, info


def test_cgal_fp64_trace_matches_oracle(cuda):
    """Converged eigenvectors: every iteration matches the oracle closely (CGAL
    has no interior-point tail to amplify rounding)."""
    W = wl.er_graph(150, 1200, 4)
    oout, otr, gout, gtr, info = _run_both(W, 12, 64)
    assert info["status"] == 0 and info["iterations"] == 12
    for a, b in zip(otr, gtr):
        assert abs(a["eig0"] - b["eig0"]) <= 1e-9 * max(1.0, abs(a["eig0"])), a["t"]
        for key in KEYS:
            assert _rel(a[key], b[key]) < 1e-8, (a["t"], key, a[key], b[key])
    # vectors: 1e-8 relative to their largest entry (entries near zero carry the
    # absolute error of the large ones)
    for g, o in ((gout.y, oout.y), (gout.z, oout.z), (gout.P, oout.P)):
        o = np.asarray(o)
        np.testing.assert_allclose(g.cpu().numpy(), o, rtol=0, atol=1e-8 * np.abs(o).max())


def test_cgal_dense_X_mode(cuda):
    W = wl.er_graph(80, 500, 5)
    oout, otr, gout, gtr, info = _run_both(W, 6, 64, sketch_dim=-1)
    for a, b in zip(otr, gtr):
        assert _rel(a["primal_obj"], b["primal_obj"]) < 1e-8
    np.testing.assert_allclose(gout.X.cpu().numpy(), oout.X, rtol=0,
                               atol=1e-8 * np.abs(oout.X).max())


def test_cgal_fp32_close_to_fp64(cuda):
    # a generic spectrum: on a torus spin glass the smallest eigenvalues are
    # nearly degenerate and the two precisions may pick different vectors of
    # the same eigenspace
    W = wl.er_graph(200, 1500, 6)
    oout, otr, gout, gtr, info = _run_both(W, 8, 32, tol=1e-6)
    assert info["status"] == 0
    # FP32 Ritz vectors (residual 1e-6) carry ~1e-4 relative error into v^T C v
    for a, b in zip(otr, gtr):
        assert _rel(a["primal_obj"], b["primal_obj"]) < 1e-3, (a["t"], a["primal_obj"],
                                                                 b["primal_obj"])


def test_cgal_stops_at_first_iteration_meeting_eps(cuda):
    from usbs_gb300 import solver
    W = wl.er_graph(60, 500, 2)
    st = omaxcut.initialize_state(W, 4)
    n, eps = 60, 5e-2
    out, tr, info = solver.cgal(st, n, n, 1.0 * n * st.SCALE_X, 1.0, 3000, np.inf, eps, eps, eps,
                                32, 20, 1e-7, 1.0, None, None, None, return_trace=True)
    assert info["iterations"] < 3000
    last = tr[-1]
    assert last["obj_gap"] <= eps and last["infeas_gap"] <= eps and last["max_infeas"] <= eps
    for r in tr[:-1]:
        assert r["obj_gap"] > eps or r["infeas_gap"] > eps or r["max_infeas"] > eps
