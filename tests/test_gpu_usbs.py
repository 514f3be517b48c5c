"""GPU parity of the device USBS iteration against the FP64 oracle."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import maxcut as omaxcut
from oracle import rng as orng
from oracle import usbs as ousbs
from usbs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

S = wl.MAXCUT_SETTINGS
KEYS = ["primal_obj", "obj_ub", "lb_spec_est", "pen_dual_obj", "cand_pen_dual_obj", "eta",
        "obj_gap", "infeas_gap", "max_infeas", "tr_X"]


def _run_both(W, iters, precision, sketch_dim=10, k_curr=10, k_past=1, eps=1e-7, restarts=10):
    from usbs_gb300 import solver
    st = omaxcut.initialize_state(W, sketch_dim)
    n = st.C.shape[0]
    q0 = orng.default_q0(n)
    mL = min(n, 32)
    otr = []
    oout, ofin = ousbs.usbs(st, n, n, 2.0 * n, 2.0, S["rho"], S["beta"], k_curr, k_past, iters,
                            np.inf, -1.0, -1.0, -1.0, mL, restarts, eps, S["subprob_max_iters"],
                            q0=q0, trace=otr)
    gout, gtr, info = solver.usbs(st, n, n, 2.0 * n, 2.0, S["rho"], S["beta"], k_curr, k_past,
                                  iters, np.inf, -1.0, -1.0, -1.0, mL, restarts, eps,
                                  S["subprob_max_iters"], 1.0, None, None, None, q0=q0,
                                  precision=precision, return_trace=True)
    return st, oout, ofin, otr, gout, gtr, info


def _rel(a, b):
    return abs(a - b) / max(1.0, abs(a), abs(b))


def test_usbs_fp64_trace_matches_oracle(cuda):
    """Plain FP64 device path vs the FP64 oracle, iteration by iteration, on a
    configuration whose eigenproblems are resolved (Lanczos converges, so the
    bundle basis is determined by the problem and not by rounding)."""
    W = wl.er_graph(300, 4000, 7)
    st, oout, ofin, otr, gout, gtr, info = _run_both(W, 5, 64, k_curr=4, k_past=1, eps=1e-9,
                                                     restarts=200)
    assert info["status"] == 0 and info["iterations"] == 5
    # The interior-point solves stop at mu <= eps; within a few ulps of that
    # floor the number of IPM steps is decided by rounding, so the values are
    # compared, not the step counts.  Differences grow ~10x per outer iteration
    # (the bundle trajectory amplifies them), hence the looser later bound.
    for a, b in zip(otr, gtr):
        assert bool(a["descent"]) == bool(b["descent"]), a["t"]
        tol = (1e-7, 1e-6, 1e-5)[a["t"]] if a["t"] < 3 else 1e-4
        for key in KEYS:
            if key == "eta" and a["t"] == 0:
                # z_bar = 0 and bar_primal_obj = 0 at t = 0: eta is degenerate in the
                # subproblem and its value does not enter the iteration
                continue
            assert _rel(a[key], b[key]) < tol, (a["t"], key, a[key], b[key])
    np.testing.assert_allclose(gout.y.cpu().numpy(), oout.y, rtol=1e-3, atol=1e-4)
    np.testing.assert_allclose(gout.z.cpu().numpy(), oout.z, rtol=1e-3, atol=1e-4)
    assert _rel(gout.primal_obj, oout.primal_obj) < 1e-4


def test_usbs_fp64_first_iteration_1e9(cuda):
    """The first outer iteration reproduces the FP64 oracle to 1e-9 relative."""
    W = wl.er_graph(300, 4000, 7)
    st, oout, ofin, otr, gout, gtr, info = _run_both(W, 1, 64, k_curr=4, k_past=1, eps=1e-9,
                                                     restarts=200)
    for key in ("primal_obj", "obj_ub", "lb_spec_est", "pen_dual_obj", "cand_pen_dual_obj",
                "tr_X"):
        assert _rel(otr[0][key], gtr[0][key]) < 1e-9, (key, otr[0][key], gtr[0][key])


def test_usbs_fp64_reference_settings_first_step(cuda):
    """With the reference's default Lanczos budget the trailing Ritz vectors are
    unconverged; the first step still agrees to their sensitivity (~1e-4)."""
    W = wl.er_graph(300, 4000, 7)
    st, oout, ofin, otr, gout, gtr, info = _run_both(W, 1, 64)
    assert _rel(otr[0]["primal_obj"], gtr[0]["primal_obj"]) < 1e-3
    assert _rel(otr[0]["lb_spec_est"], gtr[0]["lb_spec_est"]) < 1e-3


def test_usbs_fp32_mixed_step_close_to_fp64(cuda):
    """FP32 Lanczos + FP64 rest vs the FP64 oracle on a resolved configuration."""
    W = wl.torus_graph(30, 1)
    st, oout, ofin, otr, gout, gtr, info = _run_both(W, 3, 32, k_curr=4, k_past=1, eps=1e-9,
                                                     restarts=100)
    assert info["status"] == 0
    # FP32 Ritz vectors are accurate to ~1e-6; the bundle trajectory amplifies
    # such differences from the second step on, so compare the first
    for a, b in list(zip(otr, gtr))[:1]:
        assert _rel(a["primal_obj"], b["primal_obj"]) < 1e-3, (a["t"], a["primal_obj"],
                                                                b["primal_obj"])


def test_usbs_dense_X_mode(cuda):
    W = wl.er_graph(120, 900, 9)
    st, oout, ofin, otr, gout, gtr, info = _run_both(W, 2, 64, sketch_dim=-1, k_curr=4,
                                                     k_past=1, eps=1e-9, restarts=200)
    for a, b in zip(otr, gtr):
        assert _rel(a["primal_obj"], b["primal_obj"]) < (1e-7, 1e-6)[a["t"]]
    np.testing.assert_allclose(gout.X.cpu().numpy(), oout.X, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("precision", [64, 32])
def test_usbs_stops_at_first_iteration_meeting_eps(cuda, precision):
    """cond_func (solver/usbs.py:533-540): the loop stops at the first iteration
    whose obj_gap, infeas_gap and max_infeas are all at or below their eps."""
    from usbs_gb300 import solver
    W = wl.er_graph(60, 500, 2)
    st = omaxcut.initialize_state(W, 4)
    n, eps = 60, 5e-2
    out, tr, info = solver.usbs(st, n, n, 2.0 * n, 2.0, 0.01, 0.25, 3, 1, 3000, np.inf, eps, eps,
                                eps, 32, 10, 1e-7, 100, 1.0, None, None, None,
                                precision=precision, return_trace=True)
    assert info["iterations"] < 3000
    last = tr[-1]
    assert last["obj_gap"] <= eps and last["infeas_gap"] <= eps and last["max_infeas"] <= eps
    for r in tr[:-1]:
        assert r["obj_gap"] > eps or r["infeas_gap"] > eps or r["max_infeas"] > eps


def test_usbs_precisions_agree_on_solution(cuda):
    """FP64 and mixed precision reach the same objective at the same gap."""
    from usbs_gb300 import solver
    W = wl.er_graph(80, 800, 3)
    st = omaxcut.initialize_state(W, 4)
    n, eps = 80, 2e-2
    vals = []
    for precision in (64, 32):
        out, info = solver.usbs(st, n, n, 2.0 * n, 2.0, 0.01, 0.25, 3, 1, 4000, np.inf, eps, eps,
                                eps, 32, 10, 1e-7, 100, 1.0, None, None, None,
                                precision=precision, return_info=True)
        assert info["obj_gap"] <= eps, info
        vals.append(out.primal_obj)
    assert abs(vals[0] - vals[1]) / abs(vals[0]) < 2 * eps


def test_usbs_qap_fp64_trace_matches_oracle(cuda):
    """QAP relaxation (general triples, '<=' rows, the upsilon alternating
    minimisation of solver/usbs.py:359-433) on the device vs the FP64 oracle."""
    from oracle import qap as oqap
    from usbs_gb300 import solver
    l = 5
    D, Wf = wl.qap_instance(l, 0, grid=5)
    st = oqap.initialize_state(D, Wf, 6)
    n, m = st.C.shape[0], st.b.shape[0]
    assert np.any(st.b_ineq_mask > 0)
    trace_factor, rho = 2.0, 0.005
    trace_ub = trace_factor * float(l + 1) * st.SCALE_X
    q0 = orng.default_q0(n)
    mL = min(n, 32)
    iters = 4
    otr = []
    oout, ofin = ousbs.usbs(st, n, m, trace_ub, trace_factor, rho, 0.25, 2, 0, iters, np.inf,
                            -1.0, -1.0, -1.0, mL, 300, 1e-9, 100, q0=q0, trace=otr)
    gout, gtr, info = solver.usbs(st, n, m, trace_ub, trace_factor, rho, 0.25, 2, 0, iters,
                                  np.inf, -1.0, -1.0, -1.0, mL, 300, 1e-9, 100, 1.0, None, None,
                                  None, q0=q0, precision=64, return_trace=True)
    assert info["status"] == 0 and info["iterations"] == iters
    for a, b in zip(otr, gtr):
        tol = (1e-7, 1e-6, 1e-5)[a["t"]] if a["t"] < 3 else 1e-4
        for key in ("primal_obj", "obj_ub", "pen_dual_obj", "obj_gap", "infeas_gap",
                    "max_infeas", "tr_X"):
            assert _rel(a[key], b[key]) < tol, (a["t"], key, a[key], b[key])
    np.testing.assert_allclose(gout.y.cpu().numpy(), oout.y, rtol=1e-3, atol=1e-5)


def test_usbs_isolated_nodes_first_iteration(cuda):
    """Resolved configuration (Lanczos to 1e-9), one outer iteration, on a graph
    with many isolated nodes (zero rows of C; the pattern keeps only the
    constraint diagonal there).  The 131 isolated nodes all get the same
    y_cand entry, so -C + A*(y_cand) has a 131-fold eigenvalue that Lanczos
    resolves only to its tolerance, in the oracle as here: 1e-7."""
    W = wl.er_graph(300, 120, 9)
    assert (np.asarray(W.sum(axis=1)).ravel() == 0).sum() > 100
    st, oout, ofin, otr, gout, gtr, info = _run_both(W, 1, 64, k_curr=4, k_past=1, eps=1e-9,
                                                     restarts=200)
    assert info["status"] == 0
    for key in ("primal_obj", "obj_ub", "lb_spec_est", "pen_dual_obj", "cand_pen_dual_obj",
                "tr_X"):
        assert _rel(otr[0][key], gtr[0][key]) < 1e-7, (key, otr[0][key], gtr[0][key])


def _hub_graph(seed=0):
    """12 hubs with 10, 12, ..., 32 leaves of their own and 40 random
    leaf-leaf edges: the 12 smallest eigenvalues of -C are about 0.5 apart."""
    rows, cols, nxt = [], [], 12
    for h in range(12):
        for _ in range(10 + 2 * h):
            rows.append(h)
            cols.append(nxt)
            nxt += 1
    rs = np.random.default_rng(seed)
    for _ in range(40):
        a, b = rs.integers(12, nxt, 2)
        if a != b:
            rows.append(a)
            cols.append(b)
    W = sp.coo_matrix((np.ones(len(rows)), (rows, cols)), shape=(nxt, nxt))
    return sp.csr_matrix(((W + W.T) > 0).astype(float))


def test_usbs_largest_bundle_first_iteration_1e9(cuda):
    """k = k_curr + k_past = 12, the largest bundle the IPM takes (svec
    dimension 78), one outer iteration at 1e-9 on the quantities the IPMs
    determine.  eigsh_smallest returns alpha[:num_desired] after the
    saved-first reordering (solver/lanczos.py:224-227, 280-281): past k_left + 1
    of them these are Ritz values from the top of the spectrum, chosen by
    argmax of the gap ratio.  On a well separated spectrum that choice does not
    depend on rounding, so both sides take the same start vectors."""
    W = _hub_graph()
    st, oout, ofin, otr, gout, gtr, info = _run_both(W, 1, 64, k_curr=11, k_past=1, eps=1e-9,
                                                     restarts=200)
    assert info["status"] == 0
    # (eta is degenerate at t = 0: z_bar = 0 and bar_primal_obj = 0, and it does
    # not enter the iteration)
    for key in ("primal_obj", "lb_spec_est", "tr_X", "trS"):
        assert _rel(otr[0][key], gtr[0][key]) < 1e-9, (key, otr[0][key], gtr[0][key])


def test_usbs_zero_iterations_returns_the_start(cuda):
    """max_iters = 0: the loop runs no body (utils/loop.py:80-115); the state
    comes back unchanged."""
    from usbs_gb300 import solver
    W = wl.er_graph(200, 1000, 3)
    st = omaxcut.initialize_state(W, 10)
    n = st.C.shape[0]
    rs = np.random.default_rng(1)
    st = st._replace(y=rs.standard_normal(n), P=rs.standard_normal((n, 10)), tr_X=3.0,
                     primal_obj=1.5)
    out, info = solver.usbs(st, n, n, 2.0 * n, 2.0, S["rho"], S["beta"], 10, 1, 0, np.inf, -1.0,
                            -1.0, -1.0, 32, 10, 1e-7, 100, q0=orng.default_q0(n),
                            return_info=True)
    assert info["iterations"] == 0
    np.testing.assert_array_equal(out.y.cpu().numpy(), st.y)
    np.testing.assert_array_equal(out.P.cpu().numpy(), st.P)
    assert out.tr_X == 3.0 and out.primal_obj == 1.5


def test_usbs_renumbered_matches_plain(cuda):
    """usbs(renumber=True) solves the RCM-renumbered problem and returns the
    result in the original numbering: the same iterates up to the order of
    floating-point sums (resolved configuration, FP64)."""
    from usbs_gb300 import solver
    W = wl.er_graph(300, 4000, 7)
    st = omaxcut.initialize_state(W, 10)
    n = st.C.shape[0]
    q0 = orng.default_q0(n)
    kw = dict(q0=q0, precision=64, return_trace=True)
    args = (st, n, n, 2.0 * n, 2.0, S["rho"], S["beta"], 4, 1, 2, np.inf, -1.0, -1.0, -1.0, 32,
            200, 1e-9, S["subprob_max_iters"])
    a, atr, _ = solver.usbs(*args, **kw)
    b, btr, binfo = solver.usbs(*args, renumber=True, **kw)
    assert binfo["status"] == 0
    for key in ("primal_obj", "obj_ub", "lb_spec_est", "pen_dual_obj", "tr_X"):
        assert _rel(atr[0][key], btr[0][key]) < 1e-9, (key, atr[0][key], btr[0][key])
    np.testing.assert_allclose(b.P.cpu().numpy(), a.P.cpu().numpy(), rtol=1e-6,
                               atol=1e-6 * np.abs(a.P.cpu().numpy()).max())
    np.testing.assert_allclose(b.y.cpu().numpy(), a.y.cpu().numpy(), rtol=1e-6, atol=1e-8)


@pytest.mark.parametrize("precision,cond_base", [(64, 1.0), (32, 1.5)])
def test_usbs_graph_replay_equals_eager(cuda, monkeypatch, precision, cond_base):
    """The captured CUDA graph of the outer iteration runs the same kernels on
    the same data as the eager iteration: traces and final iterates are
    bit-identical, with condition checks every iteration (base 1) and in
    geometric blocks (base 1.5, several graph launches between host waits)."""
    from usbs_gb300 import solver
    W = wl.torus_graph(30, 1)
    st = omaxcut.initialize_state(W, 10)
    n = st.C.shape[0]
    q0 = orng.default_q0(n)
    args = (st, n, n, 2.0 * n, 2.0, S["rho"], S["beta"], 10, 1, 12, np.inf, -1.0, -1.0, -1.0, 32,
            10, 1e-7, S["subprob_max_iters"], cond_base)
    kw = dict(q0=q0, precision=precision, return_trace=True, return_info=True)
    monkeypatch.setenv("USBS_GRAPH", "0")
    a, atr, ainfo = solver.usbs(*args, **kw)
    monkeypatch.setenv("USBS_GRAPH", "1")
    b, btr, binfo = solver.usbs(*args, **kw)
    assert ainfo["graph_iterations"] == 0
    assert binfo["graph_iterations"] == binfo["iterations"] == 12
    assert ainfo["kernel_launches"] == binfo["kernel_launches"]
    assert len(atr) == len(btr) == 12
    for x, y in zip(atr, btr):
        assert np.array_equal(np.array(list(x.values())), np.array(list(y.values())),
                              equal_nan=True), (x, y)
    for f in ("y", "z", "P"):
        assert np.array_equal(getattr(a, f).cpu().numpy(), getattr(b, f).cpu().numpy()), f
    assert a.primal_obj == b.primal_obj and a.tr_X == b.tr_X
    assert binfo["lanczos_launches"] >= 1 and binfo["lanczos_ms"] > 0


@pytest.mark.parametrize("precision,renumber", [(64, False), (32, False), (64, True)])
def test_usbs_single_pass_rows_equals_two_passes(cuda, monkeypatch, precision, renumber):
    """MaxCut's constraints are single diagonal entries, so the solver evaluates
    A(F F^T) in the pass over V's rows that updates the sketch and the kept
    directions, one kernel instead of two.  Each value is computed as the
    separate constraint kernel computes it: traces and final iterates are
    bit-identical to the two-pass solve (USBS_FUSED_ROWS=0), with one launch
    fewer per outer iteration; the row-to-constraint map also holds after an
    RCM renumbering."""
    from usbs_gb300 import solver
    W = wl.torus_graph(30, 1)
    st = omaxcut.initialize_state(W, 10)
    n = st.C.shape[0]
    q0 = orng.default_q0(n)
    args = (st, n, n, 2.0 * n, 2.0, S["rho"], S["beta"], 10, 1, 6, np.inf, -1.0, -1.0, -1.0, 32,
            10, 1e-7, S["subprob_max_iters"])
    kw = dict(q0=q0, precision=precision, return_trace=True, return_info=True,
              renumber=renumber)
    monkeypatch.setenv("USBS_FUSED_ROWS", "0")
    a, atr, ainfo = solver.usbs(*args, **kw)
    monkeypatch.setenv("USBS_FUSED_ROWS", "1")
    b, btr, binfo = solver.usbs(*args, **kw)
    assert ainfo["status"] == binfo["status"] == 0
    assert len(atr) == len(btr) == 6
    assert ainfo["kernel_launches"] - binfo["kernel_launches"] == 6
    for x, y in zip(atr, btr):
        assert np.array_equal(np.array(list(x.values())), np.array(list(y.values())),
                              equal_nan=True), (x, y)
    for f in ("y", "z", "P"):
        assert np.array_equal(getattr(a, f).cpu().numpy(), getattr(b, f).cpu().numpy()), f
    assert a.primal_obj == b.primal_obj and a.tr_X == b.tr_X


def test_usbs_graph_not_used_with_inequalities(cuda):
    """The QAP relaxation decides its upsilon loop on the host: it runs eagerly."""
    from usbs_gb300 import solver
    from oracle import qap as oqap
    D, Wf = wl.qap_instance(6, 0, grid=5)
    st = oqap.initialize_state(D, Wf, 6)
    n, m = st.C.shape[0], st.b.shape[0]
    _, info = solver.usbs(st, n, m, 14.0 * st.SCALE_X, 2.0, 0.005, 0.25, 2, 0, 2, np.inf, -1.0,
                          -1.0, -1.0, min(n, 32), 10, 1e-7, 100, q0=orng.default_q0(n),
                          precision=64, return_info=True)
    assert info["status"] == 0 and info["graph_iterations"] == 0
