"""The device solver against the FP64 oracle on the benchmark configurations'
own instances, at the reference's settings (k_curr 10, k_past 1, sketch 10,
rho 0.01, beta 0.25, 32 Lanczos vectors x 10 restarts, IPM tolerance 1e-7):

* ER(800, 19176) of seed 0 (the G1-scale instance), and
* the 100 x 100 +-1 torus of seed 1 (the bench's main workload).

Both start from the same start vector.  The plain FP64 path reproduces the
oracle's first outer iteration to 1e-7 relative (measured on GB300: at most
4e-8 on these instances; tr_X to 2e-6, as its first value is set by the
interior-point stop near mu = eps) and the next two to 1e-6 and 1e-5.  From
there the two trajectories part: with 10 restarts the trailing Ritz vectors
are not converged and are fixed by rounding, and the bundle iteration
amplifies any difference about tenfold per step (measured: 1e-5 at t = 3,
1e-3 at t = 4, 1e-2 at t = 5).  The mixed path (FP32 Lanczos) is held to 1e-3
on its first iteration (measured: 4e-4)."""
import numpy as np
import pytest

from oracle import maxcut as omaxcut
from oracle import rng as orng
from oracle import usbs as ousbs
from usbs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

S = wl.MAXCUT_SETTINGS
KEYS = ["primal_obj", "obj_ub", "lb_spec_est", "pen_dual_obj", "cand_pen_dual_obj", "cand_eig0",
        "obj_gap", "infeas_gap", "max_infeas", "tr_X"]
GRAPHS = {"er800": lambda: wl.er_graph(800, 19176, 0), "torus100": lambda: wl.torus_graph(100, 1)}


def _run(name, iters, precision):
    from usbs_gb300 import solver
    st = omaxcut.initialize_state(GRAPHS[name](), 10)
    n = st.C.shape[0]
    q0 = orng.default_q0(n)
    args = (n, n, 2.0 * n, 2.0, S["rho"], S["beta"], 10, 1, iters, np.inf, -1.0, -1.0, -1.0, 32,
            10, 1e-7, 100)
    otr = []
    ousbs.usbs(st, *args, q0=q0, trace=otr)
    _, gtr, info = solver.usbs(st, *args, 1.0, None, None, None, q0=q0, precision=precision,
                               return_trace=True)
    assert info["status"] == 0 and info["iterations"] == iters
    return otr, gtr


def _rel(a, b):
    return abs(a - b) / max(1.0, abs(a), abs(b))


@pytest.mark.parametrize("name", ["er800", "torus100"])
def test_fp64_first_iterations_match_oracle(cuda, name):
    otr, gtr = _run(name, 3, 64)
    for a, b in zip(otr, gtr):
        t = a["t"]
        assert bool(a["descent"]) == bool(b["descent"]), t
        for key in KEYS:
            tol = (1e-7, 1e-6, 1e-5)[t]
            if key == "tr_X" and t == 0:
                tol = 1e-5
            assert _rel(a[key], b[key]) < tol, (name, t, key, a[key], b[key])


@pytest.mark.parametrize("name", ["er800", "torus100"])
def test_mixed_first_iteration_close_to_oracle(cuda, name):
    otr, gtr = _run(name, 1, 32)
    for key in KEYS:
        assert _rel(otr[0][key], gtr[0][key]) < 1e-3, (name, key, otr[0][key], gtr[0][key])


# A problem on the stream path (n > 40,960): a 50,000-node random geometric
# 6-NN graph, the shape of the 10^6-node configuration at a size the oracle
# solves in seconds.
GRAPHS["rgg50k"] = lambda: wl.rgg_knn_graph(50000, 6, 5)


def test_stream_path_solve_matches_oracle(cuda):
    from usbs_gb300 import _lib
    assert _lib.load().usbs_lanczos_kernel(50000, 32, 64) == 2
    assert _lib.load().usbs_lanczos_kernel(50000, 32, 32) == 2
    otr, gtr = _run("rgg50k", 2, 64)
    for a, b in zip(otr, gtr):
        for key in KEYS:
            tol = (1e-7, 1e-5)[a["t"]]     # measured: 3e-6 at t = 1
            if key == "tr_X" and a["t"] == 0:
                tol = 1e-5
            assert _rel(a[key], b[key]) < tol, (a["t"], key, a[key], b[key])
    # FP32 Lanczos with 10 restarts leaves lambda_min about 1e-3 off at this n;
    # obj_ub scales it by trace_ub / 2 = n (measured: 1.8e-3 relative)
    otr, gtr = _run("rgg50k", 1, 32)
    for key in KEYS:
        assert _rel(otr[0][key], gtr[0][key]) < 5e-3, (key, otr[0][key], gtr[0][key])
