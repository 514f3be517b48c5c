"""Pins the CPU oracle with mathematics (the reference ships no golden vectors,
and its JAX implementation cannot run here).  CPU only."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import lanczos, loop, operators, rng
from oracle import maxcut as omaxcut
from oracle import usbs as ousbs
from oracle import ipm as oipm


def test_splitmix64_known_answer():
    # Vigna's splitmix64 with state 0: first output 0xE220A8397B1DCDAF
    z = rng._splitmix64(np.array([0], dtype=np.uint64))
    assert int(z[0]) == 0xE220A8397B1DCDAF
    z = rng._splitmix64(np.array([0x9E3779B97F4A7C15], dtype=np.uint64))
    assert int(z[0]) == 0x6E789E6AA1B965F4


def test_hash_normal_moments():
    x = rng.hash_normal(7, 200000)
    assert abs(x.mean()) < 0.01
    assert abs(x.std() - 1.0) < 0.01
    assert np.array_equal(x, rng.hash_normal(7, 200000))
    assert not np.array_equal(x[:10], rng.hash_normal(8, 10))


def test_cond_schedule_matches_reference_formula():
    # utils/loop.py:86-92 worked by hand for base 2, maxiter 100:
    # num = ceil(log(99)/log 2) + 1 = 8 -> 1,2,4,...,64; cumsum >= 100 from 64 on
    assert loop.cond_schedule(100, 2.0) == [1, 2, 4, 8, 16, 32, 37]
    assert sum(loop.cond_schedule(1000, 1.5)) == 1000
    assert loop.cond_schedule(5, 1.0) == [1] * 5


def test_while_loop_semantics():
    # body runs while cond holds, at most maxiter times, cond checked after each body
    calls = []
    out = loop.while_loop(lambda v: v < 5, lambda v: calls.append(v) or v + 1, 0, 100)
    assert out == 5 and calls == [0, 1, 2, 3, 4]
    assert loop.while_loop(lambda v: True, lambda v: v + 1, 0, 7) == 7
    assert loop.while_loop(lambda v: True, lambda v: v + 1, 0, 10, cond_exp_base=2.0) == 10


def _path_laplacian(n):
    W = sp.diags([np.ones(n - 1), np.ones(n - 1)], [-1, 1])
    return (sp.diags(np.asarray(W.sum(1)).ravel()) - W).tocsr()


def test_lanczos_path_laplacian_spectrum():
    n = 200
    L = _path_laplacian(n)
    exact = 2.0 - 2.0 * np.cos(np.pi * np.arange(n) / n)
    A_idx = np.zeros((0, 3), dtype=np.int64)
    q0 = rng.default_q0(n)
    vals, vecs, st = lanczos.eigsh_smallest(n, L, np.zeros(0), A_idx, np.zeros(1), q0, 3, 32,
                                            200, 1e-10)
    np.testing.assert_allclose(vals, exact[:3], atol=1e-8)
    r = L @ vecs - vecs * vals[None, :]
    assert np.linalg.norm(r, axis=0).max() < 1e-6
    np.testing.assert_allclose(vecs.T @ vecs, np.eye(3), atol=1e-10)


def test_lanczos_adjoint_term_diagonal_shift():
    # C + A*(w) with diag triples and w = s 1 shifts the spectrum by s
    n = 120
    L = _path_laplacian(n)
    A_data, A_idx, _, _ = omaxcut.get_all_problem_data(n)
    q0 = rng.default_q0(n)
    v0, _, _ = lanczos.eigsh_smallest(n, L, A_data, A_idx, np.zeros(n), q0, 2, 32, 100, 1e-10)
    v1, _, _ = lanczos.eigsh_smallest(n, L, A_data, A_idx, np.full(n, 3.5), q0, 2, 32, 100, 1e-10)
    np.testing.assert_allclose(v1, v0 + 3.5, atol=1e-8)


def test_A_adjoint_identity():
    rs = np.random.default_rng(0)
    n, m, T = 50, 30, 400
    A_idx = np.stack([rs.integers(0, m, T), rs.integers(0, n, T), rs.integers(0, n, T)], 1)
    A_data = rs.standard_normal(T)
    u = rs.standard_normal(n)
    z = rs.standard_normal(m)
    lhs = u @ operators.apply_A_adjoint_slim(n, A_data, A_idx, z, u)
    rhs = z @ operators.apply_A_operator_slim(m, A_data, A_idx, u)
    assert abs(lhs - rhs) < 1e-10 * (1 + abs(lhs))
    V = rs.standard_normal((n, 4))
    bat = operators.apply_A_operator_batched(m, A_data, A_idx, V)
    ref = sum(operators.apply_A_operator_slim(m, A_data, A_idx, V[:, j]) for j in range(4))
    np.testing.assert_allclose(bat, ref, rtol=1e-12, atol=1e-12)


def test_create_Q_base_matches_tensor_definition():
    rs = np.random.default_rng(1)
    n, m, T, k = 20, 9, 60, 3
    A_idx = np.stack([rs.integers(0, m, T), rs.integers(0, n, T), rs.integers(0, n, T)], 1)
    A_data = rs.standard_normal(T)
    V = rs.standard_normal((n, k))
    U = operators.create_svec_matrix(k)
    # solver/utils.py:53-65 written out with the explicit m x k x k tensor
    base = np.zeros((m, k, k))
    for t in range(T):
        base[A_idx[t, 0]] += A_data[t] * np.outer(V[A_idx[t, 1]], V[A_idx[t, 2]])
    proj = U @ base.reshape(m, k * k).T
    ref = (proj[:, None, :] * proj[None, :, :]).sum(-1)
    np.testing.assert_allclose(operators.create_Q_base(m, k, U, A_data, A_idx, V), ref,
                               rtol=1e-12, atol=1e-12)


def test_svec_isometry():
    k = 5
    U = operators.create_svec_matrix(k)
    rs = np.random.default_rng(2)
    A = rs.standard_normal((k, k)); A = A + A.T
    B = rs.standard_normal((k, k)); B = B + B.T
    assert abs(operators.svec(U, A) @ operators.svec(U, B) - np.sum(A * B)) < 1e-12
    np.testing.assert_allclose(operators.svec_inv(U, operators.svec(U, A), k), A, atol=1e-12)


def _complete_graph(n):
    W = np.ones((n, n)) - np.eye(n)
    return sp.csr_matrix(W)


@pytest.mark.parametrize("n", [12])
def test_usbs_complete_graph_value(n):
    """MaxCut SDP of K_n with unit weights: max <L/4, X> s.t. diag X = 1 is n^2/4."""
    st = omaxcut.initialize_state(_complete_graph(n), 4)
    out, fin = ousbs.usbs(st, n, n, 2.0 * n, 2.0, 0.01, 0.25, 3, 1, 300, np.inf, 1e-6, 1e-6,
                          1e-6, min(n, 32), 10, 1e-7, 100)
    assert abs(out.primal_obj - n * n / 4.0) / (n * n / 4.0) < 2e-3
    assert fin["max_infeas"] < 1e-2
    # the dual bound never falls below the primal value it certifies
    assert fin["obj_ub"] >= out.primal_obj - 1e-6 * n * n


def test_lb_ipm_is_a_lower_model_value():
    """The spectral lower-bound IPM (solver/usbs.py:195-356) at y with tr_X_bar = 0
    returns b.y - max over the bundle face, which never exceeds the penalised dual."""
    n, k = 40, 3
    rs = np.random.default_rng(3)
    W = sp.random(n, n, density=0.2, random_state=4)
    W = ((W + W.T) > 0).astype(float)
    W.setdiag(0)
    st = omaxcut.initialize_state(sp.csr_matrix(W), 4)
    C = st.C.toarray()
    V, _ = np.linalg.qr(rs.standard_normal((n, k)))
    U = operators.create_svec_matrix(k)
    y = rs.standard_normal(n) * 0.1
    GC = V.T @ C @ V
    Gy = V.T @ np.diag(y) @ V
    trace_ub = 2.0 * n
    lb = oipm.compute_lb_spec_est_ipm(U, k, trace_ub, y.sum(), GC, Gy, 0.0, 0.0, 0.0, 1e-9, 100)
    lam = np.linalg.eigvalsh(GC - Gy)
    # bundle model: b.y + trace_ub * max(lambda_max(V^T (C - A*y) V), 0)
    model = y.sum() + trace_ub * max(lam[-1], 0.0)
    assert abs(lb - model) < 1e-5 * (1 + abs(model))


def test_reconstruct_from_sketch_recovers_low_rank():
    """utils/common.py:99-116 on the sketch of a rank-3 PSD matrix: the Nystrom
    factors give X back up to the rho shift (rho ~ n 1e-6 lambda_max here)."""
    from oracle import common as ocommon
    rng = np.random.default_rng(11)
    n, s = 200, 8
    V = np.linalg.qr(rng.standard_normal((n, 3)))[0]
    X = (V * np.array([5.0, 2.0, 1.0])) @ V.T
    Om = rng.standard_normal((n, s))
    E, lam = ocommon.reconstruct_from_sketch(Om, X @ Om)
    assert np.all(np.diff(lam) <= 0.0)
    assert np.allclose(lam[:3], [5.0, 2.0, 1.0], rtol=1e-2)
    assert np.abs(lam[3:]).max() < 1e-12
    assert np.abs((E * lam) @ E.T - X).max() < 1e-2


def test_compute_max_cut_known_answers():
    """utils/maxcut_helpers.py:292-302: the sketch of v v^T for the 2-colouring
    of an even torus cuts every edge; a zero sketch (Cholesky fails, NaN
    signs) gives the all -1 vector, whose Laplacian cut value is 0."""
    from usbs_gb300 import workloads as wl
    side = 10
    W = wl.torus_graph(side, 0, weights="unit")
    n = W.shape[0]
    i = np.arange(n)
    v = np.where(((i // side) + (i % side)) % 2 == 0, 1.0, -1.0)
    C = omaxcut.laplacian_objective(W)
    Om = np.random.default_rng(1).standard_normal((n, 6))
    assert omaxcut.compute_max_cut(np.outer(v, v @ Om), Om, None, C) == W.nnz / 2
    assert omaxcut.compute_max_cut(np.zeros((n, 6)), Om, None, C) == 0.0


def test_usbs_invariants_along_the_trace():
    """Invariants of the iteration (the reference's definitions): tr X stays
    within trace_ub, the best dual bound only decreases and stays above the
    primal value of the nearly feasible X, and diag X moves to 1 (max_infeas
    falls) as the gap closes.  At these settings 200 iterations reach a gap of
    about 5e-2."""
    from usbs_gb300 import workloads as wl
    n = 40
    st = omaxcut.initialize_state(wl.er_graph(n, 300, 3), 4)
    tr = []
    out, fin = ousbs.usbs(st, n, n, 2.0 * n, 2.0, 0.01, 0.25, 4, 1, 200, np.inf, 1e-5, 1e-5,
                          1e-5, 32, 50, 1e-9, 100, trace=tr)
    assert len(tr) > 2
    for r in tr:
        assert r["tr_X"] <= 2.0 * n * (1 + 1e-9)
    ubs = [r["obj_ub"] for r in tr]
    assert all(b <= a + 1e-12 * abs(a) for a, b in zip(ubs, ubs[1:]))     # best bound so far
    last = tr[-1]
    assert last["max_infeas"] < 0.05 and last["max_infeas"] < tr[0]["max_infeas"] / 10
    assert last["obj_ub"] >= last["primal_obj"]
    assert last["obj_gap"] < 0.1 < tr[0]["obj_gap"]


def _golden():
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "known_answers.json")
    with open(path) as f:
        return json.load(f)


def test_golden_laplacian_spectra():
    """tests/golden/known_answers.json (closed forms): the oracle's eigsh on the
    path and cycle Laplacians.  A single-vector Krylov method sees a double
    eigenvalue once in exact arithmetic, so for the cycle the third returned
    value is either the second copy of lambda_1 or lambda_3."""
    g = _golden()
    A_idx = np.zeros((0, 3), dtype=np.int64)
    n = g["path_laplacian"]["n"]
    want = np.array(g["path_laplacian"]["smallest"])
    vals, _, _ = lanczos.eigsh_smallest(n, _path_laplacian(n), np.zeros(0), A_idx, np.zeros(1),
                                        rng.default_q0(n), len(want), 32, 300, 1e-11)
    np.testing.assert_allclose(vals, want, atol=1e-8)
    n = g["cycle_laplacian"]["n"]
    lam = g["cycle_laplacian"]["smallest"]
    W = sp.diags([np.ones(n - 1), np.ones(n - 1)], [-1, 1]).tolil()
    W[0, n - 1] = W[n - 1, 0] = 1.0
    W = W.tocsr()
    L = (sp.diags(np.asarray(W.sum(1)).ravel()) - W).tocsr()
    vals, _, _ = lanczos.eigsh_smallest(n, L, np.zeros(0), A_idx, np.zeros(1), rng.default_q0(n),
                                        3, 32, 300, 1e-11)
    assert abs(vals[0] - lam[0]) < 1e-8 and abs(vals[1] - lam[1]) < 1e-8
    assert min(abs(vals[2] - lam[2]), abs(vals[2] - lam[3])) < 1e-8


def test_golden_maxcut_sdp_even_torus():
    """The MaxCut SDP value of the bipartite 6 x 6 torus is |E| = 72."""
    from usbs_gb300 import workloads as wl
    g = _golden()["maxcut_sdp_even_torus"]
    n = g["n"]
    st = omaxcut.initialize_state(wl.torus_graph(g["side"], 0, weights="unit"), 4)
    out, fin = ousbs.usbs(st, n, n, 2.0 * n, 2.0, 0.01, 0.25, 3, 1, 300, np.inf, 1e-6, 1e-6,
                          1e-6, min(n, 32), 10, 1e-7, 100)
    assert abs(out.primal_obj - g["value"]) / g["value"] < 2e-3


@pytest.mark.parametrize("idx", range(4))
def test_golden_maxcut_sdp_vertex_transitive(idx):
    """Vertex-transitive graphs (odd cycles, the Petersen graph, the odd torus):
    the MaxCut SDP value is (n/4) lambda_max(L), strictly above the maximum
    cut; the oracle's solve reaches it."""
    from usbs_gb300 import workloads as wl
    g = _golden()["maxcut_sdp_vertex_transitive"][idx]
    W = wl.graph_from_spec(g["graph"])
    n = W.shape[0]
    assert n == g["n"]
    L = np.diag(np.asarray(W.sum(axis=1)).ravel()) - W.toarray()
    assert abs(n / 4.0 * np.linalg.eigvalsh(L)[-1] - g["value"]) < 1e-12 * g["value"]
    st = omaxcut.initialize_state(W, 4)
    out, fin = ousbs.usbs(st, n, n, 2.0 * n, 2.0, 0.01, 0.25, 3, 1, 300, np.inf, 1e-6, 1e-6,
                          1e-6, min(n, 32), 10, 1e-7, 100)
    assert abs(out.primal_obj - g["value"]) / g["value"] < 1e-4
    assert fin["max_infeas"] < 1e-4


@pytest.mark.parametrize("idx", [0, 2, 3])
def test_golden_cgal_approaches_vertex_transitive_value(idx):
    """The oracle's CGAL (solver/cgal.py) on the vertex-transitive known answers
    (C_7, the Petersen graph, the odd 5 x 5 torus): its primal value approaches
    (n/4) lambda_max(L) at CGAL's sublinear rate, within 5e-3 relative after
    2000 iterations and closer than after 500."""
    from oracle import cgal as ocgal
    from usbs_gb300 import workloads as wl
    g = _golden()["maxcut_sdp_vertex_transitive"][idx]
    W = wl.graph_from_spec(g["graph"])
    n = W.shape[0]
    st = omaxcut.initialize_state(W, 4)
    errs = []
    for iters in (500, 2000):
        out, fin = ocgal.cgal(st, n, n, float(n), 1.0, iters, np.inf, -1.0, -1.0, -1.0,
                              min(n, 32), 10, 1e-7)
        errs.append(abs(out.primal_obj - g["value"]) / g["value"])
    assert errs[1] < 5e-3 and errs[1] < errs[0]
    assert fin["max_infeas"] < 5e-3


@pytest.mark.parametrize("k", [2, 4, 6, 11])
def test_quad_ipm_solution_is_certified_optimal(k):
    """solve_quad_subprob_ipm (solver/usbs.py:25-192) minimises the convex
    quadratic f(x) = x^T Q x / 2 + h^T x, x = (svec S, eta), over S psd,
    eta >= 0, tr S + eta <= 1.  A feasible x is optimal exactly when the
    gradient's inner product with x equals the minimum of that linear function
    over the set, min(0, lambda_min(grad_S f), d f / d eta), which needs no
    solver to evaluate: an optimality certificate independent of the reference."""
    U = operators.create_svec_matrix(k)
    s = k * (k + 1) // 2
    rs = np.random.default_rng(k)
    B = rs.standard_normal((s + 1, s + 1))
    Q = B @ B.T / (s + 1)
    h = rs.standard_normal(s + 1) * 2.0
    consts = (1.0, Q[:s, :s], Q[:s, s], Q[s, s], h[:s], h[s])
    eta, S = oipm.solve_quad_subprob_ipm(U, k, 1.0, consts, 0.5, np.eye(k) / (2 * k), 1e-9, 200)
    assert np.linalg.eigvalsh(S)[0] > -1e-12 and eta > -1e-12
    assert np.trace(S) + eta <= 1.0 + 1e-9
    x = np.append(operators.svec(U, S), eta)
    g = Q @ x + h
    lowest = min(0.0, np.linalg.eigvalsh(operators.svec_inv(U, g[:s], k))[0], g[s])
    assert 0.0 <= g @ x - lowest <= 1e-6 * max(1.0, np.abs(g).max())


@pytest.mark.parametrize("k,g2", [(3, 0.0), (5, -4.0), (11, 0.0)])
def test_lb_ipm_value_equals_its_closed_form(k, g2):
    """compute_lb_spec_est_ipm (solver/usbs.py:195-356) minimises the linear
    g_1 . svec S + g_2 eta over the same set; that minimum is
    min(0, lambda_min(G_1), g_2), so the returned b.y - minimum has a closed
    form (G_1 = V^T (A*(y) - C) V, g_2 from z_bar . y - the bar objective)."""
    U = operators.create_svec_matrix(k)
    rs = np.random.default_rng(10 + k)
    G = rs.standard_normal((k, k))
    G = G + G.T
    by = 3.0
    lb = oipm.compute_lb_spec_est_ipm(U, k, 1.0, by, np.zeros((k, k)), G, g2, 0.0, 1.0, 1e-9, 200)
    closed = by - min(0.0, np.linalg.eigvalsh(G)[0], g2)
    assert abs(lb - closed) <= 1e-6 * max(1.0, abs(closed))


def test_lanczos_matches_dense_eigh_on_a_maxcut_operator():
    """The oracle's thick-restart Lanczos on C + A*(y) of an Erdos-Renyi MaxCut
    instance with a random y: its converged smallest eigenpairs equal LAPACK's
    dense eigendecomposition of the same matrix (built column by column from
    the oracle's own adjoint, itself checked by the adjoint identity)."""
    from usbs_gb300 import workloads as wl
    st = omaxcut.initialize_state(wl.er_graph(150, 900, 5), 4)
    n = st.C.shape[0]
    y = np.random.default_rng(7).standard_normal(n) * 0.5
    M = st.C.toarray() + operators.apply_A_adjoint_batched(n, st.A_data, st.A_indices, y,
                                                           np.eye(n))
    M = 0.5 * (M + M.T)
    exact = np.linalg.eigvalsh(M)[:5]
    vals, vecs, _ = lanczos.eigsh_smallest(n, st.C, st.A_data, st.A_indices, y, rng.default_q0(n),
                                           5, 32, 300, 1e-10)
    np.testing.assert_allclose(vals, exact, rtol=0, atol=1e-8 * np.abs(exact).max())
    r = M @ vecs - vecs * vals[None, :]
    assert np.linalg.norm(r, axis=0).max() < 1e-6 * np.abs(exact).max()
