"""GPU parity of the rounding callbacks (reconstruct_from_sketch, compute_max_cut)
and of the per-check log lines against the FP64 oracle."""
import re

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import common as ocommon
from oracle import maxcut as omaxcut
from oracle import rng as orng
from usbs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

S = wl.MAXCUT_SETTINGS


def _psd_sketch(n, s, rank, seed, decay=True):
    rng = np.random.default_rng(seed)
    V = np.linalg.qr(rng.standard_normal((n, rank)))[0]
    lam = (1.0 / (1.0 + np.arange(rank)) ** 2) if decay else np.ones(rank)
    X = (V * (n * lam)) @ V.T
    Om = rng.standard_normal((n, s))
    return X, Om, X @ Om


@pytest.mark.parametrize("n,s,rank", [(300, 10, 10), (1000, 10, 3), (777, 32, 40)])
def test_reconstruct_from_sketch_matches_oracle(cuda, n, s, rank):
    from usbs_gb300 import rounding
    _, Om, P = _psd_sketch(n, s, rank, n + s)
    oE, olam = ocommon.reconstruct_from_sketch(Om, P)
    E, lam = rounding.reconstruct_from_sketch(Om, P)
    E, lam = E.cpu().numpy(), lam.cpu().numpy()
    scale = olam.max()
    np.testing.assert_allclose(lam, olam, rtol=1e-9, atol=1e-10 * scale)
    # columns with a well separated singular value agree up to sign
    rho2 = olam + 0.0
    for j in range(min(s, rank)):
        gap = min([abs(rho2[j] - rho2[q]) for q in range(s) if q != j] + [np.inf])
        if gap > 1e-6 * scale:
            assert abs(E[:, j] @ oE[:, j]) > 1 - 1e-8, j


def _column_values(E, C):
    with np.errstate(invalid="ignore"):
        Wb = 2.0 * (E > 0).astype(float) - 1.0
    return np.einsum("ij,ij->j", Wb, C @ Wb)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_compute_max_cut_matches_oracle(cuda, seed):
    from usbs_gb300 import rounding
    n = 600
    W = wl.er_graph(n, 3000, seed, weights="pm1" if seed == 2 else "unit")
    C = omaxcut.laplacian_objective(W)
    rng = np.random.default_rng(seed)
    # sketch of a PSD matrix built from 12 +-1 cut vectors with distinct
    # weights, so that every column of E is determined up to its sign (a
    # repeated singular value leaves its columns defined only up to rotation,
    # in the reference as here)
    Vb = np.sign(rng.standard_normal((n, 12)))
    X = (Vb * np.linspace(12.0, 1.0, 12)) @ Vb.T
    Om = rng.standard_normal((n, 10))
    P = X @ Om
    oE, _ = ocommon.reconstruct_from_sketch(Om, P)
    ocols = _column_values(oE, C)
    oval = omaxcut.compute_max_cut(P, Om, None, C)
    val, cols, signs = rounding.max_cut_values(P, Om, C)
    cols = cols.cpu().numpy()
    # the sign patterns agree wherever E is not within rounding of zero
    tiny = np.abs(oE) < 1e-9 * np.abs(oE).max()
    assert not tiny.any()
    np.testing.assert_allclose(cols, ocols, rtol=1e-12, atol=1e-9)
    assert abs(float(val.item()) - oval) <= 1e-12 * max(1.0, abs(oval))
    bits = signs.cpu().numpy().astype(np.int64) & ((1 << 10) - 1)
    obits = ((oE > 0).astype(np.int64) << np.arange(10)[None, :]).sum(axis=1)
    for j in range(10):
        bj, oj = (bits >> j) & 1, (obits >> j) & 1
        assert (bj == oj).all() or (bj == 1 - oj).all(), j
    assert rounding.compute_max_cut(P, Om, None, C) == float(val.item())


def test_compute_max_cut_bipartite_known_answer(cuda):
    """A 2-colourable torus and X = v v^T for its colouring: every edge is cut."""
    from usbs_gb300 import rounding
    side = 40
    W = wl.torus_graph(side, 0, weights="unit")
    n = W.shape[0]
    i = np.arange(n)
    v = np.where(((i // side) + (i % side)) % 2 == 0, 1.0, -1.0)
    C = omaxcut.laplacian_objective(W)
    Om = np.random.default_rng(5).standard_normal((n, 8))
    P = np.outer(v, v @ Om)
    assert rounding.compute_max_cut(P, Om, None, C) == W.nnz / 2
    assert omaxcut.compute_max_cut(P, Om, None, C) == W.nnz / 2


def test_compute_max_cut_zero_sketch(cuda):
    """P = 0: B is not positive definite; the reference's Cholesky gives NaNs,
    every sign is -1 and each column's value is 1^T C 1."""
    from usbs_gb300 import rounding
    W = wl.er_graph(200, 800, 3, weights="pm1")
    C = omaxcut.laplacian_objective(W) + sp.diags(np.linspace(0.0, 1.0, 200))
    Om = np.random.default_rng(0).standard_normal((200, 6))
    P = np.zeros_like(Om)
    val, cols, signs = rounding.max_cut_values(P, Om, C)
    ones = np.ones(200)
    assert (signs.cpu().numpy() == 0).all()
    np.testing.assert_allclose(cols.cpu().numpy(), np.full(6, ones @ (C @ ones)), rtol=1e-13)
    assert abs(float(val.item()) - omaxcut.compute_max_cut(P, Om, None, C)) < 1e-12
    E, lam = rounding.reconstruct_from_sketch(Om, P)
    assert np.isnan(lam.cpu().numpy()).all()


LINE = re.compile(r"^t: (\d+) - curr_time: ([.0-9e+-]+) - pen_dual_obj: (\S+)"
                  r" - cand_pen_dual_obj: (\S+) - lb_spec_est: (\S+) - primal_obj: (\S+)"
                  r" - dual_obj: (\S+) - primal_obj_ub: (\S+) - obj_gap: (\S+)"
                  r" - infeas_gap: (\S+) - max_infeas: (\S+) - callback_val: (.+)$")


def test_usbs_rounding_callback_and_log_lines(cuda):
    """usbs() with the reference's rounding callback and log lines: one line per
    condition check (t = 0 included) in the reference's format; the callback's
    last value equals the oracle's compute_max_cut on the returned sketch; the
    logged numbers equal the trace records and b . y of the returned y."""
    from usbs_gb300 import solver
    W = wl.er_graph(400, 2400, 7)
    st = omaxcut.initialize_state(W, 10)
    n = st.C.shape[0]
    Cu = (st.C / st.SCALE_C).tocsr()
    from usbs_gb300 import rounding
    lines = []
    iters = 12
    out, recs, info = solver.usbs(st, n, n, 2.0 * n, 2.0, S["rho"], S["beta"], 10, 1, iters,
                                  np.inf, -1.0, -1.0, -1.0, 32, 10, 1e-7,
                                  S["subprob_max_iters"], 1.0, rounding.compute_max_cut, None, Cu,
                                  q0=orng.default_q0(n), precision=64, return_trace=True,
                                  log=lines.append)
    assert info["iterations"] == iters
    assert len(lines) == iters + 1
    parsed = [LINE.match(l) for l in lines]
    assert all(parsed), lines[0]
    assert [int(m.group(1)) for m in parsed] == list(range(iters + 1))
    sx, sc = float(st.SCALE_X), float(st.SCALE_C)
    # t = 0: the initial state (solver/usbs.py:731-764)
    m0 = parsed[0]
    assert float(m0.group(8)) == np.inf and float(m0.group(5)) == 0.0
    assert float(m0.group(7)) == pytest.approx(float(st.b @ st.y), abs=1e-12)
    for t in range(1, iters + 1):
        m, r = parsed[t], recs[t - 1]
        assert float(m.group(3)) == r["pen_dual_obj"]
        assert float(m.group(6)) == pytest.approx(r["primal_obj"] / (sc * sx), rel=1e-15)
        assert float(m.group(9)) == r["obj_gap"]
        assert float(m.group(10)) == r["infeas_gap"]
        assert float(m.group(7)) == r["dual_obj"]
    y = out.y.cpu().numpy() if hasattr(out.y, "cpu") else np.asarray(out.y)
    assert float(parsed[-1].group(7)) == pytest.approx(float(st.b @ y), rel=1e-12, abs=1e-12)
    # callback values: the device rounding of the sketch at each check
    P = out.P.cpu().numpy()
    oval = omaxcut.compute_max_cut(P, st.Omega, None, Cu)
    assert info["callback_vals"][iters] == pytest.approx(oval, rel=1e-12)
    assert float(parsed[-1].group(12)) == info["callback_vals"][iters]


def test_cgal_log_lines(cuda):
    from usbs_gb300 import solver
    W = wl.er_graph(300, 1500, 8)
    st = omaxcut.initialize_state(W, 10)
    n = st.C.shape[0]
    lines = []
    solver.cgal(st, n, n, float(n), 1.0, 6, np.inf, -1.0, -1.0, -1.0, 32, 10, 1e-7,
                q0=orng.default_q0(n), log=lines.append)
    pat = re.compile(r"^t: (\d+) - curr_time: \S+ - primal_obj: \S+ - obj_gap: \S+"
                     r" - infeas_gap: \S+ - max_infeas: \S+ - callback_val: None$")
    assert len(lines) == 7 and all(pat.match(l) for l in lines), lines[:2]
    assert [int(pat.match(l).group(1)) for l in lines] == list(range(7))


def _lifted_perm_sketch(l, s, seed):
    """Sketch of x x^T for the lifted vector of a random assignment (x_0 = 1,
    x[1 + loc + l fac] = 1) plus a small PSD perturbation."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(l)
    x = np.zeros(l * l + 1)
    x[0] = 1.0
    x[1 + perm + l * np.arange(l)] = 1.0
    V = rng.standard_normal((l * l + 1, 3))
    X = np.outer(x, x) + 1e-3 * (V @ V.T)
    Om = rng.standard_normal((l * l + 1, s))
    return perm, X @ Om, Om


def _qap_candidates_oracle(E, l, D, W):
    from scipy.optimize import linear_sum_assignment
    out = []
    for sgn in (1.0, -1.0):
        for i in range(min(l, E.shape[1])):
            c = (sgn * E[1:, i]).reshape(l, l)
            r, col = linear_sum_assignment(c.max() - c)
            pm = np.zeros((l, l))
            pm[r, col] = 1.0
            out.append((float(np.trace(W @ pm @ D @ pm.T)), col.copy()))
    return out


def test_qap_round_recovers_the_encoded_assignment(cuda):
    """The dominant column of E is the lifted assignment vector: its
    candidate (positive or negative, by the column's sign) is that assignment."""
    from usbs_gb300 import rounding
    l = 8
    D, W = wl.qap_instance(l, 3, grid=5)
    perm, P, Om = _lifted_perm_sketch(l, l, 4)
    val, cand, perms = rounding.qap_round_values(P, Om, l, D, W)
    perms = perms.cpu().numpy()
    pm = np.zeros((l, l))
    pm[np.arange(l), perm] = 1.0
    obj = float(np.trace(W @ pm @ D @ pm.T))
    assert (perms[0] == perm).all() or (perms[l] == perm).all()
    j = 0 if (perms[0] == perm).all() else l
    assert float(cand[j].item()) == obj
    assert float(val.item()) <= obj


@pytest.mark.parametrize("l,s,seed", [(6, 6, 0), (9, 9, 1), (12, 8, 2)])
def test_qap_round_matches_oracle(cuda, l, s, seed):
    """Value exact (integer W, D); each column's pair of candidates (the sign
    of an E column is arbitrary) equal to the oracle's."""
    import pickle
    from oracle import qap as oqap
    from usbs_gb300 import rounding
    D, W = wl.qap_instance(l, seed, grid=5)
    rng = np.random.default_rng(seed)
    V = rng.standard_normal((l * l + 1, 2 * l))
    X = (V * np.linspace(3.0, 0.1, 2 * l)) @ V.T
    Om = rng.standard_normal((l * l + 1, s))
    P = X @ Om
    oval = oqap.qap_round(P, Om, pickle.dumps({"l": l}), {"D": D, "W": W})
    val, cand, perms = rounding.qap_round_values(P, Om, l, D, W)
    assert float(val.item()) == oval
    oE, _ = ocommon.reconstruct_from_sketch(Om, P)
    oc = _qap_candidates_oracle(oE, l, D, W)
    s2 = min(l, s)
    cand = cand.cpu().numpy()
    for i in range(s2):
        assert sorted([cand[i], cand[s2 + i]]) == sorted([oc[i][0], oc[s2 + i][0]]), i
    assert rounding.qap_round(P, Om, pickle.dumps({"l": l}), {"D": D, "W": W}) == oval


def test_usbs_qap_rounding_callback(cuda):
    """qap_round as usbs()'s callback on the QAP relaxation: its value at the
    last check equals the oracle's qap_round on the returned sketch."""
    import pickle
    from oracle import qap as oqap
    from usbs_gb300 import rounding, solver
    l = 5
    D, Wf = wl.qap_instance(l, 0, grid=5)
    st = oqap.initialize_state(D, Wf, l)
    n, m = st.C.shape[0], st.b.shape[0]
    trace_ub = 2.0 * float(l + 1) * st.SCALE_X
    static, nonstatic = pickle.dumps({"l": l}), {"D": D, "W": Wf}
    iters = 4
    out, info = solver.usbs(st, n, m, trace_ub, 2.0, 0.005, 0.25, 2, 0, iters, np.inf, -1.0, -1.0,
                            -1.0, min(n, 32), 300, 1e-9, 100, 1.0, rounding.qap_round, static,
                            nonstatic, q0=orng.default_q0(n), precision=64, return_info=True)
    assert info["iterations"] == iters
    P = out.P.cpu().numpy()
    assert info["callback_vals"][iters] == oqap.qap_round(P, st.Omega, static, nonstatic)
