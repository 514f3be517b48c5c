"""MaxCut warm starts (utils/maxcut_helpers.py:95-289): the package's state
transforms against the oracle's, on a solved-looking state grown to a larger
graph with some edges re-sampled."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import maxcut as omaxcut
from oracle.common import scale_sdp_state as oscale
from usbs_gb300 import workloads as wl
from usbs_gb300.problems import maxcut as pmaxcut


def _graphs(n_old=300, n=330, seed=0):
    Wo = wl.er_graph(n_old, 6 * n_old, seed)
    Wn = sp.lil_matrix((n, n))
    Wn[:n_old, :n_old] = Wo
    extra = wl.er_graph(n, 60, seed + 1)
    return Wo, sp.csr_matrix(Wn + extra - Wn.multiply(extra > 0))


def _solved_state(Wo, sketch_dim, seed=2):
    """A cold state with a PSD iterate, duals and objective filled in (scaled)."""
    rng = np.random.default_rng(seed)
    st = omaxcut.initialize_state(Wo, sketch_dim)
    n = st.C.shape[0]
    V = rng.standard_normal((n, 15))
    X = (V * np.linspace(3.0, 0.2, 15)) @ V.T
    us = st._replace(SCALE_C=1.0, SCALE_X=1.0, SCALE_A=np.ones(n), C=st.C.tocsr())
    us = us._replace(X=X if sketch_dim == -1 else None,
                     P=None if sketch_dim == -1 else X @ st.Omega,
                     y=rng.standard_normal(n), z=np.diagonal(X).copy(),
                     tr_X=float(np.trace(X)), primal_obj=float((st.C @ X).trace()))
    sc = us._replace(SCALE_C=0.37, SCALE_X=1.0 / n)
    return oscale(sc)


def _same(a, b, rtol=1e-12):
    for f in a._fields:
        x, y = getattr(a, f), getattr(b, f)
        if x is None or y is None:
            assert x is None and y is None, f
            continue
        if sp.issparse(x):
            x, y = x.toarray(), y.toarray()
        x = np.asarray(x.detach().cpu() if hasattr(x, "detach") else x, float)
        y = np.asarray(y, float)
        np.testing.assert_allclose(x, y, rtol=rtol, atol=rtol * max(1.0, np.abs(y).max()),
                                   err_msg=f)


@pytest.mark.parametrize("sketch_dim", [10, -1])
def test_implicit_warm_start_matches_oracle(sketch_dim):
    Wo, Wn = _graphs()
    old = _solved_state(Wo, sketch_dim)
    _same(pmaxcut.implicit_warm_start(old, Wn, sketch_dim),
          omaxcut.get_implicit_warm_start_state(old, Wn, sketch_dim))


def test_dual_only_warm_start_matches_oracle():
    Wo, Wn = _graphs()
    old = _solved_state(Wo, 10)
    _same(pmaxcut.dual_only_warm_start(old, Wn, 10),
          omaxcut.get_dual_only_warm_start_state(old, Wn, 10))


def test_explicit_warm_start_dense_matches_oracle():
    Wo, Wn = _graphs()
    old = _solved_state(Wo, -1)
    _same(pmaxcut.explicit_warm_start(old, Wn, -1),
          omaxcut.get_explicit_warm_start_state(old, Wn, -1))


@pytest.mark.gpu
def test_explicit_warm_start_sketch_matches_oracle(cuda):
    """The sketch is reconstructed on the device; X_hat = S S^T does not depend
    on the sign (or, within a repeated singular value, the rotation) of E's
    columns, so P, z, tr_X and primal_obj agree to the reconstruction's
    accuracy."""
    Wo, Wn = _graphs()
    old = _solved_state(Wo, 10)
    _same(pmaxcut.explicit_warm_start(old, Wn, 10),
          omaxcut.get_explicit_warm_start_state(old, Wn, 10), rtol=1e-8)


# ---- QAP (utils/qap_helpers.py:384-621) ----

def _same_qap(a, b, rtol):
    """As _same, with the constraint triples compared as a set: the package's
    builder lists the same (constraint, i, j, a) triples in another order."""
    def sorted_triples(st):
        idx = np.asarray(st.A_indices)
        o = np.lexsort((idx[:, 2], idx[:, 1], idx[:, 0]))
        return idx[o], np.asarray(st.A_data)[o]
    ia, da = sorted_triples(a)
    ib, db = sorted_triples(b)
    np.testing.assert_array_equal(ia, ib)
    np.testing.assert_allclose(da, db, rtol=rtol)
    _same(a._replace(A_indices=None, A_data=None), b._replace(A_indices=None, A_data=None), rtol)

def _qap_solved(l_old, l, sketch_dim, seed=3):
    """A solved-looking QAP state on the first l_old facilities of an l-facility
    instance, and that instance's (D, W)."""
    from oracle import common as ocommon
    from oracle import qap as oqap
    D, W = wl.qap_instance(l, seed, grid=6)
    st = oqap.initialize_state(D[:l_old, :l_old], W[:l_old, :l_old], sketch_dim)
    us = ocommon.unscale_sdp_state(st)
    n, m = us.C.shape[0], us.b.shape[0]
    rng = np.random.default_rng(seed)
    V = rng.standard_normal((n, 2 * l))
    X = (V * np.linspace(2.0, 0.1, 2 * l)) @ V.T
    us = us._replace(X=X if sketch_dim == -1 else None,
                     P=None if sketch_dim == -1 else X @ us.Omega,
                     y=rng.standard_normal(m), z=rng.standard_normal(m),
                     tr_X=float(np.trace(X)), primal_obj=float((us.C @ X).trace()))
    return ocommon.scale_sdp_state(us), D, W


@pytest.mark.parametrize("sketch_dim", ["l", -1])
def test_qap_implicit_and_dual_only_warm_starts_match_oracle(sketch_dim):
    from oracle import qap as oqap
    from usbs_gb300.problems import qap as pqap
    l_old, l = 4, 6
    sd = l if sketch_dim == "l" else -1
    old, D, W = _qap_solved(l_old, l, sd)
    _same_qap(pqap.implicit_warm_start(old, D, W, sd),
              oqap.get_implicit_warm_start_state(old, D, W, sd), rtol=1e-9)
    _same_qap(pqap.dual_only_warm_start(old, D, W, sd),
              oqap.get_dual_only_warm_start_state(old, D, W, sd), rtol=1e-9)


def test_qap_explicit_warm_start_dense_matches_oracle():
    from oracle import qap as oqap
    from usbs_gb300.problems import qap as pqap
    old, D, W = _qap_solved(4, 6, -1)
    _same_qap(pqap.explicit_warm_start(old, D, W, -1),
              oqap.get_explicit_warm_start_state(old, D, W, -1), rtol=1e-9)


def test_qap_warm_start_moves_the_lifted_indices():
    """Facility f at location i of the old instance (index 1 + i + l_old f)
    lands on 1 + i + l f; the new facility's rows stay empty."""
    from usbs_gb300.problems import qap as pqap
    l_old, l = 3, 4
    old, D, W = _qap_solved(l_old, l, -1)
    new = pqap.implicit_warm_start(old, D, W, -1)
    Xo = np.asarray(old.X) / old.SCALE_X
    Xn = np.asarray(new.X) / new.SCALE_X
    for f in range(l_old):
        for i in range(l_old):
            a, b = 1 + i + l_old * f, 1 + i + l * f
            assert Xn[b, 0] == pytest.approx(Xo[a, 0], rel=1e-12)
    assert not Xn[1 + (l - 1) + l * np.arange(l), :].any()


@pytest.mark.gpu
def test_qap_explicit_warm_start_sketch_matches_oracle(cuda):
    from oracle import qap as oqap
    from usbs_gb300.problems import qap as pqap
    old, D, W = _qap_solved(4, 6, 6)
    _same_qap(pqap.explicit_warm_start(old, D, W, 6),
              oqap.get_explicit_warm_start_state(old, D, W, 6), rtol=1e-8)



@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["implicit", "dual_only"])
def test_warm_start_from_a_device_result_stays_on_the_device(cuda, kind):
    """A finished solve's result (device tensors) warm-starts the grown problem
    on the device: same values as the host transform of the same state, and the
    iterate never leaves the GPU."""
    import torch
    from usbs_gb300 import solver
    Wo, Wn = _graphs()
    st = pmaxcut.initialize_state(Wo, 10)
    n = st.C.shape[0]
    res = solver.usbs(st, n, n, 2.0 * n, 2.0, 0.01, 0.25, 4, 1, 3, np.inf, -1.0, -1.0, -1.0, 32,
                      10, 1e-7, 100, precision=64)
    assert res.y.is_cuda and res.z.is_cuda and res.P.is_cuda
    host = res._replace(y=res.y.cpu().numpy(), z=res.z.cpu().numpy(), P=res.P.cpu().numpy())
    fn = pmaxcut.implicit_warm_start if kind == "implicit" else pmaxcut.dual_only_warm_start
    dev_ws, host_ws = fn(res, Wn, 10), fn(host, Wn, 10)
    fields = ("y", "z", "P", "Omega") if kind == "implicit" else ("y",)
    for f in fields:
        d = getattr(dev_ws, f)
        assert isinstance(d, torch.Tensor) and d.is_cuda, f
        np.testing.assert_allclose(d.cpu().numpy(), np.asarray(getattr(host_ws, f)), rtol=1e-13,
                                   atol=1e-13)
    assert abs(dev_ws.primal_obj - host_ws.primal_obj) <= 1e-12 * max(1.0, abs(host_ws.primal_obj))
    assert dev_ws.tr_X == host_ws.tr_X and dev_ws.SCALE_X == host_ws.SCALE_X
    # and the grown problem solves from either start to the same iterates
    m = Wn.shape[0]
    a = solver.usbs(dev_ws, m, m, 2.0 * m * dev_ws.SCALE_X, 2.0, 0.01, 0.25, 4, 1, 2, np.inf,
                    -1.0, -1.0, -1.0, 32, 10, 1e-7, 100, precision=64)
    b = solver.usbs(host_ws, m, m, 2.0 * m * host_ws.SCALE_X, 2.0, 0.01, 0.25, 4, 1, 2, np.inf,
                    -1.0, -1.0, -1.0, 32, 10, 1e-7, 100, precision=64)
    np.testing.assert_allclose(a.y.cpu().numpy(), b.y.cpu().numpy(), rtol=1e-9, atol=1e-12)


@pytest.mark.gpu
def test_service_warm_starts_a_request_from_its_parent(cuda):
    from usbs_gb300.serving import SolveRequest, SolverService
    Wo, Wn = _graphs()
    n, m = Wo.shape[0], Wn.shape[0]
    base = dict(trace_factor=2.0, rho=0.01, beta=0.25, k_curr=4, k_past=1, max_iters=3,
                max_time=np.inf, obj_gap_eps=-1.0, infeas_gap_eps=-1.0, max_infeas_eps=-1.0,
                lanczos_inner_iterations=32, lanczos_max_restarts=10, subprob_eps=1e-7,
                subprob_max_iters=100)
    with SolverService(max_slots=4, reserve_bytes=1 << 30) as svc:
        parent = svc.submit(SolveRequest(pmaxcut.initialize_state(Wo, 10), precision=64, n=n,
                                         m=n, trace_ub=2.0 * n, **base))
        child = svc.submit(SolveRequest(
            pmaxcut.initialize_state(Wn, 10), precision=64, n=m, m=m, trace_ub=2.0 * m,
            warm_from=parent, warm_start=lambda res, cold: pmaxcut.implicit_warm_start(res, Wn, 10),
            **base))
        child.wait(600)
        assert child.warmed and child.start >= parent.finish
        # the same warm start done by hand from the parent's result
        from usbs_gb300 import solver
        ws = pmaxcut.implicit_warm_start(parent.result, Wn, 10)
        ref = solver.usbs(ws, m, m, 2.0 * m * ws.SCALE_X, precision=64, **{
            k: v for k, v in base.items() if k != "trace_factor"}, trace_factor=2.0)
    np.testing.assert_allclose(child.result.y.cpu().numpy(), ref.y.cpu().numpy(), rtol=1e-12,
                               atol=1e-14)
