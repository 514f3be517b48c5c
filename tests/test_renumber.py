"""RCM renumbering of an SDP instance (usbs_gb300.renumber): the permuted
problem is the same problem, and the state maps back exactly."""
import numpy as np

from oracle.common import apply_A_operator_mx
from usbs_gb300 import renumber as rn
from usbs_gb300 import workloads as wl
from usbs_gb300.problems import maxcut, qap


def test_rcm_narrows_the_band_and_commutes_with_the_operator():
    W = wl.rgg_knn_graph(3000, 6, 1)
    st = maxcut.initialize_state(W, 4)
    n = st.C.shape[0]
    perm = rn.rcm_permutation(st.C, st.A_indices, n)
    assert sorted(perm) == list(range(n))
    Cp, idx = rn.permute_problem(st.C, st.A_indices, perm)
    coo, coo_p = st.C.tocoo(), Cp.tocoo()
    assert np.abs(coo_p.row - coo_p.col).max() < np.abs(coo.row - coo.col).max() / 10
    x = np.random.default_rng(0).standard_normal(n)
    np.testing.assert_allclose(Cp @ x[perm], (st.C @ x)[perm], rtol=1e-14, atol=1e-14)


def test_constraints_of_the_permuted_iterate_are_unchanged():
    """A(P^T X P) with renumbered triples equals A(X): y, z, b stay in
    constraint space (QAP, general triples)."""
    D, Wf = wl.qap_instance(4, 0, grid=5)
    st = qap.initialize_state(D, Wf, -1)
    n, m = st.C.shape[0], st.b.shape[0]
    rs = np.random.default_rng(1)
    V = rs.standard_normal((n, 5))
    X = V @ V.T
    perm = rn.rcm_permutation(st.C, st.A_indices, n)
    _, idx = rn.permute_problem(st.C, st.A_indices, perm)
    np.testing.assert_allclose(apply_A_operator_mx(n, m, st.A_data, idx, X[perm][:, perm]),
                               apply_A_operator_mx(n, m, st.A_data, st.A_indices, X),
                               rtol=1e-12, atol=1e-12)


def test_state_round_trip():
    W = wl.er_graph(200, 800, 2)
    st = maxcut.initialize_state(W, 5)
    n = st.C.shape[0]
    rs = np.random.default_rng(3)
    st = st._replace(P=rs.standard_normal((n, 5)))
    perm = rn.rcm_permutation(st.C, st.A_indices, n)
    back = rn.unpermute_state(rn.permute_state(st, perm), st, perm)
    np.testing.assert_array_equal(back.P, st.P)
    np.testing.assert_array_equal(back.Omega, st.Omega)
    dense = maxcut.initialize_state(W, -1)
    dense = dense._replace(X=rs.standard_normal((n, n)))
    back = rn.unpermute_state(rn.permute_state(dense, perm), dense, perm)
    np.testing.assert_array_equal(back.X, dense.X)
