"""The seeded synthetic instances that stand in for the reference's benchmark
archives have the stated shapes.  CPU only."""
import numpy as np

from usbs_gb300 import workloads as wl


def _check_adjacency(A, n):
    assert A.shape == (n, n)
    assert abs(A - A.T).nnz == 0
    assert np.all(A.diagonal() == 0)


def test_er_graph_gset_scale():
    A = wl.er_graph(800, 19176, 0)
    _check_adjacency(A, 800)
    assert A.nnz == 2 * 19176 and np.all(A.data == 1.0)
    B = wl.er_graph(800, 19176, 0)
    assert (A != B).nnz == 0                       # seeded


def test_torus_graph_spin_glass():
    A = wl.torus_graph(100, 1)
    _check_adjacency(A, 10 ** 4)
    assert A.nnz == 2 * 20000
    assert set(np.unique(A.data)) <= {-1.0, 1.0}
    deg = np.diff(A.indptr)
    assert np.all(deg == 4)


def test_rgg_knn_graph_small():
    A = wl.rgg_knn_graph(2000, 6, 0)
    _check_adjacency(A, 2000)
    assert np.all(np.diff(A.indptr) >= 6)          # every point keeps its 6 neighbours


def test_qap_instance_shapes():
    D, W = wl.qap_instance(30, 0)
    assert D.shape == W.shape == (30, 30)
    for M in (D, W):
        assert np.allclose(M, M.T) and np.all(np.diag(M) == 0)
    assert np.count_nonzero(D) >= np.count_nonzero(W)      # the denser matrix first
    F = W if W.max() <= 10 else D
    assert F.min() >= 0 and F.max() <= 10 and np.allclose(F, np.round(F))
