"""Instance readers (scripts/warm_start_maxcut_usbs.py:81-95,
utils/qap_helpers.py:26-154) on files the tests write."""
import numpy as np
import pytest
import scipy.io
import scipy.sparse as sp

from usbs_gb300.problems import loaders, qap
from usbs_gb300 import workloads as wl


def test_maxcut_mat_gset_and_dimacs(tmp_path):
    W = sp.csc_matrix(wl.er_graph(50, 200, 0))
    g = tmp_path / "Gset" / "G_test.mat"
    g.parent.mkdir()
    scipy.io.savemat(g, {"Problem": {"name": "G_test", "A": W}})
    got, drop = loaders.load_maxcut_mat(g)
    assert drop == 0 and (got != W).nnz == 0
    got, drop = loaders.load_maxcut_mat(g, warm_start_frac=0.9)
    assert drop == 5 and (got != W[:45, :45]).nnz == 0
    d = tmp_path / "DIMACS10" / "g.mat"
    d.parent.mkdir()
    scipy.io.savemat(d, {"Problem": {"name": "g", "title": "t", "A": W}})
    got, _ = loaders.load_maxcut_mat(d)
    assert (got != W).nnz == 0
    other = tmp_path / "x.mat"
    scipy.io.savemat(other, {"Problem": {"A": W}})
    with pytest.raises(ValueError):
        loaders.load_maxcut_mat(other)


def test_qaplib_reader(tmp_path):
    n = 5
    rs = np.random.default_rng(0)
    A = rs.integers(0, 9, (n, n)).astype(float)          # dense: becomes D
    B = np.where(rs.random((n, n)) < 0.3, rs.integers(1, 5, (n, n)), 0).astype(float)
    f = tmp_path / "t5.dat"
    f.write_text(f"  {n}\n\n" + "\n".join(" ".join(f"{int(v)}" for v in r) for r in B) + "\n\n"
                 + "\n".join(" ".join(f"{int(v)}" for v in r) for r in A) + "\n")
    l, D, W = loaders.load_qaplib(f)
    assert l == n and (D == A).all() and (W == B).all()      # the sparser one is W
    l, D, W = loaders.load_qaplib(f, num_drop=2)
    assert l == 3 and (D == A[:3, :3]).all() and (W == B[:3, :3]).all()
    st = qap.initialize_state(D, W, 3)
    assert st.C.shape == (10, 10)


def _write_tsp(path, header, body):
    path.write_text("\n".join(f"{k} : {v}" for k, v in header.items()) + "\n" + body + "\nEOF\n")


def test_tsplib_explicit_formats(tmp_path):
    n = 5
    rs = np.random.default_rng(1)
    M = rs.integers(1, 50, (n, n))
    M = np.triu(M, 1) + np.triu(M, 1).T
    cases = {
        "FULL_MATRIX": " ".join(str(v) for v in M.ravel()),
        "UPPER_ROW": " ".join(str(v) for v in M[np.triu_indices(n, 1)]),
        "UPPER_DIAG_ROW": " ".join(str(v) for v in M[np.triu_indices(n, 0)]),
        "LOWER_DIAG_ROW": " ".join(str(v) for v in M[np.tril_indices(n, 0)]),
    }
    for fmt, vals in cases.items():
        f = tmp_path / f"{fmt}.tsp"
        _write_tsp(f, {"NAME": "t", "TYPE": "TSP", "DIMENSION": n, "EDGE_WEIGHT_TYPE": "EXPLICIT",
                       "EDGE_WEIGHT_FORMAT": fmt}, "EDGE_WEIGHT_SECTION\n" + vals)
        l, D, W = loaders.load_tsplib(f)
        assert l == n and (D == M).all(), fmt
    # canonical tour, weight 1/2 each way; rows sum to 1
    assert np.allclose(W.sum(axis=1), 1.0) and W[0, 1] == 0.5 and W[n - 1, 0] == 0.5
    l, D, W = loaders.load_tsplib(tmp_path / "FULL_MATRIX.tsp", num_drop=2)
    assert l == 3 and (D == M[:3, :3]).all() and W[2, 0] == 0.5


def test_tsplib_coordinate_rules(tmp_path):
    pts = np.array([[0.0, 0.0], [3.0, 4.0], [10.0, 0.0]])
    body = "NODE_COORD_SECTION\n" + "\n".join(f"{i + 1} {x} {y}" for i, (x, y) in enumerate(pts))
    got = {}
    for kind in ("EUC_2D", "CEIL_2D", "ATT", "GEO"):
        f = tmp_path / f"{kind}.tsp"
        _write_tsp(f, {"NAME": "t", "TYPE": "TSP", "DIMENSION": 3, "EDGE_WEIGHT_TYPE": kind}, body)
        got[kind] = loaders.load_tsplib(f)[1]
    assert got["EUC_2D"][0, 1] == 5.0 and got["EUC_2D"][1, 2] == 8.0      # sqrt(65) = 8.06
    assert got["CEIL_2D"][1, 2] == 9.0
    assert got["ATT"][0, 2] == 4.0            # ceil(sqrt(100 / 10))
    assert (got["GEO"] == got["GEO"].T).all() and got["GEO"][0, 1] > 0
    f = tmp_path / "bad.tsp"
    _write_tsp(f, {"NAME": "t", "TYPE": "TSP", "DIMENSION": 3, "EDGE_WEIGHT_TYPE": "MAN_2D"}, body)
    with pytest.raises(ValueError):
        loaders.load_tsplib(f)
