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
