"""Host-side layout of the problem data, and the C ABI library (CPU only)."""
import ctypes
import os
import re

import numpy as np
import pytest
import scipy.sparse as sp

from usbs_gb300 import problem as P
from usbs_gb300 import workloads as wl
from oracle import maxcut as omaxcut
from oracle import qap as oqap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _check_layout(C, A_data, A_idx, m):
    L = P.layout(C, A_data, A_idx, m=m)
    n = C.shape[0]
    # union pattern holds C exactly and every triple position
    M = sp.csr_matrix((L.c_val, L.col, L.rowptr), shape=(n, n))
    assert abs(M - C).max() == 0
    pos = set(zip(np.repeat(np.arange(n), np.diff(L.rowptr)), L.col))
    assert all((i, j) in pos for i, j in zip(A_idx[:, 1], A_idx[:, 2]))
    # slot map: every triple exactly once, on its (i, j)
    prow = np.repeat(np.arange(n), np.diff(L.rowptr))
    seen = np.zeros(A_data.size, dtype=int)
    for p in range(L.nnz):
        for q in range(L.slot_ptr[p], L.slot_ptr[p + 1]):
            t = L.slot_tid[q]
            seen[t] += 1
            assert A_idx[t, 1] == prow[p] and A_idx[t, 2] == L.col[p]
    assert np.all(seen == 1)
    # constraint-sorted copy reproduces A(u u^T)
    u = np.random.default_rng(0).standard_normal(n)
    ref = np.bincount(A_idx[:, 0], weights=A_data * u[A_idx[:, 1]] * u[A_idx[:, 2]], minlength=m)
    got = np.zeros(m)
    for c in range(m):
        s = slice(L.con_ptr[c], L.con_ptr[c + 1])
        got[c] = np.sum(L.t_a[s] * u[L.t_row[s]] * u[L.t_col[s]])
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)
    # row-sorted copy reproduces A*(z) u
    z = np.random.default_rng(1).standard_normal(m)
    ref = np.bincount(A_idx[:, 1], weights=A_data * z[A_idx[:, 0]] * u[A_idx[:, 2]], minlength=n)
    got = np.array([np.sum(L.r_a[L.row_ptr[i]:L.row_ptr[i + 1]]
                           * z[L.r_con[L.row_ptr[i]:L.row_ptr[i + 1]]]
                           * u[L.r_col[L.row_ptr[i]:L.row_ptr[i + 1]]]) for i in range(n)])
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)
    return L


def test_layout_maxcut():
    W = wl.er_graph(60, 300, 0)
    st = omaxcut.initialize_state(W, 4)
    L = _check_layout(st.C, st.A_data, st.A_indices, 60)
    assert L.diag_constraints


def test_layout_qap_small():
    D, W = wl.qap_instance(4, 0, grid=4)
    st = oqap.initialize_state(D, W, 4)
    L = _check_layout(st.C, st.A_data, st.A_indices, st.b.shape[0])
    assert not L.diag_constraints


def test_layout_rejects_bad_triples():
    C = sp.eye(4, format="csr")
    try:
        P.layout(C, np.ones(1), np.array([[0, 7, 0]]), m=1)
    except ValueError:
        return
    raise AssertionError("out-of-range triple accepted")


def _declared_functions():
    hdr = open(os.path.join(ROOT, "include", "usbs_gb300.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(usbs_[A-Za-z0-9_]+)\s*\(", hdr)))


def test_library_builds_and_exports_every_declared_symbol():
    from usbs_gb300 import build, _lib
    path = build.build()
    lib = ctypes.CDLL(path)
    names = _declared_functions()
    assert len(names) >= 8
    for name in names:
        assert hasattr(lib, name), f"{name} declared in include/usbs_gb300.h but not exported"
    assert set(names) <= set(_lib.SIGNATURES), "ctypes signatures missing for some entry points"
    lib.usbs_abi_version.restype = ctypes.c_int
    assert lib.usbs_abi_version() == 5


def _as_set(A_data, A_idx, b, mask):
    trip = {}
    for (c, i, j), a in zip(np.asarray(A_idx), np.asarray(A_data)):
        trip[(int(c), int(i), int(j))] = trip.get((int(c), int(i), int(j)), 0.0) + float(a)
    return trip


@pytest.mark.parametrize("l", [3, 5])
def test_product_qap_builder_matches_oracle(l):
    """usbs_gb300.problems.qap builds the same SDP as the oracle restatement of
    utils/qap_helpers.py:157-381 (same constraints, right-hand sides, masks and scales)."""
    from usbs_gb300.problems import qap as pqap
    D, W = wl.qap_instance(l, 1, grid=6)
    a = oqap.initialize_state(D, W, 4)
    b = pqap.initialize_state(D, W, 4)
    assert (a.C != b.C).nnz == 0
    np.testing.assert_array_equal(a.b_ineq_mask, b.b_ineq_mask)
    np.testing.assert_allclose(b.b, a.b, rtol=1e-12, atol=0)
    np.testing.assert_allclose(b.SCALE_A, a.SCALE_A, rtol=1e-10)
    assert b.SCALE_C == pytest.approx(a.SCALE_C, rel=1e-14)
    assert b.SCALE_X == a.SCALE_X
    ta, tb = _as_set(a.A_data, a.A_indices, a.b, a.b_ineq_mask), \
        _as_set(b.A_data, b.A_indices, b.b, b.b_ineq_mask)
    assert ta.keys() == tb.keys()
    assert max(abs(ta[k] - tb[k]) for k in ta) < 1e-12


@pytest.mark.parametrize("shape", [(1, 1), (255, 3), (257, 7), (1000, 12), (3001, 2)])
def test_sell_layout_covers_every_entry_once(shape):
    n, avg = shape
    rs = np.random.default_rng(n)
    lens = rs.integers(0, 2 * avg + 1, size=n)
    rowptr = np.concatenate([[0], np.cumsum(lens)])
    col = rs.integers(0, n, size=int(rowptr[-1])).astype(np.int32)
    L = P.sell_layout(rowptr, col)
    src = L["sl_src"]
    real = src[src >= 0]
    assert np.array_equal(np.sort(real), np.arange(rowptr[-1]))        # each entry once
    np.testing.assert_array_equal(L["sl_col"][src >= 0], col[real])
    assert np.all(L["sl_col"][src < 0] == 0)
    nsl = (n + 31) // 32
    assert L["sl_ptr"].size == nsl + 1 and np.all(np.diff(L["sl_ptr"]) % 32 == 0)
    # positions inside each window form a permutation of the window's slots
    row = L["sl_row"].astype(np.int64)
    for w0 in range(0, nsl * 32, 256):
        seg = row[w0:w0 + 256]
        assert np.array_equal(np.sort(seg), np.arange(seg.size))
    # entry k of the row at sorted position q sits at sl_ptr[q // 32] + 32 k + q % 32
    order = (np.arange(n) // 256) * 256 + row[:n]
    for q in rs.integers(0, n, size=min(n, 50)):
        r = order[q]
        for k in range(lens[r]):
            e = L["sl_ptr"][q // 32] + 32 * k + q % 32
            assert src[e] == rowptr[r] + k


def test_reference_style_calls_reuse_the_device_layout():
    """eigsh_smallest(n, C, A_data, A_indices, ...) with host arrays, called
    again with the same problem (as the reference's solver loop does), reuses
    the resident layout; a changed array, even changed in place, gets a new one;
    device inputs are laid out afresh."""
    from usbs_gb300 import api
    st = omaxcut.initialize_state(wl.er_graph(50, 200, 1), 2)
    n = st.C.shape[0]
    made = []

    def make():
        made.append(object())
        return made[-1]

    api._LAYOUTS.clear()
    a = api._problem_for(st.C, st.A_data, st.A_indices, n, "cuda", make=make)
    b = api._problem_for(st.C.copy(), st.A_data.copy(), st.A_indices.copy(), n, "cuda", make=make)
    assert a is b and len(made) == 1
    Ad = st.A_data.copy()
    Ad[3] *= 2.0
    c = api._problem_for(st.C, Ad, st.A_indices, n, "cuda", make=make)
    assert c is not a and len(made) == 2
    C2 = st.C.copy()
    C2.data[0] += 1.0
    d = api._problem_for(C2, st.A_data, st.A_indices, n, "cuda", make=make)
    assert d is not a and len(made) == 3
    e = api._problem_for(st.C, st.A_data, st.A_indices, n + 1, "cuda", make=make)   # other m
    assert e is not a and len(made) == 4
    assert api._problem_for(st.C, list(st.A_data), st.A_indices, n, "cuda", make=make) is made[-1]
    assert len(made) == 5                                  # not a host array: no caching
    for _ in range(10):                                    # bounded
        Ad = Ad.copy()
        Ad[0] += 1.0
        api._problem_for(st.C, Ad, st.A_indices, n, "cuda", make=make)
    assert len(api._LAYOUTS) == api._LAYOUTS_MAX
    api._LAYOUTS.clear()
