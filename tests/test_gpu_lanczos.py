"""GPU parity of the operator callbacks and of eigsh_smallest against the oracle."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import lanczos as olz
from oracle import maxcut as omaxcut
from oracle import operators as oops
from oracle import qap as oqap
from oracle import rng as orng
from usbs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def test_apply_A_operator_and_adjoint_qap(cuda):
    from usbs_gb300 import api
    from usbs_gb300.problem import DeviceProblem, layout
    D, W = wl.qap_instance(6, 0, grid=5)
    st = oqap.initialize_state(D, W, 6)
    n, m = st.C.shape[0], st.b.shape[0]
    prob = DeviceProblem(layout(st.C, st.A_data, st.A_indices, m=m), cuda)
    rs = np.random.default_rng(0)
    U = rs.standard_normal((n, 3))
    z = rs.standard_normal(m)
    got = _np(api.apply_A_operator_batched(m, None, None, U, problem=prob))
    ref = oops.apply_A_operator_batched(m, st.A_data, st.A_indices, U)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)
    got = _np(api.apply_A_adjoint_batched(n, None, None, z, U, problem=prob))
    ref = oops.apply_A_adjoint_batched(n, st.A_data, st.A_indices, z, U)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)
    got = _np(api.apply_A_operator_slim(m, st.A_data, st.A_indices, U[:, 0], n=n))
    np.testing.assert_allclose(got, oops.apply_A_operator_slim(m, st.A_data, st.A_indices,
                                                               U[:, 0]), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("precision,tol", [(64, 1e-13), (32, 2e-6)])
def test_operator_apply_maxcut(cuda, precision, tol):
    from usbs_gb300 import api
    from usbs_gb300.problem import DeviceProblem, layout
    Wg = wl.torus_graph(40, 1)
    st = omaxcut.initialize_state(Wg, 4)
    n = st.C.shape[0]
    prob = DeviceProblem(layout(st.C, st.A_data, st.A_indices, m=n), cuda)
    rs = np.random.default_rng(1)
    w = rs.standard_normal(n)
    x = rs.standard_normal(n)
    ref = olz.make_operator((-st.C).tocsr(), st.A_data, st.A_indices, w)(x)
    got = _np(api.operator_apply(prob, -1.0, w, x, precision=precision)).astype(np.float64)
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


def _subspace_gap(A, B):
    """Largest principal-angle sine between the column spans of A and B."""
    qa, _ = np.linalg.qr(A)
    qb, _ = np.linalg.qr(B)
    s = np.linalg.svd(qa.T @ qb, compute_uv=False)
    return float(np.sqrt(max(0.0, 1.0 - s.min() ** 2)))


@pytest.mark.parametrize("name,nd,restarts,tol", [("er", 5, 200, 1e-9), ("torus", 4, 300, 1e-9),
                                                  ("er", 11, 10, 1e-7)])
def test_eigsh_fp64_matches_oracle(cuda, name, nd, restarts, tol):
    """Converged Ritz pairs agree to round-off.  With the reference's default
    budget (10 restarts, tol 1e-7) the trailing Ritz vectors are not converged;
    those directions depend on summation order in any two FP64 implementations,
    so only the converged ones are held to round-off there."""
    from usbs_gb300 import api
    from usbs_gb300.problem import DeviceProblem, layout
    Wg = wl.er_graph(800, 19176, 0) if name == "er" else wl.torus_graph(30, 1)
    st = omaxcut.initialize_state(Wg, 4)
    n = st.C.shape[0]
    prob = DeviceProblem(layout(st.C, st.A_data, st.A_indices, m=n), cuda)
    y = np.random.default_rng(2).standard_normal(n) * 0.5
    q0 = orng.default_q0(n)
    ov, oV, ost = olz.eigsh_smallest(n, (-st.C).tocsr(), st.A_data, st.A_indices, y, q0, nd, 32,
                                     restarts, tol)
    gv, gV, info = api.eigsh_smallest(n, prob, None, None, y, q0, nd, 32, restarts, tol,
                                      c_scale=-1.0, precision=64, return_info=True)
    gv, gV = _np(gv), _np(gV)
    assert info.status == 0
    assert info.restarts == ost["restart"] and info.num_converged == ost["nconv"]
    nc = min(nd, ost["nconv"])
    np.testing.assert_allclose(gv[:nc], ov[:nc], rtol=1e-9, atol=1e-9 * np.abs(ov).max())
    for j in range(nc):
        assert abs(gV[:, j] @ oV[:, j]) > 1 - 1e-12, j
    # unconverged tail: still Ritz values of the same operator to the residual level
    assert np.abs(gv - ov).max() <= 1e-4 * np.abs(ov).max()
    np.testing.assert_allclose(gV.T @ gV, np.eye(nd), atol=1e-10)
    # residuals: ||Op v - theta v|| small for the converged pairs
    Op = (-st.C).toarray() + np.diag(y)
    r = np.linalg.norm(Op @ gV[:, :nc] - gV[:, :nc] * gv[None, :nc], axis=0)
    assert r.max() < 10 * tol + 1e-9


def test_eigsh_fp32_close_to_oracle(cuda):
    from usbs_gb300 import api
    from usbs_gb300.problem import DeviceProblem, layout
    Wg = wl.torus_graph(60, 1)
    st = omaxcut.initialize_state(Wg, 4)
    n = st.C.shape[0]
    prob = DeviceProblem(layout(st.C, st.A_data, st.A_indices, m=n), cuda)
    y = np.zeros(n)
    q0 = orng.default_q0(n)
    ov, oV, _ = olz.eigsh_smallest(n, (-st.C).tocsr(), st.A_data, st.A_indices, y, q0, 10, 32, 10,
                                   1e-7)
    gv, gV, info = api.eigsh_smallest(n, prob, None, None, y, q0, 10, 32, 10, 1e-7, c_scale=-1.0,
                                      precision=32, return_info=True)
    gv = _np(gv)
    scale = np.abs(ov).max()
    assert np.abs(gv - ov).max() < 1e-4 * scale
    assert info.status == 0


def test_eigsh_path_laplacian_known_spectrum(cuda):
    from usbs_gb300 import api
    n = 500
    W = sp.diags([np.ones(n - 1), np.ones(n - 1)], [-1, 1]).tocsr()
    L = (sp.diags(np.asarray(W.sum(1)).ravel()) - W).tocsr()
    A_data, A_idx, _, _ = omaxcut.get_all_problem_data(n)
    exact = 2.0 - 2.0 * np.cos(np.pi * np.arange(n) / n)
    gv, gV = api.eigsh_smallest(n, L, A_data, A_idx, np.zeros(n), orng.default_q0(n), 3, 32,
                                300, 1e-10)
    np.testing.assert_allclose(_np(gv), exact[:3], atol=1e-8)


def test_eigsh_breakdown_small_operator(cuda):
    """n < inner iterations forces a Krylov breakdown (solver/lanczos.py:107-117)."""
    from usbs_gb300 import api
    n = 8
    rs = np.random.default_rng(5)
    Wd = rs.random((n, n)); Wd = np.triu(Wd, 1); Wd = Wd + Wd.T
    st = omaxcut.initialize_state(sp.csr_matrix(Wd), 2)
    A_data, A_idx = st.A_data, st.A_indices
    q0 = orng.default_q0(n)
    ov, oV, _ = olz.eigsh_smallest(n, (-st.C).tocsr(), A_data, A_idx, np.zeros(n), q0, 3, 8, 3,
                                   1e-12)
    gv, gV, info = api.eigsh_smallest(n, st.C, A_data, A_idx, np.zeros(n), q0, 3, 8, 3, 1e-12,
                                      c_scale=-1.0, return_info=True)
    np.testing.assert_allclose(_np(gv), ov, atol=1e-9)
    ex = np.linalg.eigvalsh((-st.C).toarray())[:3]
    np.testing.assert_allclose(_np(gv), ex, atol=1e-9)


def _ragged_csr(n, base_len, long_rows, long_len, seed):
    rs = np.random.default_rng(seed)
    lens = rs.integers(0, 2 * base_len + 1, size=n)
    lens[rs.choice(n, size=min(long_rows, n), replace=False)] = long_len
    rowptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    col = rs.integers(0, n, size=int(rowptr[-1])).astype(np.int32)
    val = rs.standard_normal(int(rowptr[-1]))
    return sp.csr_matrix((val, col, rowptr), shape=(n, n))


# (n, typical entries per row, rows with long_len entries, long_len): tails that are
# not multiples of 16 bytes, tiles above the staging capacity, empty rows, dense rows
@pytest.mark.parametrize("shape", [(1, 1, 0, 0), (257, 3, 0, 0), (1000, 7, 3, 40),
                                   (5003, 2, 2, 4000), (4099, 12, 1, 300), (3001, 30, 0, 0)])
@pytest.mark.parametrize("precision", [64, 32])
def test_operator_apply_ragged_csr(cuda, shape, precision):
    import ctypes
    import torch
    from usbs_gb300 import _lib
    lib = _lib.load()
    M = _ragged_csr(*shape, seed=shape[0])
    n, nnz = M.shape[0], M.nnz
    vt = torch.float64 if precision == 64 else torch.float32
    rs = np.random.default_rng(3)
    x = rs.standard_normal(n)
    rp = torch.tensor(M.indptr, dtype=torch.int32, device=cuda)
    cl = torch.tensor(M.indices, dtype=torch.int32, device=cuda)
    vv = torch.tensor(M.data, dtype=vt, device=cuda)
    xx = torch.tensor(x, dtype=vt, device=cuda)
    y = torch.full((n,), float("nan"), dtype=vt, device=cuda)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.usbs_operator_apply(n, nnz, p(rp), p(cl), p(vv), p(xx), p(y), precision, s) == 0
    got = y.double().cpu().numpy()
    Mv = M.astype(np.float32).astype(np.float64) if precision == 32 else M
    xr = x.astype(np.float32).astype(np.float64) if precision == 32 else x
    ref = Mv @ xr
    scale = np.abs(Mv).sum(axis=1).A1 * np.abs(xr).max() + 1e-300
    tol = 1e-13 if precision == 64 else 2e-6
    assert np.all(np.abs(got - ref) <= tol * scale)


@pytest.mark.parametrize("shape", [(1, 1, 0, 0), (257, 3, 0, 0), (1000, 7, 3, 40),
                                   (5003, 2, 2, 4000), (4099, 12, 1, 300)])
@pytest.mark.parametrize("precision", [64, 32])
def test_sell_apply_matches_csr(cuda, shape, precision):
    """usbs_operator_apply_sell on the sliced-ELL layout equals the CSR apply."""
    import ctypes
    import torch
    from usbs_gb300 import _lib
    from usbs_gb300.problem import sell_layout
    lib = _lib.load()
    M = _ragged_csr(*shape, seed=shape[0] + 1)
    n = M.shape[0]
    vt = torch.float64 if precision == 64 else torch.float32
    L = sell_layout(M.indptr, M.indices)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    dev = lambda a, dt: torch.tensor(a, dtype=dt, device=cuda)
    csr_val = dev(M.data, vt)
    sl_val = torch.empty(max(L["stored"], 1), dtype=vt, device=cuda)
    src = dev(L["sl_src"], torch.int32)
    assert lib.usbs_gather_values(L["stored"], p(src), p(csr_val), p(sl_val), precision, s) == 0
    x = dev(np.random.default_rng(5).standard_normal(n), vt)
    y = torch.full((n,), float("nan"), dtype=vt, device=cuda)
    assert lib.usbs_operator_apply_sell(n, p(dev(L["sl_ptr"], torch.int32)),
                                        p(dev(L["sl_col"], torch.int32)), p(sl_val),
                                        p(dev(L["sl_row"], torch.uint8)), p(x), p(y), precision,
                                        s) == 0
    torch.cuda.synchronize()
    xr = x.double().cpu().numpy()
    Mv = M.astype(np.float32).astype(np.float64) if precision == 32 else M
    ref = Mv @ xr
    scale = np.abs(Mv).sum(axis=1).A1 * np.abs(xr).max() + 1e-300
    tol = 1e-13 if precision == 64 else 2e-6
    assert np.all(np.abs(y.double().cpu().numpy() - ref) <= tol * scale)


@pytest.mark.parametrize("a_words,b_words,blocks", [(1000, 3000, 7), (4096, 0, 1), (0, 777, 3)])
def test_stream_probe_reads_every_word_once(cuda, a_words, b_words, blocks):
    """usbs_stream_probe (the bandwidth reference of the bench's SpMV leg) reads
    each 16-byte word of both buffers exactly once: the blocks' XORs combine to
    the XOR of a, their sums to the sum of b; unaligned sizes are rejected."""
    import ctypes
    import torch
    from usbs_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(a_words + b_words)
    a = torch.tensor(rng.integers(-2 ** 31, 2 ** 31, 4 * max(a_words, 1)), dtype=torch.int32,
                     device=cuda)
    b = torch.tensor(rng.integers(-8, 9, 4 * max(b_words, 1)), dtype=torch.float32, device=cuda)
    sums = torch.full((blocks,), float("nan"), dtype=torch.float32, device=cuda)
    xors = torch.full((blocks,), -1, dtype=torch.int32, device=cuda)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.usbs_stream_probe(p(a), 16 * a_words, p(b), 16 * b_words, blocks, p(sums), p(xors),
                                 s) == 0
    torch.cuda.synchronize()
    want_x = np.bitwise_xor.reduce(a.cpu().numpy()[:4 * a_words]) if a_words else 0
    got_x = np.bitwise_xor.reduce(xors.cpu().numpy())
    assert got_x == want_x
    # small integers: every partial sum is exact in FP32
    assert float(sums.double().sum()) == float(b.cpu().numpy()[:4 * b_words].sum())
    assert lib.usbs_stream_probe(p(a), 8, p(b), 0, 1, p(sums), p(xors), s) == -2


# Problems too large for one cluster: the cooperative team kernel while x fits
# in shared memory (n = 15,625 in FP64), the stream path past that (a
# sequence of full-GPU launches; n > 20,480 in FP64, 40,960 in FP32)
@pytest.mark.parametrize("side,precision,kind", [(125, 64, 0), (150, 64, 2), (210, 32, 2)])
def test_eigsh_team_and_stream_paths_match_oracle(cuda, side, precision, kind):
    from usbs_gb300 import _lib, api
    from usbs_gb300.problem import DeviceProblem, layout
    Wg = wl.er_graph(side * side, 4 * side * side, side)
    st = omaxcut.initialize_state(Wg, 4)
    n = st.C.shape[0]
    assert _lib.load().usbs_lanczos_kernel(n, 32, precision) == kind
    prob = DeviceProblem(layout(st.C, st.A_data, st.A_indices, m=n), cuda)
    y = np.random.default_rng(3).standard_normal(n) * 0.5
    q0 = orng.default_q0(n)
    nd, restarts, tol = 4, 60, (1e-8 if precision == 64 else 1e-5)
    ov, oV, ost = olz.eigsh_smallest(n, (-st.C).tocsr(), st.A_data, st.A_indices, y, q0, nd, 32,
                                     restarts, tol)
    gv, gV, info = api.eigsh_smallest(n, prob, None, None, y, q0, nd, 32, restarts, tol,
                                      c_scale=-1.0, precision=precision, return_info=True)
    gv, gV = _np(gv), _np(gV).astype(np.float64)
    assert info.status == 0
    scale = np.abs(ov).max()
    if precision == 64:
        assert ost["nconv"] >= nd
        assert info.restarts == ost["restart"] and info.num_converged == ost["nconv"]
        np.testing.assert_allclose(gv, ov, rtol=1e-9, atol=1e-9 * scale)
        for j in range(nd):
            assert abs(gV[:, j] @ oV[:, j]) > 1 - 1e-10, j
    else:
        assert np.abs(gv - ov).max() < 1e-4 * scale
    Op = ((-st.C) + sp.diags(y)).tocsr()
    r = np.linalg.norm(Op @ gV - gV * gv[None, :], axis=0)
    assert r.max() < (1e-6 if precision == 64 else 1e-2) * scale


def _maxcut_case(cuda, Wg, seed):
    from usbs_gb300.problem import DeviceProblem, layout
    st = omaxcut.initialize_state(Wg, 4)
    n = st.C.shape[0]
    prob = DeviceProblem(layout(st.C, st.A_data, st.A_indices, m=n), cuda)
    y = np.random.default_rng(seed).standard_normal(n) * 0.5
    return st, prob, y, orng.default_q0(n)


# Many independent instances in one launch: six small graphs run as clusters
# of one launch; with a 22,500-node graph in the batch every problem runs on
# the cooperative team kernel, one team per problem
@pytest.mark.parametrize("with_large,precision", [(False, 64), (True, 64), (False, 32),
                                                   (True, 32)])
def test_eigsh_batched_matches_oracle(cuda, with_large, precision):
    from usbs_gb300 import api
    graphs = [wl.er_graph(300 + 100 * i, 2000 + 900 * i, 10 + i) for i in range(6)]
    if with_large:
        graphs.insert(2, wl.er_graph(22500, 90000, 150))
    cases = [_maxcut_case(cuda, g, 20 + i) for i, g in enumerate(graphs)]
    nd, restarts = 4, 200
    tol = 1e-9 if precision == 64 else 1e-5
    out = api.eigsh_smallest_batched([(p, y, q0) for _, p, y, q0 in cases], nd, 32, restarts, tol,
                                     c_scale=-1.0, precision=precision, return_info=True)
    assert len(out) == len(cases)
    for (st, p, y, q0), (gv, gV, info) in zip(cases, out):
        n = p.n
        ov, oV, ost = olz.eigsh_smallest(n, (-st.C).tocsr(), st.A_data, st.A_indices, y, q0, nd,
                                         32, restarts, tol)
        gv, gV = _np(gv), _np(gV).astype(np.float64)
        assert info.status == 0 and ost["nconv"] >= nd
        scale = np.abs(ov).max()
        if precision == 64:
            np.testing.assert_allclose(gv, ov, rtol=1e-9, atol=1e-9 * scale)
            for j in range(nd):
                assert abs(gV[:, j] @ oV[:, j]) > 1 - 1e-10, (n, j)
        else:
            assert np.abs(gv - ov).max() < 1e-4 * scale, n
            Op = ((-st.C) + sp.diags(y)).tocsr()
            r = np.linalg.norm(Op @ gV - gV * gv[None, :], axis=0)
            assert r.max() < 1e-2 * scale, n


def test_eigsh_batched_many_matches_single_calls(cuda):
    """More problems than one launch takes (48): the batch splits; every result
    equals that of a separate eigsh_smallest call to round-off."""
    from usbs_gb300 import api
    cases = [_maxcut_case(cuda, wl.er_graph(200 + 7 * i, 1200 + 40 * i, 100 + i), 300 + i)
             for i in range(53)]
    nd, restarts, tol = 3, 100, 1e-9
    out = api.eigsh_smallest_batched([(p, y, q0) for _, p, y, q0 in cases], nd, 32, restarts, tol,
                                     c_scale=-1.0, precision=64)
    for (st, p, y, q0), (gv, gV) in zip(cases, out):
        sv, sV = api.eigsh_smallest(p.n, p, None, None, y, q0, nd, 32, restarts, tol,
                                    c_scale=-1.0, precision=64)
        sv, gv = _np(sv), _np(gv)
        np.testing.assert_allclose(gv, sv, rtol=1e-10, atol=1e-10 * np.abs(sv).max())
        G = _np(gV).T @ _np(sV)
        assert np.abs(np.abs(np.diag(G)) - 1).max() < 1e-9


def test_lanczos_autotune_records_a_choice_and_keeps_parity(cuda):
    """The tuner times the cluster sizes on a batch, records the fastest for
    the class, and the class's later launches (which use it) still match the
    oracle; an explicit rows-per-CTA request in a solve overrides the table."""
    from usbs_gb300 import api, solver
    api.set_lanczos_tuning([], clear=True)
    cases = [_maxcut_case(cuda, wl.er_graph(1500 + 200 * i, 12000, 40 + i), 50 + i)
             for i in range(4)]
    probs = [(p, y, q0) for _, p, y, q0 in cases]
    nd, restarts, tol = 4, 200, 1e-9
    r = api.lanczos_autotune(probs, nd, 32, restarts, tol, c_scale=-1.0, precision=64)
    assert r["rows_per_cta"] in api.TUNE_CANDIDATES
    timed = [m for m in r["ms"].values() if m is not None]
    assert len(timed) >= 2 and min(timed) == r["ms"][r["rows_per_cta"]]
    tab = api.lanczos_tuning()
    assert tab == [{"precision": 64, "log2_count": 2, "log2_max_n": 11,
                    "rows_per_cta": r["rows_per_cta"]}]
    out = api.eigsh_smallest_batched(probs, nd, 32, restarts, tol, c_scale=-1.0, precision=64)
    for (st, p, y, q0), (gv, _) in zip(cases, out):
        ov, _, _ = olz.eigsh_smallest(p.n, (-st.C).tocsr(), st.A_data, st.A_indices, y, q0, nd,
                                      32, restarts, tol)
        np.testing.assert_allclose(_np(gv), ov, rtol=1e-9, atol=1e-9 * np.abs(ov).max())
    api.set_lanczos_tuning([], clear=True)
    # a solve's own packing: same iterates as the default spread to round-off
    st = omaxcut.initialize_state(wl.er_graph(2000, 12000, 3), 10)
    n = st.C.shape[0]
    args = (st, n, n, 2.0 * n, 2.0, 0.01, 0.25, 4, 1, 2, np.inf, -1.0, -1.0, -1.0, 32, 200, 1e-9,
            100)
    a, atr, _ = solver.usbs(*args, q0=orng.default_q0(n), precision=64, return_trace=True)
    b, btr, _ = solver.usbs(*args, q0=orng.default_q0(n), precision=64, return_trace=True,
                            lanczos_rows_per_cta=640)
    for key in ("primal_obj", "obj_ub", "pen_dual_obj", "tr_X"):
        assert abs(atr[0][key] - btr[0][key]) <= 1e-9 * max(1.0, abs(atr[0][key])), key


# The stream path's breakdown branch: on the zero operator every Lanczos step
# breaks down (y = 0), and each step's vector is replaced by a Gaussian vector
# keyed by the step, orthogonalised twice against the basis
# (solver/lanczos.py:107-117).  The oracle draws the same vectors.
@pytest.mark.parametrize("precision", [64, 32])
def test_stream_path_breakdown_on_zero_operator(cuda, precision):
    from usbs_gb300 import _lib, api
    from usbs_gb300.problem import DeviceProblem, layout
    n = 50000
    C = sp.csr_matrix((n, n))
    A_idx = np.stack([np.arange(n)] * 3, 1)
    assert _lib.load().usbs_lanczos_kernel(n, 32, precision) == 2
    prob = DeviceProblem(layout(C, np.ones(n), A_idx, m=n), cuda)
    y = np.zeros(n)
    q0 = orng.default_q0(n)
    ov, oV, ost = olz.eigsh_smallest(n, C, np.ones(n), A_idx, y, q0, 4, 32, 3, 1e-7)
    gv, gV, info = api.eigsh_smallest(n, prob, None, None, y, q0, 4, 32, 3, 1e-7, c_scale=-1.0,
                                      precision=precision, return_info=True)
    gv, gV = _np(gv), _np(gV).astype(np.float64)
    assert info.status == 0 and info.breakdowns > 0
    assert info.restarts == ost["restart"] and info.num_converged == ost["nconv"]
    assert np.abs(gv).max() < 1e-12 and np.abs(ov).max() < 1e-12
    G = gV.T @ gV
    assert np.abs(G - np.eye(4)).max() < (1e-12 if precision == 64 else 1e-5)
