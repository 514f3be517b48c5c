"""usbs_eigsh_smallest_noalloc (fixed static device scratch) against
usbs_eigsh_smallest (caller workspace), both called through the C ABI.

Kept in its own file, collected last, so that it runs both alone and after
every other test has used the library on the same device."""
import ctypes

import numpy as np
import pytest

from usbs_gb300 import workloads as wl

STATIC_SCRATCH_BYTES = 16 << 20     # USBS_EIGSH_STATIC_SCRATCH_BYTES


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


# the three Lanczos paths: one cluster (ER 600), the cooperative team kernel
# (ER 15,000 in FP64) and the stream path (RGG 25,000 in FP64, ER 45,000 in
# FP32), whose scratch also holds per-CTA partial sums, barrier counters or
# the loop's control block and the operator's sliced-ELL copy
GRAPHS = {"er600": lambda: wl.er_graph(600, 6000, 5),
          "er15k": lambda: wl.er_graph(15000, 60000, 21),
          "rgg25k": lambda: wl.rgg_knn_graph(25000, 6, 22),
          "er45k": lambda: wl.er_graph(45000, 120000, 23)}
KIND = {"er600": 1, "er15k": 0, "rgg25k": 2, "er45k": 2}


def _setup(device, precision, graph="er600"):
    import torch
    from oracle import maxcut as omaxcut
    from usbs_gb300.problem import DeviceProblem, layout
    Wg = GRAPHS[graph]()
    st = omaxcut.initialize_state(Wg, 4)
    n = st.C.shape[0]
    prob = DeviceProblem(layout(st.C, st.A_data, st.A_indices, m=n), device)
    vt = torch.float64 if precision == 64 else torch.float32
    rs = np.random.default_rng(11)
    ys, q0s = [], []
    for _ in range(2):
        ys.append(torch.tensor(rs.standard_normal(n), dtype=torch.float64, device=device))
        q = rs.standard_normal(n)
        q0s.append(torch.tensor(q / np.linalg.norm(q), dtype=vt, device=device))
    return prob, n, vt, ys, q0s


def _call(lib, noalloc, prob, n, vt, y, q0, precision, nd=6, inner=32, restarts=60, tol=1e-9):
    import torch
    dev = y.device
    ld = (n + 31) // 32 * 32
    Q = torch.zeros((inner + 1, ld), dtype=vt, device=dev)
    evals = torch.zeros(nd, dtype=torch.float64, device=dev)
    info = torch.zeros(16, dtype=torch.int32, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    args = (n, prob.nnz, _ptr(prob.rowptr), _ptr(prob.col), _ptr(prob.c_val), -1.0,
            _ptr(prob.slot_ptr), _ptr(prob.slot_tid), _ptr(prob.t_con), _ptr(prob.t_a0), _ptr(y),
            _ptr(q0), nd, inner, restarts, tol, precision, _ptr(Q), ld, _ptr(evals), _ptr(info))
    if noalloc:
        rc = lib.usbs_eigsh_smallest_noalloc(*args, stream)
    else:
        need = lib.usbs_eigsh_workspace_bytes(n, prob.nnz, inner, precision)
        ws = torch.empty(need, dtype=torch.uint8, device=dev)
        rc = lib.usbs_eigsh_smallest(*args, _ptr(ws), need, stream)
    assert rc == 0, lib.usbs_last_error().decode()
    torch.cuda.synchronize(dev)
    return (evals.cpu().numpy(), Q[:nd, :n].t().double().cpu().numpy(),
            info.cpu().numpy())


@pytest.mark.gpu
@pytest.mark.parametrize("graph,precision,rtol", [("er600", 64, 1e-12), ("er600", 32, 1e-6),
                                                  ("er15k", 64, 1e-12), ("rgg25k", 64, 1e-12),
                                                  ("er45k", 32, 1e-6)])
def test_noalloc_matches_workspace_entry_point(cuda, graph, precision, rtol):
    from usbs_gb300 import _lib
    lib = _lib.load()
    prob, n, vt, ys, q0s = _setup(cuda, precision, graph)
    assert lib.usbs_lanczos_kernel(n, 32, precision) == KIND[graph]
    assert lib.usbs_eigsh_workspace_bytes(n, prob.nnz, 32, precision) <= STATIC_SCRATCH_BYTES
    # two no-alloc calls in a row on different inputs: the second reuses the
    # scratch the first left behind
    got = [_call(lib, True, prob, n, vt, ys[i], q0s[i], precision) for i in range(2)]
    ref = [_call(lib, False, prob, n, vt, ys[i], q0s[i], precision) for i in range(2)]
    for (gv, gV, gi), (rv, rV, ri) in zip(got, ref):
        assert gi[5] == 0 and ri[5] == 0                  # no status bits
        np.testing.assert_array_equal(gi[1:5], ri[1:5])    # converged, restarts, breakdowns, matvecs
        np.testing.assert_allclose(gv, rv, rtol=rtol, atol=rtol * np.abs(rv).max())
        np.testing.assert_allclose(gV, rV, rtol=0, atol=rtol * 10)
    assert not np.allclose(got[0][0], got[1][0])           # the two inputs differ


@pytest.mark.gpu
def test_noalloc_rejects_oversize_on_device(cuda):
    _check_oversize_rejected()


def test_noalloc_rejects_oversize():
    """Size check on the host: rejected before any device work."""
    _check_oversize_rejected()


def _check_oversize_rejected():
    from usbs_gb300 import _lib
    lib = _lib.load()
    n, nnz = 1_000_000, 8_000_000                          # ~80 MB of FP64 scratch
    assert lib.usbs_eigsh_workspace_bytes(n, nnz, 32, 64) > STATIC_SCRATCH_BYTES
    null = ctypes.c_void_p(0)
    rc = lib.usbs_eigsh_smallest_noalloc(n, nnz, null, null, null, -1.0, null, null, null, null,
                                         null, null, 4, 32, 10, 1e-7, 64, null, n, null, null, null)
    assert rc == -2
    msg = lib.usbs_last_error().decode()
    assert "static scratch" in msg and str(STATIC_SCRATCH_BYTES) in msg
