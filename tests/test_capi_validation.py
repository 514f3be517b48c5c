"""The C ABI rejects bad arguments on the host, before any device work: each
call below returns -2 with a message naming the problem.  Runs without a GPU."""
import ctypes

import pytest

from usbs_gb300 import _lib

P = ctypes.c_void_p
FAKE = ctypes.c_void_p(256)        # never dereferenced: every call fails its checks first


@pytest.fixture(scope="module")
def lib():
    lib = _lib.load()
    lib.usbs_last_error.restype = ctypes.c_char_p
    return lib


def _err(lib):
    return lib.usbs_last_error().decode()


@pytest.mark.parametrize("n,ldq,inner,nd,restarts,prec,word", [
    (0, 32, 32, 4, 10, 64, "bad sizes"),        # empty problem
    (100, 99, 32, 4, 10, 64, "bad sizes"),      # ldq < n
    (100, 128, 33, 4, 10, 64, "bad sizes"),     # more than 32 inner vectors
    (100, 128, 8, 9, 10, 64, "bad sizes"),      # more eigenpairs than inner vectors
    (100, 128, 32, 0, 10, 64, "bad sizes"),     # no eigenpair asked for
    (100, 128, 32, 4, -1, 64, "bad sizes"),     # negative restart budget
    (100, 128, 32, 4, 10, 16, "precision"),     # unsupported precision
])
def test_eigsh_rejects_bad_sizes(lib, n, ldq, inner, nd, restarts, prec, word):
    rc = lib.usbs_eigsh_smallest(n, 300, FAKE, FAKE, FAKE, -1.0, FAKE, FAKE, FAKE, FAKE, FAKE, FAKE,
                                 nd, inner, restarts, 1e-7, prec, FAKE, ldq, FAKE, FAKE, FAKE,
                                 1 << 30, None)
    assert rc == -2 and word in _err(lib)


def test_eigsh_rejects_small_workspace_and_bad_nnz(lib):
    rc = lib.usbs_eigsh_smallest(100, 300, FAKE, FAKE, FAKE, -1.0, FAKE, FAKE, FAKE, FAKE, FAKE,
                                 FAKE, 4, 32, 10, 1e-7, 64, FAKE, 128, FAKE, FAKE, FAKE, 16, None)
    assert rc == -2 and "workspace" in _err(lib)
    rc = lib.usbs_eigsh_smallest(100, -1, FAKE, FAKE, FAKE, -1.0, FAKE, FAKE, FAKE, FAKE, FAKE,
                                 FAKE, 4, 32, 10, 1e-7, 64, FAKE, 128, FAKE, FAKE, FAKE, 1 << 30,
                                 None)
    assert rc == -2 and "nnz" in _err(lib)


def test_rounding_rejects_wide_sketch_and_missing_operands(lib):
    assert lib.usbs_round_workspace_bytes(1000, 32) > 0
    assert lib.usbs_round_workspace_bytes(1000, 33) == 0
    assert lib.usbs_round_workspace_bytes(0, 8) == 0
    ws = lib.usbs_round_workspace_bytes(1000, 8)
    rc = lib.usbs_maxcut_round(1000, 33, FAKE, FAKE, 1024, FAKE, FAKE, FAKE, 1e-6, FAKE, None,
                               None, FAKE, ws, None)
    assert rc == -2 and "s must be" in _err(lib)
    rc = lib.usbs_maxcut_round(1000, 8, FAKE, FAKE, 999, FAKE, FAKE, FAKE, 1e-6, FAKE, None, None,
                               FAKE, ws, None)
    assert rc == -2 and "ld=999" in _err(lib)
    rc = lib.usbs_maxcut_round(1000, 8, FAKE, FAKE, 1024, None, FAKE, FAKE, 1e-6, FAKE, None, None,
                               FAKE, ws, None)
    assert rc == -2 and "null" in _err(lib)
    rc = lib.usbs_maxcut_round(1000, 8, FAKE, FAKE, 1024, FAKE, FAKE, FAKE, 1e-6, FAKE, None, None,
                               FAKE, ws - 1, None)
    assert rc == -2 and "workspace" in _err(lib)
    rc = lib.usbs_reconstruct_from_sketch(1000, 8, FAKE, FAKE, 1024, 1e-6, FAKE, 999, FAKE, FAKE,
                                          ws, None)
    assert rc == -2 and "lde" in _err(lib)


def test_operator_entry_points_reject_bad_sizes(lib):
    assert lib.usbs_lanczos_kernel(1000, 32, 16) == -2
    rc = lib.usbs_apply_A_operator(10, 0, FAKE, FAKE, FAKE, FAKE, FAKE, 16, FAKE, None)
    assert rc == -2 and "bad sizes" in _err(lib)
    rc = lib.usbs_apply_A_adjoint(100, 2, FAKE, FAKE, FAKE, FAKE, FAKE, FAKE, 99, FAKE, 128, None)
    assert rc == -2 and "bad sizes" in _err(lib)


def test_qap_round_rejects_bad_sizes(lib):
    assert lib.usbs_qap_round_workspace_bytes(30, 30) > 0
    assert lib.usbs_qap_round_workspace_bytes(65, 8) == 0
    assert lib.usbs_qap_round_workspace_bytes(30, 33) == 0
    ws = lib.usbs_qap_round_workspace_bytes(10, 10)
    rc = lib.usbs_qap_round(65, 10, FAKE, FAKE, 4232, FAKE, FAKE, 1e-6, FAKE, None, None, FAKE,
                            ws, None)
    assert rc == -2 and "l=65" in _err(lib)
    rc = lib.usbs_qap_round(10, 10, FAKE, FAKE, 101, None, FAKE, 1e-6, FAKE, None, None, FAKE, ws,
                            None)
    assert rc == -2 and "null" in _err(lib)
    rc = lib.usbs_qap_round(10, 10, FAKE, FAKE, 100, FAKE, FAKE, 1e-6, FAKE, None, None, FAKE, ws,
                            None)
    assert rc == -2 and "ld=100" in _err(lib)
    rc = lib.usbs_qap_round(10, 10, FAKE, FAKE, 101, FAKE, FAKE, 1e-6, FAKE, None, None, FAKE,
                            ws - 8, None)
    assert rc == -2 and "workspace" in _err(lib)


def test_eigsh_batched_rejects_bad_problems(lib):
    from usbs_gb300.api import EigshProblem
    lib.usbs_eigsh_smallest_batched.argtypes = [ctypes.c_int, ctypes.POINTER(EigshProblem),
                                                ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                ctypes.c_int, P]
    arr = (EigshProblem * 2)()
    for p in arr:
        p.n, p.nnz, p.num_desired, p.ldq = 100, 300, 4, 128
        p.workspace, p.workspace_bytes = 256, 1 << 30
    assert lib.usbs_eigsh_smallest_batched(0, arr, 32, 10, 1e-7, 64, None) == 0   # nothing to do
    assert lib.usbs_eigsh_smallest_batched(2, arr, 33, 10, 1e-7, 64, None) == -2
    assert "inner_iterations" in _err(lib)
    arr[1].ldq = 99
    assert lib.usbs_eigsh_smallest_batched(2, arr, 32, 10, 1e-7, 64, None) == -2
    assert "problem 1" in _err(lib) and "bad sizes" in _err(lib)
    arr[1].ldq = 128
    arr[0].workspace_bytes = 16
    assert lib.usbs_eigsh_smallest_batched(2, arr, 32, 10, 1e-7, 64, None) == -2
    assert "problem 0" in _err(lib) and "workspace" in _err(lib)
    assert lib.usbs_eigsh_smallest_batched(2, arr, 32, 10, 1e-7, 16, None) == -2


def test_lanczos_tuning_table_and_autotune_arguments(lib):
    from usbs_gb300 import api
    api.set_lanczos_tuning([], clear=True)
    assert lib.usbs_lanczos_tuning_put(16, 1, 100, 640) == -2           # precision
    assert lib.usbs_lanczos_tuning_put(32, 1, 100, 8) == -2             # rows per CTA < 16
    assert lib.usbs_lanczos_tuning_put(32, 0, 100, 640) == -2           # count
    api.set_lanczos_tuning([{"precision": 32, "log2_count": 5, "log2_max_n": 12,
                             "rows_per_cta": 640},
                            {"precision": 64, "log2_count": 0, "log2_max_n": 9,
                             "rows_per_cta": 128}])
    got = sorted((e["precision"], e["log2_count"], e["log2_max_n"], e["rows_per_cta"])
                 for e in api.lanczos_tuning())
    assert got == [(32, 5, 12, 640), (64, 0, 9, 128)]
    assert lib.usbs_lanczos_tuning_put(32, 33, 5000, 0) == 0            # erase that class
    assert [e["precision"] for e in api.lanczos_tuning()] == [64]
    api.set_lanczos_tuning([], clear=True)
    assert api.lanczos_tuning() == []
    best = ctypes.c_int(0)
    assert lib.usbs_lanczos_autotune(0, FAKE, 32, 10, 1e-7, 32, None, ctypes.byref(best),
                                     None) == -2
    assert lib.usbs_lanczos_autotune(49, FAKE, 32, 10, 1e-7, 32, None, ctypes.byref(best),
                                     None) == -2
