"""ctypes binding of libusbs_gb300.so (the C ABI in include/usbs_gb300.h).

The library is built in-tree by :mod:`usbs_gb300.build`.  Nothing here falls
back to another implementation: if the library cannot be loaded every entry
point raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libusbs_gb300.so")

_lib = None

c_int, c_ll, c_double, c_size_t, c_void_p = (ctypes.c_int, ctypes.c_longlong, ctypes.c_double,
                                              ctypes.c_size_t, ctypes.c_void_p)
P = c_void_p

# name -> (restype, argtypes); must match include/usbs_gb300.h
SIGNATURES = {
    "usbs_abi_version": (c_int, []),
    "usbs_last_error": (ctypes.c_char_p, []),
    "usbs_device_info": (c_int, [c_int, P, P, P]),
    "usbs_assemble_operator": (c_int, [c_ll, P, c_double, P, P, P, P, P, P, c_int, P]),
    "usbs_operator_apply": (c_int, [c_int, c_ll, P, P, P, P, P, c_int, P]),
    "usbs_operator_apply_sell": (c_int, [c_int, P, P, P, P, P, P, c_int, P]),
    "usbs_gather_values": (c_int, [c_ll, P, P, P, c_int, P]),
    "usbs_stream_probe": (c_int, [P, c_ll, P, c_ll, c_int, P, P, P]),
    "usbs_apply_A_operator": (c_int, [c_int, c_int, P, P, P, P, P, c_int, P, P]),
    "usbs_apply_A_adjoint": (c_int, [c_int, c_int, P, P, P, P, P, P, c_int, P, c_int, P]),
    "usbs_lanczos_kernel": (c_int, [c_int, c_int, c_int]),
    "usbs_eigsh_workspace_bytes": (c_size_t, [c_int, c_ll, c_int, c_int]),
    "usbs_eigsh_smallest": (c_int, [c_int, c_ll, P, P, P, c_double, P, P, P, P, P, P, c_int, c_int, c_int,
                                    c_double, c_int, P, c_int, P, P, P, c_size_t, P]),
    # struct-array entry point; usbs_gb300.api installs the exact ctypes types
    "usbs_eigsh_smallest_batched": (c_int, [c_int, P, c_int, c_int, c_double, c_int, P]),
    "usbs_lanczos_autotune": (c_int, [c_int, P, c_int, c_int, c_double, c_int, P, P, P]),
    "usbs_lanczos_tuning_get": (c_int, [P, P, c_int]),
    "usbs_lanczos_tuning_put": (c_int, [c_int, c_int, c_int, c_int]),
    "usbs_lanczos_tuning_clear": (None, []),
    "usbs_eigsh_smallest_noalloc": (c_int, [c_int, c_ll, P, P, P, c_double, P, P, P, P, P, P, c_int,
                                            c_int, c_int, c_double, c_int, P, c_int, P, P, P]),
    # struct-typed entry points; usbs_gb300.solver installs the exact ctypes types
    "usbs_solve_workspace_bytes": (c_size_t, [P, P]),
    "usbs_solve": (c_int, [P, P, P, P, c_size_t, P, P, P]),
    "usbs_cgal_workspace_bytes": (c_size_t, [P, P]),
    "usbs_cgal_solve": (c_int, [P, P, P, P, c_size_t, P, P, P]),
    "usbs_round_workspace_bytes": (c_size_t, [c_int, c_int]),
    "usbs_reconstruct_from_sketch": (c_int, [c_int, c_int, P, P, c_int, c_double, P, c_int, P, P,
                                             c_size_t, P]),
    "usbs_maxcut_round": (c_int, [c_int, c_int, P, P, c_int, P, P, P, c_double, P, P, P, P,
                                  c_size_t, P]),
    "usbs_qap_round_workspace_bytes": (c_size_t, [c_int, c_int]),
    "usbs_qap_round": (c_int, [c_int, c_int, P, P, c_int, P, P, c_double, P, P, P, P, c_size_t,
                               P]),
    "usbs_selftest_wait_limits": (c_int, [c_int, c_int, c_ll, P, P, P]),
}


class LibraryError(RuntimeError):
    pass


def load(build_if_missing=True):
    """Load (building first if needed) and return the ctypes library handle."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise LibraryError(f"{LIB_PATH} is missing; run python -m usbs_gb300.build")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.usbs_abi_version() != 5:
        raise LibraryError("libusbs_gb300 ABI version mismatch")
    _lib = lib
    return lib


def check(rc, what):
    if rc != 0:
        msg = _lib.usbs_last_error().decode() if _lib is not None else ""
        raise LibraryError(f"{what} failed (rc={rc}): {msg}")
