"""ctypes binding of the native library libsod_gb300.so (C ABI declared in include/sod_gb300.h).

The package has no CPU fallback: if the shared library is missing or fails to load, every entry
point raises.  Buffers may be numpy arrays (host) or torch CUDA tensors (device); the library
detects device pointers itself and stages host buffers through its own device memory.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsod_gb300.so")

SOD_OK, SOD_ERR_INVALID_ARG, SOD_ERR_OOM, SOD_ERR_CUDA, SOD_ERR_NO_DEVICE, SOD_ERR_TIMEOUT, \
    SOD_ERR_UNSUPPORTED, SOD_ERR_CAPACITY = range(8)
G, H, B_TRANS, B_ANGULAR = 0, 1, 2, 3
KINDS = {"G": G, "H": H, "B_trans": B_TRANS, "B_angular": B_ANGULAR}
COLLOCATION, GALERKIN = 0, 1
C128, C64, F64, F32, BF16 = 0, 1, 2, 3, 4
PART_REGULAR, PART_SINGULAR, PART_ALL = 1, 2, 3
HISTORY_ENGINE_AUTO, HISTORY_ENGINE_CUDA_CORES, HISTORY_ENGINE_TENSOR_CORES = 0, 1, 2
PRECISION_AUTO, PRECISION_FP32, PRECISION_COMPENSATED = 0, 1, 2

# every function the header declares, with its ctypes signature
_c = ctypes
_P = _c.c_void_p
_SIGS = {
    "sod_version": ([], _c.c_int),
    "sod_last_error": ([], _c.c_char_p),
    "sod_triangle_rule": ([_c.c_int, _P, _P], _c.c_int),
    "sod_cq_frequencies": ([_c.c_int, _c.c_double, _c.c_int, _P, _P, _P], _c.c_int),
    "sod_context_create": ([_c.c_int, _P], _c.c_int),
    "sod_context_destroy": ([_P], _c.c_int),
    "sod_context_set_stream": ([_P, _P], _c.c_int),
    "sod_context_synchronize": ([_P], _c.c_int),
    "sod_context_set_tuning": ([_P, _c.c_int, _c.c_int], _c.c_int),
    "sod_context_set_wait_test": ([_P, _c.c_int], _c.c_int),
    "sod_context_set_precision": ([_P, _c.c_int], _c.c_int),
    "sod_context_launch_count": ([_P], _c.c_int64),
    "sod_mesh_create": ([_P, _P, _c.c_int, _P, _c.c_int, _P, _P, _P], _c.c_int),
    "sod_mesh_destroy": ([_P], _c.c_int),
    "sod_face_colouring": ([_P, _c.c_int, _c.c_int, _c.c_int, _P, _P], _c.c_int),
    "sod_cqbem_assemble": ([_P, _P, _c.c_int, _c.c_int, _c.c_double, _c.c_double, _c.c_double, _c.c_double,
                            _c.c_double, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _P, _c.c_int], _c.c_int),
    "sod_cqbem_assemble_frequencies": ([_P, _P, _c.c_int, _c.c_int, _c.c_double, _c.c_double, _c.c_double, _P,
                                        _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _P, _c.c_int],
                                       _c.c_int),
    "sod_cqbem_assemble_all": ([_P, _P, _c.c_int, _c.c_double, _c.c_double, _c.c_double, _P, _c.c_int, _c.c_int,
                                _c.c_int, _c.c_int, _c.c_int, _c.c_int, _P, _P, _P, _P, _c.c_int], _c.c_int),
    "sod_cqbem_assemble_noalloc": ([_P, _P, _c.c_int, _c.c_double, _c.c_double, _c.c_double, _P, _c.c_int,
                                    _c.c_int, _c.c_int, _c.c_int, _c.c_int, _P, _c.c_int], _c.c_int),
    "sod_cqbem_precompute": ([_P, _P, _c.c_int, _c.c_double, _c.c_double, _c.c_double, _c.c_double, _c.c_int,
                              _c.c_double, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _P, _P, _P, _P, _P, _P,
                              _c.c_int], _c.c_int),
    "sod_batch_create": ([_P, _c.c_int, _c.c_int, _P], _c.c_int),
    "sod_batch_add": ([_P, _P, _c.c_double, _c.c_double, _c.c_double, _P, _c.c_int, _c.c_int, _c.c_int, _c.c_int,
                       _c.c_int, _P, _P, _P, _P], _c.c_int),
    "sod_batch_finalize": ([_P], _c.c_int),
    "sod_batch_run": ([_P], _c.c_int),
    "sod_batch_launch_count": ([_P], _c.c_int),
    "sod_batch_profile": ([_P, _c.c_int, _P, _P, _P], _c.c_int),
    "sod_batch_destroy": ([_P], _c.c_int),
    "sod_elastostatic_assemble": ([_P, _P, _c.c_int, _c.c_int, _c.c_double, _c.c_double, _c.c_int, _c.c_int,
                                   _c.c_int, _c.c_int, _P, _c.c_int], _c.c_int),
    "sod_server_create": ([_c.c_int, _c.c_int64, _c.c_int, _c.c_int, _P], _c.c_int),
    "sod_server_submit_assembly": ([_P, _P, _c.c_int, _P, _c.c_int, _c.c_double, _c.c_double, _c.c_double, _c.c_int,
                                    _c.c_double, _c.c_int, _c.c_int, _c.c_int, _P], _c.c_int),
    "sod_server_submit_step": ([_P, _c.c_int64, _P, _P, _c.c_int, _P], _c.c_int),
    "sod_server_poll": ([_P, _P, _P, _P, _c.c_int, _P], _c.c_int),
    "sod_server_result": ([_P, _c.c_int64, _P, _c.c_int], _c.c_int),
    "sod_server_drain": ([_P, _c.c_double], _c.c_int),
    "sod_server_stats": ([_P, _P, _P], _c.c_int),
    "sod_server_destroy": ([_P], _c.c_int),
    "sod_history_create": ([_P, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _P], _c.c_int),
    "sod_history_set_weights": ([_P, _c.c_int, _P, _P, _c.c_int], _c.c_int),
    "sod_history_set_b": ([_P, _c.c_int, _P], _c.c_int),
    "sod_history_push": ([_P, _P, _P, _P], _c.c_int),
    "sod_history_convolve": ([_P, _P], _c.c_int),
    "sod_history_reset": ([_P], _c.c_int),
    "sod_solver_create": ([_P, _c.c_int, _P, _P], _c.c_int),
    "sod_solver_solve": ([_P, _c.c_int, _P, _P], _c.c_int),
    "sod_solver_inverse": ([_P, _P], _c.c_int),
    "sod_solver_destroy": ([_P], _c.c_int),
    "sod_solver_keep_inverse": ([_P], _c.c_int),
    "sod_history_convolve_solve": ([_P, _P, _P], _c.c_int),
    "sod_lstsq_create": ([_P, _c.c_int, _c.c_int, _P, _P], _c.c_int),
    "sod_lstsq_rank": ([_P, _P], _c.c_int),
    "sod_lstsq_solve": ([_P, _c.c_int, _P, _P], _c.c_int),
    "sod_lstsq_pinv": ([_P, _P], _c.c_int),
    "sod_lstsq_destroy": ([_P], _c.c_int),
    "sod_elastostatic_u_p": ([_P, _P, _P, _P, _P], _c.c_int),
    "sod_elastostatic_rigid_modes": ([_P, _P, _P], _c.c_int),
    "sod_mat_write": ([_P, _c.c_char_p, _P, _c.c_int64, _c.c_int64, _c.c_int], _c.c_int),
    "sod_mat_read": ([_P, _c.c_char_p, _P, _c.c_int64, _c.c_int64], _c.c_int),
    "sod_cqbem_write_cache": ([_P, _c.c_char_p, _c.c_int, _c.c_int, _P, _P, _P, _P, _c.c_int], _c.c_int),
    "sod_history_set_engine": ([_P, _c.c_int], _c.c_int),
    "sod_history_create_compressed": ([_P, _c.c_int, _c.c_int, _c.c_double, _P], _c.c_int),
    "sod_history_compressed_matrix": ([_P, _c.c_int, _c.c_int, _P, _P, _P, _P], _c.c_int),
    "sod_history_write_cpmat": ([_P, _c.c_int, _c.c_int, _c.c_char_p], _c.c_int),
    "sod_history_bytes": ([_P, _P], _c.c_int),
    "sod_history_destroy": ([_P], _c.c_int),
    "sod_cq_inverse_transform": ([_P, _P, _c.c_int, _c.c_int64, _c.c_int, _c.c_int, _c.c_double, _P, _c.c_int],
                                 _c.c_int),
}

_lib = None


class SodError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[sod status {code}] {msg}")
        self.code = code


def load() -> ctypes.CDLL:
    """Load the native library (building it first if the sources are newer)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"native library not built: {LIB_PATH} (run surfaceonlydeformables_gb300/build.py)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib


def declared_symbols() -> list[str]:
    return list(_SIGS)


def check(rc: int) -> None:
    if rc != SOD_OK:
        raise SodError(rc, load().sod_last_error().decode(errors="replace"))


def ptr(a) -> ctypes.c_void_p | None:
    """Raw pointer of a numpy array or torch tensor (None -> NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags.c_contiguous, "arrays must be C-contiguous"
        return ctypes.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):
        assert a.is_contiguous(), "tensors must be contiguous"
        return ctypes.c_void_p(a.data_ptr())
    raise TypeError(f"unsupported buffer type {type(a)}")


def triangle_rule(order: int) -> np.ndarray:
    out = np.zeros((13, 4))
    n = ctypes.c_int()
    check(load().sod_triangle_rule(order, ptr(out), ctypes.byref(n)))
    return out[: n.value].copy()


def cq_frequencies(bdf: int, dt: float, N: int):
    """(s_l for l = 0..L/2, R, L) of the convolution quadrature (BDF1/BDF2)."""
    s = np.zeros(2 * (N // 2 + 2))
    R = ctypes.c_double()
    L = ctypes.c_int()
    check(load().sod_cq_frequencies(bdf, dt, N, ptr(s), ctypes.byref(R), ctypes.byref(L)))
    lam = L.value // 2 + 1
    return s[: 2 * lam].view(np.complex128).copy(), R.value, L.value
