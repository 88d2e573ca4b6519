"""ctypes binding of libnalgebra_cuda.so (the C ABI declared in include/nalgebra_cuda.h).

The product path: every call goes to a hand-written sm_103a kernel.  There is
no CPU fallback; if the library is missing or fails to load, the error is
raised, never hidden.
"""
from __future__ import annotations

import ctypes as C
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libnalgebra_cuda.so")
HEADER_PATH = os.path.join(os.path.dirname(_HERE), "include", "nalgebra_cuda.h")

NACU_SUCCESS = 0
NACU_ERR_CUDA = 1
NACU_ERR_UNSUPPORTED = 2
FLAG_EXACT = 1
FLAG_NO_FACTORS = 2
FLAG_SUBSTITUTE = 4
FLAG_VERIFY = 8

_vp = C.c_void_p
_i = C.c_int
_i64 = C.c_int64
_d = C.c_double
_sz = C.c_size_t

# name -> (restype, argtypes); pointers are passed as integers (device addresses).
SIGNATURES = {
    "nacu_version": (C.c_char_p, []),
    "nacu_last_error": (C.c_char_p, []),
    "nacu_device_arch": (_i, []),
    "nacu_device_count": (_i, [C.POINTER(C.c_int)]),
    "nacu_malloc": (_i, [C.POINTER(C.c_void_p), _sz]),
    "nacu_free": (_i, [_vp]),
    "nacu_host_alloc": (_i, [C.POINTER(C.c_void_p), _sz]),
    "nacu_host_free": (_i, [_vp]),
    "nacu_memcpy": (_i, [_vp, _vp, _sz, _vp]),
    "nacu_memset": (_i, [_vp, _i, _sz, _vp]),
    "nacu_stream_create": (_i, [C.POINTER(C.c_void_p)]),
    "nacu_stream_destroy": (_i, [_vp]),
    "nacu_stream_synchronize": (_i, [_vp]),
    "nacu_stream_wait": (_i, [_vp, _vp]),
    "nacu_device_synchronize": (_i, []),
    "nacu_graph_begin_capture": (_i, [_vp]),
    "nacu_graph_end_capture": (_i, [_vp, C.POINTER(C.c_void_p)]),
    "nacu_graph_launch": (_i, [_vp, _vp]),
    "nacu_graph_destroy": (_i, [_vp]),
    "nacu_dgetrf_batched": (_i, [_i, _vp, _i64, _vp, _vp, _i, _i, _vp]),
    "nacu_dgetrs_batched": (_i, [_i, _i, _vp, _i64, _vp, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_dgesv_batched": (_i, [_i, _i, _vp, _i64, _vp, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_sgesv_batched": (_i, [_i, _i, _vp, _i64, _vp, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_ragged_workspace_bytes": (_sz, [_i]),
    "nacu_dposv_ragged": (_i, [_i, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _d, _i, _vp]),
    "nacu_dpotrf_ragged": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _d, _i, _vp]),
    "nacu_dpotrs_ragged": (_i, [_i, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _sz, _i, _vp]),
    "nacu_dgetri_batched": (_i, [_i, _vp, _i64, _vp, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_dfullpivlu_batched": (_i, [_i, _i, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_dfullpivlu_solve_batched": (_i, [_i, _i, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_dcolpivqr_batched": (_i, [_i, _i, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_dcolpivqr_solve_batched": (_i, [_i, _i, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_dqr_batched": (_i, [_i, _i, _vp, _i64, _vp, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_trsv_workspace_bytes": (_sz, [_i]),
    "nacu_dtrsv": (_i, [_i, _i, _i, _i, _i, _d, _vp, _i64, _vp, _i64, _vp, _vp, _sz, _i, _vp]),
    "nacu_dqr_solve_batched": (_i, [_i, _i, _vp, _i64, _vp, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_dqr": (_i, [_i, _i, _vp, _i64, _vp, _i, _vp]),
    "nacu_qr_solve_workspace_bytes": (_sz, [_i]),
    "nacu_dqr_solve": (_i, [_i, _i, _i, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _sz, _i, _vp]),
    "nacu_dtrsv_batched": (_i, [_i, _i, _i, _i, _i, _d, _vp, _i64, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_dchol_rank1_update_batched": (_i, [_i, _vp, _i64, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_dchol_remove_column_batched": (_i, [_i, _vp, _i64, _i, _vp, _i64, _i, _i, _vp]),
    "nacu_dchol_insert_column_batched": (_i, [_i, _vp, _i64, _i, _vp, _i64, _vp, _i64, _vp, _i, _i, _vp]),
    "nacu_dposv": (_i, [_i, _vp, _i, _vp, _vp, _vp, _d, _i, _vp]),
    "nacu_dposv_ragged_noalloc": (_i, [_i, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _d, _i, _vp]),
    "nacu_mixed_workspace_bytes": (_sz, [_i, _i64]),
    "nacu_dposv_ragged_mixed": (_i, [_i, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _vp, _sz, _d, _i,
                                     _d, _i, _vp]),
    "nacu_mixed_host_workspace_bytes": (_sz, [_i, _i, _vp, _vp, _vp, _i, _i]),
    "nacu_dposv_ragged_mixed_host": (_i, [_i, _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _i, _vp, _sz, _d, _i,
                                          _d, _i, _vp]),
    "nacu_dposv_logdet_forward": (_i, [_i, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
    "nacu_sposv_logdet_forward": (_i, [_i, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
    "nacu_dposv_logdet_backward": (_i, [_i, _vp, _i64, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
    "nacu_sposv_logdet_backward": (_i, [_i, _vp, _i64, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
    "nacu_qr_workspace_bytes": (_sz, [_i]),
    "nacu_dgels_batched": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _i, _vp]),
    "nacu_getrf_workspace_bytes": (_sz, [_i]),
    "nacu_dgetrf": (_i, [_i, _vp, _i64, _vp, _vp, _vp, _sz, _vp]),
    "nacu_dgetrs": (_i, [_i, _vp, _i64, _vp, _vp, _vp, _vp, _sz, _vp]),
    "nacu_test_dgetrs_flag_timeout": (_i, [_i, _vp, _i64, _vp, _vp, _vp, _i, _i, _vp, _sz, _vp]),
    "nacu_test_rcp": (_i, [_i, _vp, _vp, _vp]),
    "nacu_ragged_tuning_layout": (_i, [_vp, _vp, _vp]),
    "nacu_ragged_set_tuning": (_i, [_vp, _i]),
    "nacu_ragged_get_tuning": (_i, [_vp, _i]),
    "nacu_ragged_autotune": (_i, [_i, _i, _i, _vp, _vp, _vp]),
    "nacu_gesv_mixed_workspace_bytes": (_sz, [_i]),
    "nacu_dgesv_mixed_ir": (_i, [_i, _vp, _i64, _vp, _vp, _d, _i, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                 C.POINTER(C.c_int), _vp, _sz, _vp]),
    "nacu_dgemm": (_i, [_i, _i, _i, _d, _vp, _i64, _vp, _i64, _d, _vp, _i64, _vp]),
    "nacu_dgemm_batched": (_i, [_i, _i, _i, _d, _vp, _i64, _i64, _vp, _i64, _i64, _d, _vp, _i64, _i64, _i, _i, _vp]),
    "nacu_gemm_split_workspace_bytes": (_sz, [_i, _i, _i]),
    "nacu_dgemm_split_bf16": (_i, [_i, _i, _i, _d, _vp, _i64, _vp, _i64, _d, _vp, _i64, _i, _vp, _sz, _vp]),
    "nacu_split_gemm_error": (_i, [C.POINTER(C.c_int)]),
    "nacu_probe_fp64_peak": (_i, [C.POINTER(C.c_double)]),
}

_lib = None


class NacuError(RuntimeError):
    pass


def header_symbols() -> list[str]:
    """Every function name declared in include/nalgebra_cuda.h."""
    text = open(HEADER_PATH).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nacu_[a-z0-9_]+)\s*\(", text)))


def load(path: str | None = None):
    """Load the library (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise NacuError(
            f"{p} is missing: build it with `python -m nalgebra_gb300.build` "
            "(nalgebra_gb300 has no CPU fallback)")
    L = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = L
        from . import tuning

        tuning.apply(L)  # the measured per-bucket tiles, when a table was saved
    return L


def check(rc: int, what: str) -> None:
    if rc != NACU_SUCCESS:
        msg = load().nacu_last_error().decode(errors="replace")
        raise NacuError(f"{what} failed with code {rc}: {msg}")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)
