"""The C-ABI library without a GPU: it builds for sm_103a, loads, exports every
symbol include/nalgebra_cuda.h declares, and rejects bad arguments with the
LAPACK-style negative codes before touching the device."""
import ctypes as C

import pytest

from nalgebra_gb300 import _lib, build


@pytest.fixture(scope="module")
def L():
    build.build()
    return _lib.load()


def test_exports_every_header_symbol(L):
    names = _lib.header_symbols()
    assert len(names) >= 10
    raw = C.CDLL(_lib.LIB_PATH)
    missing = [n for n in names if not hasattr(raw, n)]
    assert not missing, missing
    # and every declared symbol has a ctypes signature in the host binding
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_version_and_arch(L):
    assert L.nacu_version() == b"0.1.0"
    assert L.nacu_device_arch() == 103


def test_lu_argument_errors(L):
    assert L.nacu_dgesv_batched(-1, 1, 0, 0, 0, 0, 0, 0, 1, 0, 0) == -1
    assert L.nacu_dgesv_batched(129, 1, 0, 0, 0, 0, 0, 0, 1, 0, 0) == -1
    assert L.nacu_dgesv_batched(8, 17, 0, 0, 0, 0, 0, 0, 1, 0, 0) == -2
    assert b"nrhs" in L.nacu_last_error()
    assert L.nacu_dgesv_batched(8, 1, 0, 64, 0, 0, 8, 0, -1, 0, 0) == -9
    # empty work is a no-op success, no device needed
    assert L.nacu_dgesv_batched(8, 1, 0, 64, 0, 0, 8, 0, 0, 0, 0) == 0
    assert L.nacu_dgesv_batched(0, 1, 0, 0, 0, 0, 0, 0, 5, 0, 0) == 0
    # null pointers with real work
    assert L.nacu_dgesv_batched(8, 1, 0, 64, 0, 0, 8, 0, 2, 0, 0) == -3
    # stride too small
    assert L.nacu_dgesv_batched(8, 1, 1024, 10, 1024, 1024, 8, 0, 2, 0, 0) == -4


def test_cholesky_argument_errors(L):
    ws = L.nacu_ragged_workspace_bytes(10)
    assert ws >= 4
    assert L.nacu_dposv_ragged(-1, 8, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0.0, 0, 0) == -1
    assert L.nacu_dposv_ragged(3, 513, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0.0, 0, 0) == -2
    assert L.nacu_dposv_ragged(0, 8, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0.0, 0, 0) == 0
    assert L.nacu_dposv_ragged(3, 8, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0.0, 0, 0) == -3
    # workspace too small
    assert L.nacu_dposv_ragged(3, 8, 16, 16, 16, 1, 16, 16, 16, 0, 0, 16, 0, 0.0, 0, 0) == -12
    assert L.nacu_dposv(-2, 0, 0, 0, 0, 0, 0.0, 0, 0) == -1
    assert L.nacu_dposv(4, 0, 0, 0, 0, 0, 0.0, 0, 0) == -2


def test_large_qr_argument_errors(L):
    assert L.nacu_dqr(-1, 4, None, 4, None, 0, None) == -1
    assert L.nacu_dqr(4, -1, None, 4, None, 0, None) == -2
    assert L.nacu_dqr(0, 9, None, 1, None, 0, None) == 0  # empty: no work, no device needed
    assert L.nacu_dqr(5, 5, None, 5, None, 0, None) == -3
    assert L.nacu_dqr(5, 5, 1024, 4, 1024, 0, None) == -4
    assert L.nacu_dqr(5, 5, 1024, 5, None, 0, None) == -5
    assert L.nacu_qr_solve_workspace_bytes(0) == 0 and L.nacu_qr_solve_workspace_bytes(100) >= 100 * 100 * 8
    assert L.nacu_dqr_solve(16385, 4, 1, None, 1, None, None, 1, None, None, 0, 0, None) == -1
    assert L.nacu_dqr_solve(4, 5, 1, None, 4, None, None, 4, None, None, 0, 0, None) == -2
    assert L.nacu_dqr_solve(4, 4, -1, None, 4, None, None, 4, None, None, 0, 0, None) == -3
    assert L.nacu_dqr_solve(4, 4, 1, None, 4, None, None, 4, None, None, 0, 0, None) == -9
    assert L.nacu_dqr_solve(4, 4, 1, None, 4, None, None, 4, 1024, None, 0, 1, None) == -12  # EXACT
    assert L.nacu_dqr_solve(4, 4, 1, 1024, 4, 1024, 1024, 4, 1024, 1024, 8, 0, None) == -11


def test_product_has_no_cpu_fallback(tmp_path):
    with pytest.raises(_lib.NacuError):
        _lib.load(str(tmp_path / "missing.so"))


def test_product_never_imports_the_oracle():
    import os
    import re

    pkg = os.path.dirname(_lib.__file__)
    for root, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                text = open(os.path.join(root, f)).read()
                assert not re.search(r"^\s*(import|from)\s+oracle\b", text, re.M), f
                assert "liboracle" not in text, f


def test_rust_crate_binds_every_entry_point_with_its_arity():
    """nalgebra-cuda/src/ffi.rs (the crate is source here: no Rust toolchain on
    these machines) declares every entry point of include/nalgebra_cuda.h with
    the header's number of parameters."""
    import os
    import re

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    hdr = open(os.path.join(root, "include", "nalgebra_cuda.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    decl = {}
    for m in re.finditer(r"\b(nacu_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", hdr):
        args = m.group(2).strip()
        decl[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    rs = open(os.path.join(root, "nalgebra-cuda", "src", "ffi.rs")).read()
    rs = re.sub(r"//[^\n]*", "", rs)
    bound = {}
    for m in re.finditer(r"pub fn (nacu_[a-z0-9_]+)\s*\(([^)]*)\)", rs):
        args = m.group(2).strip().rstrip(",")
        bound[m.group(1)] = 0 if not args else args.count(",") + 1
    assert set(decl) == set(bound), (set(decl) ^ set(bound))
    wrong = {k: (decl[k], bound[k]) for k in decl if decl[k] != bound[k]}
    assert not wrong, wrong


# Entry points whose first argument is an order or a count: a negative value
# is rejected with -1 (LAPACK's xerbla convention) before any device work, so
# these run without a GPU.
_FIRST_ARG_IS_SIZE = [
    "nacu_dgetrf_batched", "nacu_dgetrs_batched", "nacu_dgesv_batched", "nacu_sgesv_batched", "nacu_dgetri_batched",
    "nacu_dposv_ragged", "nacu_dpotrf_ragged", "nacu_dpotrs_ragged", "nacu_dposv", "nacu_dposv_ragged_noalloc",
    "nacu_dposv_ragged_mixed", "nacu_dposv_ragged_mixed_host", "nacu_dposv_logdet_forward",
    "nacu_sposv_logdet_forward", "nacu_dposv_logdet_backward", "nacu_sposv_logdet_backward",
    "nacu_dchol_rank1_update_batched", "nacu_dchol_remove_column_batched", "nacu_dchol_insert_column_batched",
    "nacu_dfullpivlu_batched", "nacu_dfullpivlu_solve_batched", "nacu_dcolpivqr_batched",
    "nacu_dcolpivqr_solve_batched", "nacu_dqr_batched", "nacu_dqr_solve_batched", "nacu_dqr", "nacu_dqr_solve",
    "nacu_dgels_batched", "nacu_dtrsv_batched", "nacu_dtrsv", "nacu_dgetrf", "nacu_dgetrs", "nacu_dgesv_mixed_ir",
    "nacu_dgemm", "nacu_dgemm_batched", "nacu_dgemm_split_bf16", "nacu_test_rcp", "nacu_test_dgetrs_flag_timeout",
]


@pytest.mark.parametrize("name", _FIRST_ARG_IS_SIZE)
def test_negative_size_is_argument_one(L, name):
    restype, argtypes = _lib.SIGNATURES[name]
    args = []
    for t in argtypes:
        if t in (C.c_int, C.c_int64, C.c_size_t):
            args.append(0)
        elif t is C.c_double:
            args.append(0.0)
        else:
            args.append(None)  # pointers and streams
    args[0] = -1
    assert getattr(L, name)(*args) == -1, name
    assert b"argument 1" in L.nacu_last_error(), name


def test_plumbing_null_outputs_are_rejected(L):
    assert L.nacu_device_count(None) == -1
    assert L.nacu_host_alloc(None, 8) == -1
    assert L.nacu_stream_create(None) == -1
    assert L.nacu_graph_end_capture(None, None) == -1
    assert L.nacu_probe_fp64_peak(None) == -1
    assert L.nacu_ragged_get_tuning(None, 0) == -1 and L.nacu_ragged_set_tuning(None, 0) == -1
