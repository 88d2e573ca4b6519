"""TEST INFRASTRUCTURE ONLY: the CPU oracle for the nalgebra dense-linalg path.

A ctypes front end over ``liboracle.so``, the C++ restatement of nalgebra's
LU / Cholesky / Householder-QR loops (``nalgebra_ref.hpp``), plus accurate FP64
metrics (compensated Dot2 GEMM, backward error, LU reconstruction error).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may use this module, and only as the checker or the CPU baseline.
The product (``nalgebra_gb300`` and ``libnalgebra_cuda.so``) never imports it.

All matrices are column-major (Fortran order) float64 numpy arrays, the layout
of nalgebra's ``VecStorage`` (src/base/vec_storage.rs:28-32).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

_i64 = C.c_int64
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)


def build() -> str:
    """Compile liboracle.so with the committed Makefile (g++, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(
            os.path.getmtime(os.path.join(_HERE, f)) for f in ("nalgebra_ref.cpp", "nalgebra_ref.hpp")
        ):
            build()
        L = C.CDLL(_LIB_PATH)
        sig = {
            "orc_max_threads": (C.c_int, []),
            "orc_ddot": (C.c_double, [_i64, _dp, _dp]),
            "orc_dgetrf": (_i64, [_i64, _i64, _dp, _i64, _i32p]),
            "orc_sgetrf": (_i64, [_i64, _i64, _fp, _i64, _i32p]),
            "orc_dgetrs": (C.c_int, [_i64, _dp, _i64, _i32p, _dp, _i64, _i64]),
            "orc_dlu_determinant": (C.c_double, [_i64, _dp, _i64, _i64]),
            "orc_dfullpivlu": (_i64, [_i64, _i64, _dp, _i64, _i32p, _i32p]),
            "orc_dcolpivqr": (None, [_i64, _i64, _dp, _i64, _dp, _i32p]),
            "orc_dcolpivqr_solve": (C.c_int, [_i64, _dp, _i64, _dp, _i32p, _dp, _i64, _i64]),
            "orc_dfullpivlu_solve": (C.c_int, [_i64, _dp, _i64, _i32p, _i32p, _dp, _i64, _i64]),
            "orc_dtrsv": (C.c_int, [_i64, _dp, _i64, _dp, _i64, _i64, C.c_int, C.c_int, C.c_int, C.c_double]),
            "orc_dchol_rank1": (None, [_i64, _dp, _i64, _dp, C.c_double]),
            "orc_dchol_remove_column": (None, [_i64, _dp, _i64, _i64, _dp, _i64]),
            "orc_dchol_insert_column": (C.c_int, [_i64, _dp, _i64, _i64, _dp, _dp, _i64]),
            "orc_dpotrf": (C.c_int, [_i64, _dp, _i64, C.c_int, C.c_double]),
            "orc_spotrf": (C.c_int, [_i64, _fp, _i64, C.c_int, C.c_float]),
            "orc_dpotrs": (None, [_i64, _dp, _i64, _dp, _i64, _i64]),
            "orc_dpotrf_ln_det": (C.c_double, [_i64, _dp, _i64]),
            "orc_dgeqrf": (None, [_i64, _i64, _dp, _i64, _dp]),
            "orc_dqr_q_tr_mul": (None, [_i64, _i64, _dp, _i64, _dp, _dp, _i64, _i64]),
            "orc_dqr_ls_solve": (C.c_int, [_i64, _i64, _dp, _i64, _dp, _dp, _i64, _dp, _i64, _i64]),
            "orc_dqr_solve": (C.c_int, [_i64, _dp, _i64, _dp, _dp, _i64, _i64]),
            "orc_dgesv_batched": (None, [_i64, _i64, _dp, _i32p, _dp, _i64, _i32p, C.c_int]),
            "orc_dposv_ragged": (None, [_i64, _i32p, _i64p, _dp, _i64p, _dp, _i64, _i32p, _dp, C.c_int]),
            "orc_dgels_batched": (None, [_i64, _i32p, _i64, _i64p, _dp, _i64p, _dp, _dp, _dp, _i32p, C.c_int]),
            "orc_dgemm_dot2": (None, [_i64, _i64, _i64, C.c_double, _dp, _i64, _dp, _i64, C.c_double, _dp, _i64, C.c_int]),
            "orc_dgemm_gemv_order_batched": (None, [_i64, _i64, _i64, C.c_double, _dp, _i64, _i64, _dp, _i64, _i64,
                                                    C.c_double, _dp, _i64, _i64, _i64, C.c_int]),
            "orc_dbackward_error": (C.c_double, [_i64, _dp, _i64, _dp, _i64, _dp, _i64, _i64]),
            "orc_dlu_reconstruction": (C.c_double, [_i64, _dp, _i64, _dp, _i64, _i32p]),
            "orc_dposv_ragged_backward_errors": (None, [_i64, _i32p, _i64p, _dp, _i64p, _dp, _dp, _i64, C.c_int,
                                                        _dp, C.c_int]),
            "orc_dgesv_backward_error": (C.c_double, [_i64, _dp, _i64, _dp, _dp, C.c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a, ty=_dp):
    return a.ctypes.data_as(ty)


def _f64(a):
    return np.asfortranarray(a, dtype=np.float64)


def max_threads() -> int:
    return lib().orc_max_threads()


# ---- single-matrix restatements ----------------------------------------------

def dot(x, y) -> float:
    """Matrix::dotx, 8 accumulators (src/base/blas.rs:96-165)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    return lib().orc_ddot(x.size, _p(x), _p(y))


def lu(a, dtype=np.float64):
    """LU::new (src/linalg/lu.rs:93-122).

    Returns (packed L\\U, ipiv, len): ipiv[i] is the row swapped with row i at
    step i (i when none); len is PermutationSequence::len.
    """
    a = np.array(a, dtype=dtype, order="F", copy=True)
    m, n = a.shape
    ipiv = np.zeros(min(m, n), dtype=np.int32)
    if dtype == np.float32:
        ln = lib().orc_sgetrf(m, n, _p(a, _fp), max(m, 1), _p(ipiv, _i32p))
    else:
        ln = lib().orc_dgetrf(m, n, _p(a), max(m, 1), _p(ipiv, _i32p))
    return a, ipiv, int(ln)


def lu_solve(lu_, ipiv, b):
    """LU::solve (src/linalg/lu.rs:221-260).  Returns x, or None if singular."""
    lu_ = _f64(lu_)
    n = lu_.shape[0]
    x = np.array(b, dtype=np.float64, order="F", copy=True)
    x2 = x.reshape(n, -1, order="F")
    ok = lib().orc_dgetrs(n, _p(lu_), max(n, 1), _p(np.ascontiguousarray(ipiv, dtype=np.int32), _i32p),
                          _p(x2), max(n, 1), x2.shape[1])
    return x if ok else None


def full_piv_lu(a):
    """FullPivLU::new (src/linalg/full_piv_lu.rs:56-91).

    Returns (packed L\\U, ipiv, jpiv, steps): ipiv[i] / jpiv[i] are the row /
    column swapped with i at step i (i when none); steps < min(m, n) when the
    remaining submatrix was zero (nalgebra's `break`).
    """
    a = np.array(a, dtype=np.float64, order="F", copy=True)
    m, n = a.shape
    ipiv = np.zeros(min(m, n), dtype=np.int32)
    jpiv = np.zeros(min(m, n), dtype=np.int32)
    steps = lib().orc_dfullpivlu(m, n, _p(a), max(m, 1), _p(ipiv, _i32p), _p(jpiv, _i32p))
    return a, ipiv, jpiv, int(steps)


def full_piv_lu_solve(lu_, ipiv, jpiv, b):
    """FullPivLU::solve (src/linalg/full_piv_lu.rs:168-211).  Returns x, or None
    when lu[n-1][n-1] == 0 (is_invertible, :242-250)."""
    lu_ = _f64(lu_)
    n = lu_.shape[0]
    x = np.array(b, dtype=np.float64, order="F", copy=True)
    x2 = x.reshape(n, -1, order="F")
    ok = lib().orc_dfullpivlu_solve(n, _p(lu_), max(n, 1), _p(np.ascontiguousarray(ipiv, dtype=np.int32), _i32p),
                                    _p(np.ascontiguousarray(jpiv, dtype=np.int32), _i32p), _p(x2), max(n, 1),
                                    x2.shape[1])
    return x if ok else None


def full_piv_lu_determinant(lu_, ipiv, jpiv):
    """FullPivLU::determinant (src/linalg/full_piv_lu.rs:254-267): U[n-1][n-1]
    times the other diagonal entries in order, times the signs of p and q."""
    n = lu_.shape[0]
    res = float(lu_[n - 1, n - 1])
    if res == 0.0:
        return 0.0
    for i in range(n - 1):
        res *= float(lu_[i, i])
    swaps = int(np.sum(np.asarray(ipiv) != np.arange(n))) + int(np.sum(np.asarray(jpiv) != np.arange(n)))
    return res * (-1.0 if swaps % 2 else 1.0)


def col_piv_qr(a):
    """ColPivQR::new (src/linalg/col_piv_qr.rs:59-92).  Returns (packed factor:
    reflector axes at and below the diagonal, R above it; diag; jpiv)."""
    a = np.array(a, dtype=np.float64, order="F", copy=True)
    m, n = a.shape
    diag = np.zeros(min(m, n))
    jpiv = np.zeros(min(m, n), dtype=np.int32)
    lib().orc_dcolpivqr(m, n, _p(a), max(m, 1), _p(diag), _p(jpiv, _i32p))
    return a, diag, jpiv


def col_piv_qr_solve(qr_, diag, jpiv, b):
    """ColPivQR::solve_mut (col_piv_qr.rs:227-247) on a copy of b.  Returns
    (x, solved): nalgebra overwrites b even when it returns false."""
    qr_ = _f64(qr_)
    n = qr_.shape[0]
    x = np.array(b, dtype=np.float64, order="F", copy=True)
    x2 = x.reshape(n, -1, order="F")
    ok = lib().orc_dcolpivqr_solve(n, _p(qr_), max(n, 1), _p(np.ascontiguousarray(diag, dtype=np.float64)),
                                   _p(np.ascontiguousarray(jpiv, dtype=np.int32), _i32p), _p(x2), max(n, 1),
                                   x2.shape[1])
    return x, bool(ok)


def col_piv_qr_q_r(qr_, diag):
    """(Q, R) of ColPivQR::unpack (col_piv_qr.rs:97-173): Q from q_tr_mul on the
    identity, R the upper triangle with |diag| on its diagonal."""
    qr_ = _f64(qr_)
    m, n = qr_.shape
    qt = np.asfortranarray(np.eye(m))
    lib().orc_dqr_q_tr_mul(m, n, _p(qr_), max(m, 1), _p(np.ascontiguousarray(diag, dtype=np.float64)), _p(qt),
                           max(m, 1), m)
    r = np.triu(qr_[: min(m, n), :])
    r[np.arange(len(diag)), np.arange(len(diag))] = np.abs(diag)
    return qt.T[:, : min(m, n)], r


def cholesky_rank_one_update(l, x, sigma):
    """Cholesky::rank_one_update (src/linalg/cholesky.rs:277-285, 410-449) on a
    copy of the factor l (n x n, lower part used); returns the new factor."""
    out = np.array(l, dtype=np.float64, order="F", copy=True)
    xv = np.array(x, dtype=np.float64, copy=True)
    n = out.shape[0]
    lib().orc_dchol_rank1(n, _p(out), max(n, 1), _p(xv), float(sigma))
    return out


def cholesky_remove_column(l, j):
    """Cholesky::remove_column (src/linalg/cholesky.rs:365-399)."""
    l = _f64(l)
    n = l.shape[0]
    out = np.zeros((n - 1, n - 1), order="F")
    lib().orc_dchol_remove_column(n, _p(l), max(n, 1), j, _p(out), max(n - 1, 1))
    return out


def cholesky_insert_column(l, j, col):
    """Cholesky::insert_column (src/linalg/cholesky.rs:287-357); None when
    nalgebra's lower solve assertion would fail."""
    l = _f64(l)
    n = l.shape[0]
    out = np.zeros((n + 1, n + 1), order="F")
    c = np.ascontiguousarray(col, dtype=np.float64)
    ok = lib().orc_dchol_insert_column(n, _p(l), max(n, 1), j, _p(c), _p(out), n + 1)
    return out if ok else None


def triangular_solve(t, b, upper=False, trans=False, diag=None):
    """Matrix::{solve,tr_solve}_{lower,upper}_triangular_mut and
    solve_lower_triangular_with_diag_mut (src/linalg/solve.rs:55-442) on a copy
    of b; returns x, or None at a zero diagonal (nalgebra's false)."""
    t = _f64(t)
    n = t.shape[0]
    x = np.array(b, dtype=np.float64, order="F", copy=True)
    x2 = x.reshape(n, -1, order="F")
    ok = lib().orc_dtrsv(n, _p(t), max(n, 1), _p(x2), max(n, 1), x2.shape[1], int(upper), int(trans),
                         int(diag is not None), float(diag if diag is not None else 0.0))
    return x if ok else None


def lu_try_inverse(lu_, ipiv):
    """LU::try_inverse (src/linalg/lu.rs:266-297): the identity, then
    LU::solve_mut on it (lu.rs:242-260); None when some U_ii == 0."""
    n = np.asarray(lu_).shape[0]
    return lu_solve(lu_, ipiv, np.eye(n))


def lu_determinant(lu_, length) -> float:
    lu_ = _f64(lu_)
    return lib().orc_dlu_determinant(lu_.shape[0], _p(lu_), max(lu_.shape[0], 1), length)


def cholesky(a, substitute=None, dtype=np.float64):
    """Cholesky::new / new_with_substitute (src/linalg/cholesky.rs:196-272).

    Returns (factor with dirty upper triangle, info); info 0 = ok, j+1 = the
    first failing pivot column (nalgebra returns None).
    """
    a = np.array(a, dtype=dtype, order="F", copy=True)
    n = a.shape[0]
    hs = 0 if substitute is None else 1
    sv = 0.0 if substitute is None else float(substitute)
    if dtype == np.float32:
        info = lib().orc_spotrf(n, _p(a, _fp), max(n, 1), hs, sv)
    else:
        info = lib().orc_dpotrf(n, _p(a), max(n, 1), hs, sv)
    return a, int(info)


def cholesky_solve(l, b):
    """Cholesky::solve (src/linalg/cholesky.rs:122-143)."""
    l = _f64(l)
    n = l.shape[0]
    x = np.array(b, dtype=np.float64, order="F", copy=True)
    x2 = x.reshape(n, -1, order="F")
    lib().orc_dpotrs(n, _p(l), max(n, 1), _p(x2), max(n, 1), x2.shape[1])
    return x


def cholesky_ln_determinant(l) -> float:
    l = _f64(l)
    return lib().orc_dpotrf_ln_det(l.shape[0], _p(l), max(l.shape[0], 1))


def qr(a):
    """QR::new (src/linalg/qr.rs:55-76): (packed axes + R, signed diag)."""
    a = np.array(a, dtype=np.float64, order="F", copy=True)
    m, n = a.shape
    diag = np.zeros(min(m, n), dtype=np.float64)
    lib().orc_dgeqrf(m, n, _p(a), max(m, 1), _p(diag))
    return a, diag


def qr_q_tr_mul(qr_, diag, b):
    qr_ = _f64(qr_)
    m, n = qr_.shape
    x = np.array(b, dtype=np.float64, order="F", copy=True)
    x2 = x.reshape(m, -1, order="F")
    lib().orc_dqr_q_tr_mul(m, n, _p(qr_), max(m, 1), _p(np.ascontiguousarray(diag, dtype=np.float64)),
                           _p(x2), max(m, 1), x2.shape[1])
    return x


def qr_solve(qr_, diag, b):
    """QR::solve_mut (src/linalg/qr.rs:204-256) on a copy of b.  Returns
    (x, solved): nalgebra overwrites b even when it returns false."""
    qr_ = _f64(qr_)
    n = qr_.shape[0]
    x = np.array(b, dtype=np.float64, order="F", copy=True)
    x2 = x.reshape(n, -1, order="F")
    ok = lib().orc_dqr_solve(n, _p(qr_), max(n, 1), _p(np.ascontiguousarray(diag, dtype=np.float64)), _p(x2),
                             max(n, 1), x2.shape[1])
    return x, bool(ok)


def qr_r(qr_, diag):
    """QR::r (src/linalg/qr.rs:81-89): upper triangle with |diag| on the diagonal."""
    qr_ = np.asarray(qr_)
    m, n = qr_.shape
    k = min(m, n)
    r = np.triu(qr_[:k, :]).copy()
    r[np.arange(k), np.arange(k)] = np.abs(diag)
    return r


def qr_ls_solve(qr_, diag, b):
    """Least squares from the QR factors: (x, info)."""
    qr_ = _f64(qr_)
    m, n = qr_.shape
    bb = np.array(b, dtype=np.float64, order="F", copy=True).reshape(m, -1, order="F")
    x = np.zeros((n, bb.shape[1]), dtype=np.float64, order="F")
    info = lib().orc_dqr_ls_solve(m, n, _p(qr_), max(m, 1), _p(np.ascontiguousarray(diag, dtype=np.float64)),
                                  _p(bb), max(m, 1), _p(x), max(n, 1), bb.shape[1])
    return x, int(info)


# ---- batched drivers (CPU baseline) ------------------------------------------

def gesv_batched(a, b, n, nthreads=0):
    """a: (batch, n*n), row s the column-major image of system s; b: (batch,
    n*nrhs) likewise.  Returns (lu, ipiv, x, info); inputs are not modified."""
    a = np.array(a, dtype=np.float64, copy=True, order="C")
    b = np.array(b, dtype=np.float64, copy=True, order="C")
    batch = a.shape[0]
    nrhs = b.shape[1] // n
    ipiv = np.zeros((batch, n), dtype=np.int32)
    info = np.zeros(batch, dtype=np.int32)
    lib().orc_dgesv_batched(batch, n, _p(a), _p(ipiv, _i32p), _p(b), nrhs, _p(info, _i32p), nthreads)
    return a, ipiv, b, info


def posv_ragged(ns, aoff, a_flat, boff, b_flat, nrhs, nthreads=0):
    """Ragged Cholesky + solve + ln_determinant over packed column-major blocks.
    Returns (factors_flat, x_flat, info, logdet); inputs are copied."""
    a = np.array(a_flat, dtype=np.float64, copy=True)
    b = np.array(b_flat, dtype=np.float64, copy=True)
    ns = np.ascontiguousarray(ns, dtype=np.int32)
    aoff = np.ascontiguousarray(aoff, dtype=np.int64)
    boff = np.ascontiguousarray(boff, dtype=np.int64)
    count = ns.size
    info = np.zeros(count, dtype=np.int32)
    logdet = np.zeros(count, dtype=np.float64)
    lib().orc_dposv_ragged(count, _p(ns, _i32p), _p(aoff, _i64p), _p(a), _p(boff, _i64p), _p(b), nrhs,
                           _p(info, _i32p), _p(logdet), nthreads)
    return a, b, info, logdet


def gels_batched(ms, n, aoff, a_flat, boff, b_flat, nthreads=0):
    """Batched QR least squares (one RHS each).  Returns (qr_flat, diag, x, info)."""
    a = np.array(a_flat, dtype=np.float64, copy=True)
    b = np.array(b_flat, dtype=np.float64, copy=True)
    ms = np.ascontiguousarray(ms, dtype=np.int32)
    aoff = np.ascontiguousarray(aoff, dtype=np.int64)
    boff = np.ascontiguousarray(boff, dtype=np.int64)
    count = ms.size
    diag = np.zeros(count * n, dtype=np.float64)
    x = np.zeros(count * n, dtype=np.float64)
    info = np.zeros(count, dtype=np.int32)
    lib().orc_dgels_batched(count, _p(ms, _i32p), n, _p(aoff, _i64p), _p(a), _p(boff, _i64p), _p(b),
                            _p(diag), _p(x), _p(info, _i32p), nthreads)
    return a, diag.reshape(count, n), x.reshape(count, n), info


# ---- accurate metrics ----------------------------------------------------------

def gemm_dot2(alpha, a, b, beta=0.0, c=None, nthreads=0):
    """alpha*A*B + beta*C with compensated (Dot2) accumulation."""
    a = _f64(a)
    b = _f64(b)
    m, k = a.shape
    n = b.shape[1]
    out = np.zeros((m, n), dtype=np.float64, order="F") if c is None else np.array(c, dtype=np.float64, order="F", copy=True)
    lib().orc_dgemm_dot2(m, n, k, alpha, _p(a), max(m, 1), _p(b), max(k, 1), beta, _p(out), max(m, 1), nthreads)
    return out


def gemm_gemv_order(alpha, a, b, beta=0.0, c=None, nthreads=0):
    """alpha*A*B + beta*C in nalgebra's gemv order (gemm_uninit's path for a
    dimension <= 5 or static sizes, blas_uninit.rs:187-333).  a: (m, k), b:
    (k, n), or batches (batch, m, k) / (batch, k, n); returns the product(s)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    single = a.ndim == 2
    if single:
        a, b = a[None], b[None]
        c = None if c is None else np.asarray(c, dtype=np.float64)[None]
    batch, m, k = a.shape
    n = b.shape[2]
    af = np.ascontiguousarray(np.transpose(a, (0, 2, 1)))  # column-major per product
    bf = np.ascontiguousarray(np.transpose(b, (0, 2, 1)))
    cf = (np.zeros((batch, n, m)) if c is None
          else np.array(np.transpose(np.asarray(c, dtype=np.float64), (0, 2, 1)), order="C", copy=True))
    lib().orc_dgemm_gemv_order_batched(m, n, k, alpha, _p(af), max(m, 1), m * k, _p(bf), max(k, 1), k * n, beta,
                                       _p(cf), max(m, 1), m * n, batch, nthreads)
    out = np.transpose(cf, (0, 2, 1))
    return out[0] if single else out


def backward_error(a, x, b) -> float:
    """max over RHS of ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)."""
    a = _f64(a)
    n = a.shape[0]
    x = _f64(x).reshape(n, -1, order="F")
    b = _f64(b).reshape(n, -1, order="F")
    return lib().orc_dbackward_error(n, _p(a), max(n, 1), _p(x), max(n, 1), _p(b), max(n, 1), x.shape[1])


def lu_reconstruction(a, lu_, ipiv) -> float:
    """||P A - L U||_F / (||A||_F n eps64)."""
    a = _f64(a)
    lu_ = _f64(lu_)
    n = a.shape[0]
    return lib().orc_dlu_reconstruction(n, _p(a), max(n, 1), _p(lu_), max(n, 1),
                                        _p(np.ascontiguousarray(ipiv, dtype=np.int32), _i32p))


def ragged_backward_errors(ns, aoff, a_flat, boff, b_flat, x_flat, nrhs, symmetric=True, nthreads=0) -> np.ndarray:
    """Per-system normwise backward error of a ragged batch of solves, max
    over the right-hand sides, residuals by Dot2 (all host threads).  A is the
    symmetric matrix of its lower triangle when ``symmetric`` (the SPD
    solves), else the full stored matrix."""
    ns = np.ascontiguousarray(ns, dtype=np.int32)
    aoff = np.ascontiguousarray(aoff, dtype=np.int64)
    boff = np.ascontiguousarray(boff, dtype=np.int64)
    a_flat = np.ascontiguousarray(a_flat, dtype=np.float64)
    b_flat = np.ascontiguousarray(b_flat, dtype=np.float64)
    x_flat = np.ascontiguousarray(x_flat, dtype=np.float64)
    out = np.zeros(ns.size, dtype=np.float64)
    lib().orc_dposv_ragged_backward_errors(ns.size, _p(ns, _i32p), _p(aoff, _i64p), _p(a_flat), _p(boff, _i64p),
                                           _p(b_flat), _p(x_flat), int(nrhs), int(bool(symmetric)), _p(out),
                                           nthreads)
    return out


def dense_backward_error(a_colmajor_flat, n, x, b, nthreads=0) -> float:
    """Normwise backward error of one dense n x n system (A column-major,
    one right-hand side), residual by Dot2 over all host threads."""
    a = np.ascontiguousarray(a_colmajor_flat, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return lib().orc_dgesv_backward_error(int(n), _p(a), int(n), _p(x), _p(b), nthreads)
