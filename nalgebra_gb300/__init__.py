"""nalgebra_gb300: host-side mirror of nalgebra's dense solve API over the
nalgebra-cuda C ABI (include/nalgebra_cuda.h, libnalgebra_cuda.so).

The method names follow nalgebra so that code written against
``DMatrix::lu() / .cholesky() / .qr() / .solve() / gemm(alpha, a, b, beta)``
reads the same here:

=================================  ==============================================
nalgebra (reference)                here
=================================  ==============================================
``m.lu()`` lu.rs:93-122            ``DeviceMatrix.lu()`` / ``DeviceBatch.lu()``
``lu.solve(&b)`` lu.rs:221-236     ``LU.solve(b)`` -> DeviceMatrix or None
``lu.solve_mut(&mut b)``           ``LU.solve_mut(b)`` -> bool
``lu.determinant()`` lu.rs:301     ``LU.determinant()``
``lu.p()``                         ``LU.p()`` -> [(i, piv), ...]
``m.cholesky()`` cholesky.rs:196   ``DeviceMatrix.cholesky()`` -> Cholesky or None
``chol.solve(&b)`` cholesky.rs:134 ``Cholesky.solve(b)``
``chol.ln_determinant()`` :172     ``Cholesky.ln_determinant()``
=================================  ==============================================

Device memory, copies, streams and CUDA graphs go through the library's own
plumbing entry points (``_device``: nacu_malloc, nacu_memcpy, nacu_graph_*),
so the mirror needs nothing but libnalgebra_cuda.so and numpy; device arrays
of other libraries plug in through ``__cuda_array_interface__``.  Every
numerical operation is a hand-written sm_103a kernel reached through the C
ABI.  There is no CPU fallback: without a GPU or without the built library,
calls raise.
Factorizations are lazy where that lets one launch do factor + solve: ``lu()``
and ``cholesky()`` on a batch record the request, and the first ``solve``
runs the fused kernel, writing the factors as a side effect.
"""
from __future__ import annotations

import numpy as np

from . import _device as _dev
from . import _lib
from . import factor_format
from ._device import DeviceBuffer, Graph, Stream, current_stream, pinned_empty, set_stream, stream, synchronize
from ._lib import FLAG_EXACT, FLAG_NO_FACTORS, FLAG_SUBSTITUTE, NacuError

__all__ = [
    "DeviceMatrix", "DeviceBatch", "LU", "LUBatch", "Cholesky", "CholeskyBatch", "QRBatch", "solve_refined", "gemm",
    "gemm_batched",
    "PosvLogdet", "cholesky_solve_refined_host",
    "NacuError", "FLAG_EXACT", "FLAG_NO_FACTORS", "FLAG_SUBSTITUTE", "FullPivLU", "ColPivQR", "QR",
    "DeviceBuffer", "Graph", "Stream", "current_stream", "set_stream", "stream", "synchronize", "pinned_empty",
]


def _stream_ptr() -> int:
    return _dev.current_stream()


def _dev_f64(x) -> DeviceBuffer:
    """A float64 device array as it is, or a host array copied to the device."""
    return _dev.as_device(x, np.float64)


def _i32(k: int) -> DeviceBuffer:
    return _dev.zeros(max(int(k), 1), np.int32)


def _f64(k: int) -> DeviceBuffer:
    return _dev.zeros(max(int(k), 1), np.float64)


def _bytes(k: int) -> DeviceBuffer:
    return _dev.empty(max(int(k), 1), np.uint8)


def _padded_i32(v, n: int) -> DeviceBuffer:
    return _dev.from_numpy(np.append(np.asarray(v).astype(np.int32), np.zeros(max(n, 1) - n, np.int32)))


def _padded_f64(v, n: int) -> DeviceBuffer:
    return _dev.from_numpy(np.append(np.asarray(v, dtype=np.float64), np.zeros(max(n, 1) - n)))


class DeviceMatrix:
    """An nrows x ncols f64 matrix resident on the GPU, column-major like
    nalgebra's DMatrix (src/base/vec_storage.rs:28-32).  ``data`` is a flat
    float64 device buffer of nrows*ncols elements (a DeviceBuffer; a device
    array of another library is wrapped without a copy, a host array is
    copied)."""

    def __init__(self, data, nrows: int, ncols: int):
        _dev.require_gpu()
        self.data = _dev_f64(data)
        if self.data.numel() != nrows * ncols:
            raise ValueError("data size does not match nrows * ncols")
        self.nrows, self.ncols = int(nrows), int(ncols)

    @classmethod
    def from_numpy(cls, a) -> "DeviceMatrix":
        a = np.asarray(a, dtype=np.float64)
        if a.ndim == 1:
            a = a.reshape(-1, 1)
        flat = np.asfortranarray(a).ravel(order="F")
        return cls(flat, a.shape[0], a.shape[1])

    def to_numpy(self) -> np.ndarray:
        return self.data.to_numpy().reshape(self.ncols, self.nrows).T.copy()

    @property
    def shape(self):
        return (self.nrows, self.ncols)

    def is_square(self) -> bool:
        return self.nrows == self.ncols

    def clone_owned(self) -> "DeviceMatrix":
        return DeviceMatrix(self.data.clone(), self.nrows, self.ncols)

    # -- factorizations (consume self: the buffer is factored in place) --------
    def _trsv(self, b: "DeviceMatrix", upper: bool, trans: bool, diag=None, flags: int = 0) -> bool:
        """nacu_dtrsv_batched on one matrix (n <= 128), nacu_dtrsv above: b is
        overwritten."""
        n = self.nrows
        assert self.is_square() and b.nrows == n, "triangular solve dimension mismatch"
        info = _i32(1)
        if n > 128:
            ws = _bytes(_lib.load().nacu_trsv_workspace_bytes(n))
            _lib.call("nacu_dtrsv", n, b.ncols, int(upper), int(trans), int(diag is not None),
                      float(diag if diag is not None else 0.0), self.data.data_ptr(), n, b.data.data_ptr(), n,
                      info.data_ptr(), ws.data_ptr(), ws.numel(), flags, _stream_ptr())
            return int(info.item()) == 0
        _lib.call("nacu_dtrsv_batched", n, b.ncols, int(upper), int(trans), int(diag is not None),
                  float(diag if diag is not None else 0.0), self.data.data_ptr(), n * n, b.data.data_ptr(),
                  n * b.ncols, info.data_ptr(), 1, flags, _stream_ptr())
        return int(info.item()) == 0

    def solve_lower_triangular_mut(self, b: "DeviceMatrix", flags: int = 0) -> bool:
        """Matrix::solve_lower_triangular_mut (src/linalg/solve.rs:55-101)."""
        return self._trsv(b, False, False, None, flags)

    def solve_upper_triangular_mut(self, b: "DeviceMatrix", flags: int = 0) -> bool:
        """Matrix::solve_upper_triangular_mut (src/linalg/solve.rs:137-181)."""
        return self._trsv(b, True, False, None, flags)

    def tr_solve_lower_triangular_mut(self, b: "DeviceMatrix", flags: int = 0) -> bool:
        """Matrix::tr_solve_lower_triangular_mut (src/linalg/solve.rs:233-256); ad_ is the same for f64."""
        return self._trsv(b, False, True, None, flags)

    def tr_solve_upper_triangular_mut(self, b: "DeviceMatrix", flags: int = 0) -> bool:
        """Matrix::tr_solve_upper_triangular_mut (src/linalg/solve.rs:258-283)."""
        return self._trsv(b, True, True, None, flags)

    def solve_lower_triangular_with_diag_mut(self, b: "DeviceMatrix", diag: float, flags: int = 0) -> bool:
        """Matrix::solve_lower_triangular_with_diag_mut (src/linalg/solve.rs:106-134)."""
        return self._trsv(b, False, False, float(diag), flags)

    def solve_lower_triangular(self, b: "DeviceMatrix", flags: int = 0):
        """Matrix::solve_lower_triangular (solve.rs:15-34): a new matrix, or None."""
        res = b.clone_owned()
        return res if self.solve_lower_triangular_mut(res, flags) else None

    def solve_upper_triangular(self, b: "DeviceMatrix", flags: int = 0):
        res = b.clone_owned()
        return res if self.solve_upper_triangular_mut(res, flags) else None

    def tr_solve_lower_triangular(self, b: "DeviceMatrix", flags: int = 0):
        res = b.clone_owned()
        return res if self.tr_solve_lower_triangular_mut(res, flags) else None

    def tr_solve_upper_triangular(self, b: "DeviceMatrix", flags: int = 0):
        res = b.clone_owned()
        return res if self.tr_solve_upper_triangular_mut(res, flags) else None

    ad_solve_lower_triangular = tr_solve_lower_triangular
    ad_solve_upper_triangular = tr_solve_upper_triangular
    ad_solve_lower_triangular_mut = tr_solve_lower_triangular_mut
    ad_solve_upper_triangular_mut = tr_solve_upper_triangular_mut

    def lu(self, flags: int = 0) -> "LU":
        """Matrix::lu (src/linalg/decomposition.rs:48-54).  flags apply to the
        batched kernel (n <= 128)."""
        if not self.is_square():
            raise NotImplementedError("rectangular LU is not on the GPU path")
        return LU(self, flags)

    def full_piv_lu(self, flags: int = 0) -> "FullPivLU":
        """Matrix::full_piv_lu (src/linalg/decomposition.rs:39-45): factors in
        place (n <= 128)."""
        return FullPivLU(self, flags)

    def qr(self, flags: int = 0) -> "QR":
        """Matrix::qr (src/linalg/decomposition.rs:56-62): factors in place,
        any shape.  Batches of tall least-squares systems go through
        DeviceBatch.qr."""
        return QR(self, flags)

    def col_piv_qr(self, flags: int = 0) -> "ColPivQR":
        """Matrix::col_piv_qr (src/linalg/decomposition.rs:65-75): factors in
        place (n <= 128)."""
        return ColPivQR(self, flags)

    def cholesky(self, flags: int = 0, substitute: float | None = None):
        """Matrix::cholesky (decomposition.rs:257-262): Cholesky or None."""
        assert self.is_square(), "The input matrix must be square."
        ch = Cholesky(self, flags, substitute)
        return ch if ch._ok() else None


class LU:
    """LU with partial pivoting of one square matrix, packed L\\U in the matrix
    buffer, per-step pivots on the device.  n <= 128: the shared-memory batched
    kernel (batch of one); larger n: the blocked multi-SM factorization."""

    def __init__(self, m: DeviceMatrix, flags: int = 0):
        self.lu = m
        n = m.nrows
        self.flags = flags
        self.ipiv = _i32(n)
        self.info = _i32(2)
        self.large = n > 128
        if self.large:
            self._ws = _bytes(_lib.load().nacu_getrf_workspace_bytes(n))
            _lib.call("nacu_dgetrf", n, m.data.data_ptr(), n, self.ipiv.data_ptr(), self.info.data_ptr(),
                      self._ws.data_ptr(), self._ws.numel(), _stream_ptr())
        else:
            _lib.call("nacu_dgetrf_batched", n, m.data.data_ptr(), n * n, self.ipiv.data_ptr(),
                      self.info.data_ptr(), 1, flags, _stream_ptr())

    def solve_mut(self, b: DeviceMatrix) -> bool:
        """LU::solve_mut (src/linalg/lu.rs:242-260)."""
        n = self.lu.nrows
        assert b.nrows == n, "LU solve matrix dimension mismatch."
        info = _i32(1)
        if self.large:
            ok = True
            for c in range(b.ncols):
                _lib.call("nacu_dgetrs", n, self.lu.data.data_ptr(), n, self.ipiv.data_ptr(),
                          b.data.data_ptr() + c * n * 8, info.data_ptr(), self._ws.data_ptr(), self._ws.numel(),
                          _stream_ptr())
                ok = ok and int(info.item()) == 0
            return ok
        _lib.call("nacu_dgetrs_batched", n, b.ncols, self.lu.data.data_ptr(), n * n, self.ipiv.data_ptr(),
                  b.data.data_ptr(), n * b.ncols, info.data_ptr(), 1, self.flags, _stream_ptr())
        return int(info.item()) == 0

    def solve(self, b: DeviceMatrix):
        """LU::solve (src/linalg/lu.rs:221-236): a new matrix, or None."""
        res = b.clone_owned()
        return res if self.solve_mut(res) else None

    def p(self):
        """The PermutationSequence as nalgebra stores it: (i, piv) swaps in order."""
        piv = self.ipiv.to_numpy()[: self.lu.nrows]
        return [(i, int(p)) for i, p in enumerate(piv) if p != i]

    def determinant(self) -> float:
        """LU::determinant (src/linalg/lu.rs:301-314)."""
        lu = self.lu.to_numpy()
        d = 1.0
        for i in range(self.lu.nrows):
            d *= lu[i, i]
        return d * (1.0 if len(self.p()) % 2 == 0 else -1.0)

    def is_invertible(self) -> bool:
        return int(self.info.item()) == 0

    def try_inverse(self):
        """LU::try_inverse (src/linalg/lu.rs:266-297): the inverse as a new
        DeviceMatrix, or None when some U_ii == 0 (n <= 128)."""
        n = self.lu.nrows
        if self.large:
            raise NotImplementedError("try_inverse: n <= 128 (the batched kernels)")
        out = DeviceMatrix(_dev.empty(n * n, np.float64), n, n)
        info = _i32(1)
        _lib.call("nacu_dgetri_batched", n, self.lu.data.data_ptr(), n * n, self.ipiv.data_ptr(), out.data.data_ptr(),
                  n * n, info.data_ptr(), 1, self.flags, _stream_ptr())
        return out if int(info.item()) == 0 else None

    def l(self) -> np.ndarray:
        lu = self.lu.to_numpy()
        return np.tril(lu, -1) + np.eye(lu.shape[0])

    def u(self) -> np.ndarray:
        return np.triu(self.lu.to_numpy())

    def to_json(self) -> str:
        """nalgebra's serde JSON form of LU (src/linalg/lu.rs:14-38)."""
        return factor_format.lu_to_json(self.lu.to_numpy(), self.ipiv.to_numpy()[: self.lu.nrows])

    @classmethod
    def from_json(cls, s: str, flags: int = 0) -> "LU":
        """An LU from nalgebra's serde JSON form, its factors on the device."""
        lu, ipiv = factor_format.lu_from_json(s)
        n = lu.shape[0]
        obj = cls.__new__(cls)
        obj.lu, obj.flags, obj.large = DeviceMatrix.from_numpy(lu), flags, n > 128
        obj.ipiv = _padded_i32(ipiv, n)
        zero = np.nonzero(np.diag(lu) == 0)[0]
        obj.info = _dev.from_numpy(np.array([int(zero[0]) + 1 if len(zero) else 0, 0], np.int32))
        if obj.large:
            obj._ws = _bytes(_lib.load().nacu_getrf_workspace_bytes(n))
        return obj


class FullPivLU:
    """LU with full pivoting of one square matrix (n <= 128): packed L\\U in
    the matrix buffer, row and column pivots on the device."""

    def __init__(self, m: DeviceMatrix, flags: int = 0):
        assert m.is_square(), "the batched full-pivot kernel takes square matrices"
        n = m.nrows
        self.lu, self.flags = m, flags
        self.ipiv = _i32(n)
        self.jpiv = _i32(n)
        self.info = _i32(1)
        _lib.call("nacu_dfullpivlu_batched", n, 0, m.data.data_ptr(), n * n, self.ipiv.data_ptr(),
                  self.jpiv.data_ptr(), 0, 0, self.info.data_ptr(), 1, flags, _stream_ptr())

    def _solve_cols(self, b: DeviceMatrix) -> bool:
        n = self.lu.nrows
        info = _i32(1)
        for c0 in range(0, b.ncols, 16):
            k = min(16, b.ncols - c0)
            _lib.call("nacu_dfullpivlu_solve_batched", n, k, self.lu.data.data_ptr(), n * n, self.ipiv.data_ptr(),
                      self.jpiv.data_ptr(), b.data.data_ptr() + c0 * n * 8, n * k, info.data_ptr(), 1, self.flags,
                      _stream_ptr())
        return int(info.item()) == 0

    def solve_mut(self, b: DeviceMatrix) -> bool:
        """FullPivLU::solve_mut (src/linalg/full_piv_lu.rs:185-211)."""
        assert b.nrows == self.lu.nrows, "FullPivLU solve matrix dimension mismatch."
        return self._solve_cols(b)

    def solve(self, b: DeviceMatrix):
        """FullPivLU::solve (full_piv_lu.rs:168-183): a new matrix, or None."""
        res = b.clone_owned()
        return res if self.solve_mut(res) else None

    def try_inverse(self):
        """FullPivLU::try_inverse (full_piv_lu.rs:216-233): solve_mut on the
        identity, 16 columns per launch; None when not invertible."""
        n = self.lu.nrows
        out = DeviceMatrix(np.eye(n).reshape(-1), n, n)
        return out if self._solve_cols(out) else None

    def is_invertible(self) -> bool:
        """FullPivLU::is_invertible (full_piv_lu.rs:242-250): U[n-1][n-1] != 0."""
        return int(self.info.item()) == 0

    def p(self):
        piv = self.ipiv.to_numpy()[: self.lu.nrows]
        return [(i, int(q)) for i, q in enumerate(piv) if q != i]

    def q(self):
        piv = self.jpiv.to_numpy()[: self.lu.nrows]
        return [(i, int(q)) for i, q in enumerate(piv) if q != i]

    def determinant(self) -> float:
        """FullPivLU::determinant (full_piv_lu.rs:254-267)."""
        lu = self.lu.to_numpy()
        n = lu.shape[0]
        res = float(lu[n - 1, n - 1])
        if res == 0.0:
            return 0.0
        for i in range(n - 1):
            res *= float(lu[i, i])
        return res * (-1.0 if (len(self.p()) + len(self.q())) % 2 else 1.0)

    def l(self) -> np.ndarray:
        lu = self.lu.to_numpy()
        return np.tril(lu, -1) + np.eye(lu.shape[0])

    def u(self) -> np.ndarray:
        return np.triu(self.lu.to_numpy())

    def to_json(self) -> str:
        """nalgebra's serde JSON form of FullPivLU (src/linalg/full_piv_lu.rs:14-39)."""
        n = self.lu.nrows
        return factor_format.full_piv_lu_to_json(self.lu.to_numpy(), self.ipiv.to_numpy()[:n],
                                                 self.jpiv.to_numpy()[:n])

    @classmethod
    def from_json(cls, s: str, flags: int = 0) -> "FullPivLU":
        """A FullPivLU from nalgebra's serde JSON form; info is 0 when
        U[n-1][n-1] != 0, else 1 + the first zero U_ii."""
        lu, ipiv, jpiv = factor_format.full_piv_lu_from_json(s)
        n = lu.shape[0]
        obj = cls.__new__(cls)
        obj.lu, obj.flags = DeviceMatrix.from_numpy(lu), flags
        obj.ipiv = _padded_i32(ipiv, n)
        obj.jpiv = _padded_i32(jpiv, n)
        zero = np.nonzero(np.diag(lu) == 0)[0]
        inv = n == 0 or lu[n - 1, n - 1] != 0
        obj.info = _dev.from_numpy(np.array([0 if inv else int(zero[0]) + 1], np.int32))
        return obj


class QR:
    """Householder QR of one matrix (src/linalg/qr.rs:34-40): the axes and R in
    the matrix buffer, the signed diagonal on the device.  A square matrix of
    order <= 128 runs on the shared-memory batched kernel (batch of one); any
    other shape (larger, tall or wide) on the one-launch-per-step kernel
    (nacu_dqr)."""

    def __init__(self, m: DeviceMatrix, flags: int = 0):
        self.qr, self.flags = m, flags
        self.large = not m.is_square() or m.nrows > 128
        k = min(m.nrows, m.ncols)
        self.diag = _f64(k)
        self.info = _i32(1)
        if self.large:
            _lib.call("nacu_dqr", m.nrows, m.ncols, m.data.data_ptr(), max(m.nrows, 1), self.diag.data_ptr(), flags,
                      _stream_ptr())
        else:
            n = m.nrows
            _lib.call("nacu_dqr_batched", n, 0, m.data.data_ptr(), n * n, self.diag.data_ptr(), 0, 0,
                      self.info.data_ptr(), 1, flags, _stream_ptr())

    def _solve_cols(self, b: DeviceMatrix) -> bool:
        m, n = self.qr.shape
        info = _i32(1)
        if self.large:
            ws = _bytes(_lib.load().nacu_qr_solve_workspace_bytes(n))
            _lib.call("nacu_dqr_solve", m, n, b.ncols, self.qr.data.data_ptr(), max(m, 1), self.diag.data_ptr(),
                      b.data.data_ptr(), max(m, 1), info.data_ptr(), ws.data_ptr(), ws.numel(), self.flags,
                      _stream_ptr())
            return int(info.item()) == 0
        for c0 in range(0, b.ncols, 16):
            k = min(16, b.ncols - c0)
            _lib.call("nacu_dqr_solve_batched", n, k, self.qr.data.data_ptr(), n * n, self.diag.data_ptr(),
                      b.data.data_ptr() + c0 * n * 8, n * k, info.data_ptr(), 1, self.flags, _stream_ptr())
        return int(info.item()) == 0

    def solve_mut(self, b: DeviceMatrix) -> bool:
        """QR::solve_mut (src/linalg/qr.rs:204-222), square factors: b is
        overwritten even when it returns False.  Orders above 128 solve in
        FMA arithmetic (no FLAG_EXACT)."""
        assert self.qr.is_square(), "The QR decomposition must be square."
        assert b.nrows == self.qr.nrows, "QR solve matrix dimension mismatch."
        return self._solve_cols(b)

    def solve(self, b: DeviceMatrix):
        """QR::solve (qr.rs:182-198): a new matrix, or None."""
        res = b.clone_owned()
        return res if self.solve_mut(res) else None

    def solve_least_squares(self, b: DeviceMatrix):
        """The least-squares solution of a tall factor (m >= n), as
        nalgebra-lapack's QR solve (qr_util.rs:167-239): an n x nrhs
        DeviceMatrix, or None when some |diag_i| is zero."""
        m, n = self.qr.shape
        assert m >= n and b.nrows == m, "least squares needs m >= n and an m-row right-hand side"
        res = b.clone_owned()
        if not self._solve_cols(res):
            return None
        return DeviceMatrix.from_numpy(res.to_numpy()[:n])

    def try_inverse(self):
        """QR::try_inverse (qr.rs:262-279)."""
        assert self.qr.is_square(), "The QR decomposition must be square."
        n = self.qr.nrows
        out = DeviceMatrix(np.eye(n).reshape(-1), n, n)
        return out if self._solve_cols(out) else None

    def is_invertible(self) -> bool:
        """QR::is_invertible (qr.rs:281-292): square, and no diag entry zero."""
        if not self.qr.is_square():
            return False
        if self.large:
            return bool(np.all(self.diag.to_numpy()[: self.qr.nrows] != 0))
        return int(self.info.item()) == 0

    def r(self) -> np.ndarray:
        """QR::r (qr.rs:81-89): the min(m, n) x n upper trapezoid, |diag| on its
        diagonal."""
        m, n = self.qr.shape
        k = min(m, n)
        r = np.triu(self.qr.to_numpy()[:k, :])
        r[np.arange(k), np.arange(k)] = np.abs(self.diag.to_numpy()[:k])
        return r

    def to_json(self) -> str:
        """nalgebra's serde JSON form of QR (src/linalg/qr.rs:34-40)."""
        k = min(self.qr.shape)
        return factor_format.qr_to_json(self.qr.to_numpy(), self.diag.to_numpy()[:k])

    @classmethod
    def from_json(cls, s: str, flags: int = 0) -> "QR":
        """A QR from nalgebra's serde JSON form (any shape)."""
        qr, diag = factor_format.qr_from_json(s)
        m, n = qr.shape
        k = min(m, n)
        obj = cls.__new__(cls)
        obj.qr, obj.flags = DeviceMatrix.from_numpy(qr), flags
        obj.large = m != n or n > 128
        obj.diag = _padded_f64(diag, k)
        zero = np.nonzero(diag == 0)[0]
        obj.info = _dev.from_numpy(np.array([int(zero[0]) + 1 if len(zero) else 0], np.int32))
        return obj


class ColPivQR:
    """QR with column pivoting of one square matrix (n <= 128): Householder
    axes and R in the matrix buffer, the signed diagonal and the column pivots
    on the device."""

    def __init__(self, m: DeviceMatrix, flags: int = 0):
        assert m.is_square(), "the batched column-pivot kernel takes square matrices"
        n = m.nrows
        self.qr, self.flags = m, flags
        self.diag = _f64(n)
        self.jpiv = _i32(n)
        self.info = _i32(1)
        _lib.call("nacu_dcolpivqr_batched", n, 0, m.data.data_ptr(), n * n, self.diag.data_ptr(),
                  self.jpiv.data_ptr(), 0, 0, self.info.data_ptr(), 1, flags, _stream_ptr())

    def _solve_cols(self, b: DeviceMatrix) -> bool:
        n = self.qr.nrows
        info = _i32(1)
        for c0 in range(0, b.ncols, 16):
            k = min(16, b.ncols - c0)
            _lib.call("nacu_dcolpivqr_solve_batched", n, k, self.qr.data.data_ptr(), n * n, self.diag.data_ptr(),
                      self.jpiv.data_ptr(), b.data.data_ptr() + c0 * n * 8, n * k, info.data_ptr(), 1, self.flags,
                      _stream_ptr())
        return int(info.item()) == 0

    def solve_mut(self, b: DeviceMatrix) -> bool:
        """ColPivQR::solve_mut (src/linalg/col_piv_qr.rs:227-247): b is
        overwritten even when it returns False."""
        assert b.nrows == self.qr.nrows, "ColPivQR solve matrix dimension mismatch."
        return self._solve_cols(b)

    def solve(self, b: DeviceMatrix):
        """ColPivQR::solve (col_piv_qr.rs:205-221): a new matrix, or None."""
        res = b.clone_owned()
        return res if self.solve_mut(res) else None

    def try_inverse(self):
        """ColPivQR::try_inverse (col_piv_qr.rs:288-303)."""
        n = self.qr.nrows
        out = DeviceMatrix(np.eye(n).reshape(-1), n, n)
        return out if self._solve_cols(out) else None

    def is_invertible(self) -> bool:
        """ColPivQR::is_invertible (col_piv_qr.rs:307-320)."""
        return int(self.info.item()) == 0

    def p(self):
        piv = self.jpiv.to_numpy()[: self.qr.nrows]
        return [(i, int(q)) for i, q in enumerate(piv) if q != i]

    def determinant(self) -> float:
        """ColPivQR::determinant (col_piv_qr.rs:324-338): the product of diag
        in order, times the sign of p."""
        res = 1.0
        for d in self.diag.to_numpy()[: self.qr.nrows]:
            res *= float(d)
        return res * (-1.0 if len(self.p()) % 2 else 1.0)

    def r(self) -> np.ndarray:
        """ColPivQR::r (col_piv_qr.rs:97-110): the upper triangle, |diag| on
        its diagonal."""
        n = self.qr.nrows
        r = np.triu(self.qr.to_numpy())
        r[np.arange(n), np.arange(n)] = np.abs(self.diag.to_numpy()[:n])
        return r

    def to_json(self) -> str:
        """nalgebra's serde JSON form of ColPivQR (src/linalg/col_piv_qr.rs:14-43)."""
        n = self.qr.nrows
        return factor_format.col_piv_qr_to_json(self.qr.to_numpy(), self.jpiv.to_numpy()[:n],
                                                self.diag.to_numpy()[:n])

    @classmethod
    def from_json(cls, s: str, flags: int = 0) -> "ColPivQR":
        """A ColPivQR from nalgebra's serde JSON form."""
        qr, jpiv, diag = factor_format.col_piv_qr_from_json(s)
        n = qr.shape[0]
        obj = cls.__new__(cls)
        obj.qr, obj.flags = DeviceMatrix.from_numpy(qr), flags
        obj.diag = _padded_f64(diag, n)
        obj.jpiv = _padded_i32(jpiv, n)
        zero = np.nonzero(diag == 0)[0]
        obj.info = _dev.from_numpy(np.array([int(zero[0]) + 1 if len(zero) else 0], np.int32))
        return obj


def solve_refined(a: DeviceMatrix, b: DeviceMatrix, tol_units: float = 1.0, max_iter: int = 0):
    """The precision form for one large system (no nalgebra counterpart): FP32
    LU with BF16-split tensor-core trailing updates, FP64 iterative refinement
    to backward error <= tol_units * n * eps64 (GMRES-IR preconditioned by the
    FP32 factors where classical refinement stalls), FP64 fallback.  ``a`` and
    ``b`` are left unchanged.  Returns (x, info) with info = dict(iters, berr,
    fallback, gmres)."""
    import ctypes as C

    n = a.nrows
    assert a.is_square() and b.nrows == n and b.ncols == 1, "one n x n system with one right-hand side"
    x = DeviceMatrix(_dev.empty(n, np.float64), n, 1)
    ws = _bytes(_lib.load().nacu_gesv_mixed_workspace_bytes(n))
    it, berr, fb = C.c_int(0), C.c_double(0.0), C.c_int(0)
    _lib.call("nacu_dgesv_mixed_ir", n, a.data.data_ptr(), n, b.data.data_ptr(), x.data.data_ptr(),
              float(tol_units), int(max_iter), C.byref(it), C.byref(berr), C.byref(fb), ws.data_ptr(), ws.numel(),
              _stream_ptr())
    return x, {"iters": it.value, "berr": berr.value, "fallback": fb.value == 1, "gmres": fb.value == 2}


def cholesky_solve_refined_host(ns, a_offsets, a, b_offsets, b, nrhs: int, chunks: int = 8, tol_units: float = 1.0,
                                max_iter: int = 0):
    """The ragged precision-form SPD solve from host memory (no nalgebra
    counterpart; it replaces `m.cholesky()` + `.solve(&b)` per matrix,
    src/linalg/cholesky.rs:221-272, 122-143): ``a`` and ``b`` are host arrays in
    the packed ragged layout (matrix s at a[a_offsets[s]:], ns[s] x ns[s]
    column-major; its nrhs right-hand sides at b[b_offsets[s]:]).  The copies in
    and out are pipelined with the solves over ``chunks`` parts
    (nacu_dposv_ragged_mixed_host); inputs in page-locked host memory
    (``pinned_empty``) let the copies in overlap the solves, and the outputs
    are page-locked.  Returns (x, info, iters) as host arrays, x in the layout
    of b."""
    _dev.require_gpu()
    hns = np.ascontiguousarray(ns, dtype=np.int32)
    haoff, hboff = np.ascontiguousarray(a_offsets, dtype=np.int64), np.ascontiguousarray(b_offsets, dtype=np.int64)
    ha, hb = np.ascontiguousarray(a, dtype=np.float64), np.ascontiguousarray(b, dtype=np.float64)
    count = int(hns.size)
    hx = pinned_empty(hb.size, np.float64)
    hinfo = pinned_empty(count, np.int32)
    hit = pinned_empty(count, np.int32)
    n_max = int(hns.max()) if count else 0
    L = _lib.load()
    nbytes = L.nacu_mixed_host_workspace_bytes(count, n_max, hns.ctypes.data, haoff.ctypes.data, hboff.ctypes.data,
                                               int(nrhs), int(chunks))
    if count and nbytes == 0:
        raise NacuError("cholesky_solve_refined_host: invalid layout (orders or offsets)")
    ws = _bytes(max(nbytes, 256))
    s = _stream_ptr()
    _lib.call("nacu_dposv_ragged_mixed_host", count, n_max, hns.ctypes.data, haoff.ctypes.data, ha.ctypes.data,
              int(nrhs), hboff.ctypes.data, hb.ctypes.data, hx.ctypes.data if hx.size else None,
              hinfo.ctypes.data if count else None, hit.ctypes.data if count else None, int(chunks),
              ws.data_ptr(), ws.numel(), float(tol_units), int(max_iter), 0.0, 0, s)
    synchronize(s)
    return hx, hinfo, hit


def gemm(c: DeviceMatrix, alpha: float, a: DeviceMatrix, b: DeviceMatrix, beta: float, split_slices: int = 0):
    """Matrix::gemm (src/base/blas.rs:729-746): c = alpha a b + beta c, in
    place.  split_slices = 1..3 selects the BF16-split tensor-core form."""
    _dev.require_gpu()
    m, k = a.shape
    k2, n = b.shape
    assert k == k2 and c.shape == (m, n), "gemm dimension mismatch"
    if split_slices:
        wsb = _lib.load().nacu_gemm_split_workspace_bytes(m, n, k)
        ws = _bytes(wsb + 1024)
        wp = (ws.data_ptr() + 1023) // 1024 * 1024
        _lib.call("nacu_dgemm_split_bf16", m, n, k, float(alpha), a.data.data_ptr(), max(m, 1), b.data.data_ptr(),
                  max(k, 1), float(beta), c.data.data_ptr(), max(m, 1), int(split_slices), wp, wsb, _stream_ptr())
    else:
        _lib.call("nacu_dgemm", m, n, k, float(alpha), a.data.data_ptr(), max(m, 1), b.data.data_ptr(), max(k, 1),
                  float(beta), c.data.data_ptr(), max(m, 1), _stream_ptr())
    return c


def gemm_batched(c, alpha: float, a, b, beta: float, flags: int = 0):
    """Matrix::gemm over a batch (src/base/blas.rs:729-746): c[s] = alpha a[s]
    b[s] + beta c[s], in place, for C-contiguous float64 device arrays
    (DeviceBuffer, or any array with ``__cuda_array_interface__``) of shapes
    (batch, k, m), (batch, n, k) and (batch, n, m) -- each product's
    column-major image, i.e. the transposed row-major view.  ``a @ b`` for many
    matrices (src/base/ops.rs:566-570) is alpha = 1, beta = 0.  FLAG_EXACT:
    nalgebra's gemv summation order, bit for bit."""
    _dev.require_gpu()
    da, db = _dev.as_device(a, np.float64), _dev.as_device(b, np.float64)
    dc = DeviceBuffer.wrap(c)  # written in place: a device array
    if dc.dtype != np.float64:
        raise TypeError("gemm_batched: c must be a float64 device array")
    for t in (da, db, dc):
        if len(t.shape) != 3:
            raise ValueError("gemm_batched takes (batch, rows, cols) device arrays")
    batch, k, m = da.shape
    batch2, n, k2 = db.shape
    assert batch == batch2 and k == k2 and tuple(dc.shape) == (batch, n, m), "gemm_batched dimension mismatch"
    _lib.call("nacu_dgemm_batched", m, n, k, float(alpha), da.data_ptr(), max(m, 1), m * k, db.data_ptr(),
              max(k, 1), k * n, float(beta), dc.data_ptr(), max(m, 1), m * n, batch, int(flags), _stream_ptr())
    return c


class Cholesky:
    """Cholesky factor of one SPD matrix (n <= 512); the strict upper triangle
    keeps the input values, as nalgebra's l_dirty (src/linalg/cholesky.rs:115)."""

    def __init__(self, m: DeviceMatrix, flags: int = 0, substitute: float | None = None):
        self.chol = m
        self.flags = flags | (FLAG_SUBSTITUTE if substitute is not None else 0)
        self.substitute = 0.0 if substitute is None else float(substitute)
        self.info = _i32(1)
        self.logdet = _f64(1)
        _lib.call("nacu_dposv", m.nrows, m.data.data_ptr(), 0, 0, self.info.data_ptr(), self.logdet.data_ptr(),
                  self.substitute, self.flags, _stream_ptr())

    def solve_mut(self, b: DeviceMatrix) -> None:
        """Cholesky::solve_mut (src/linalg/cholesky.rs:122-129)."""
        n = self.chol.nrows
        assert b.nrows == n
        ns = _dev.from_numpy(np.array([n], np.int32))
        off = _dev.zeros(1, np.int64)
        ws = _dev.zeros(_lib.load().nacu_ragged_workspace_bytes(1), np.uint8)
        _lib.call("nacu_dpotrs_ragged", 1, n, ns.data_ptr(), off.data_ptr(), self.chol.data.data_ptr(), b.ncols,
                  off.data_ptr(), b.data.data_ptr(), 0, ws.data_ptr(), ws.numel(), self.flags, _stream_ptr())

    def solve(self, b: DeviceMatrix) -> DeviceMatrix:
        res = b.clone_owned()
        self.solve_mut(res)
        return res

    @classmethod
    def _from_factor(cls, factor: DeviceMatrix, flags: int) -> "Cholesky":
        obj = cls.__new__(cls)
        obj.chol, obj.flags, obj.substitute = factor, flags, 0.0
        obj.info, obj.logdet = None, None
        return obj

    def _ok(self) -> bool:
        return self.info is None or int(self.info.item()) == 0

    def ln_determinant(self) -> float:
        """Cholesky::ln_determinant (src/linalg/cholesky.rs:172-185): the sum of
        ln L_ii, in row order, times two; read from the device after a factor
        update."""
        if self.logdet is not None:
            return float(self.logdet.item())
        d = np.diag(self.chol.to_numpy())
        acc = 0.0
        for v in d:
            acc += float(np.log(abs(v)))
        return acc * 2.0

    def rank_one_update(self, x: DeviceMatrix, sigma: float) -> None:
        """Cholesky::rank_one_update (src/linalg/cholesky.rs:277-285): the factor
        becomes that of L L^T + sigma x x^T, in place (n <= 128); x is read only."""
        n = self.chol.nrows
        assert x.nrows == n and x.ncols == 1
        s = _dev.from_numpy(np.array([float(sigma)]))
        _lib.call("nacu_dchol_rank1_update_batched", n, self.chol.data.data_ptr(), n * n, x.data.data_ptr(), n,
                  s.data_ptr(), 1, self.flags & FLAG_EXACT, _stream_ptr())
        self.logdet = None

    def remove_column(self, j: int) -> "Cholesky":
        """Cholesky::remove_column (src/linalg/cholesky.rs:365-399): the factor
        of the matrix without row and column j (n <= 128)."""
        n = self.chol.nrows
        assert 0 <= j < n
        out = DeviceMatrix(_dev.zeros((n - 1) * (n - 1), np.float64), n - 1, n - 1)
        _lib.call("nacu_dchol_remove_column_batched", n, self.chol.data.data_ptr(), n * n, j, out.data.data_ptr(),
                  max((n - 1) * (n - 1), 0), 1, self.flags & FLAG_EXACT, _stream_ptr())
        return Cholesky._from_factor(out, self.flags & FLAG_EXACT)

    def insert_column(self, j: int, col: DeviceMatrix) -> "Cholesky":
        """Cholesky::insert_column (src/linalg/cholesky.rs:287-357): the factor of
        the matrix with col (n+1 values) inserted as row and column j (n <= 127).
        Raises ValueError where nalgebra's assertion on the lower solve fails."""
        n = self.chol.nrows
        assert 0 <= j <= n and col.nrows == n + 1 and col.ncols == 1
        out = DeviceMatrix(_dev.zeros((n + 1) * (n + 1), np.float64), n + 1, n + 1)
        info = _i32(1)
        _lib.call("nacu_dchol_insert_column_batched", n, self.chol.data.data_ptr(), n * n, j, col.data.data_ptr(),
                  n + 1, out.data.data_ptr(), (n + 1) * (n + 1), info.data_ptr(), 1, self.flags & FLAG_EXACT,
                  _stream_ptr())
        if int(info.item()) != 0:
            raise ValueError("insert_column: the lower triangular solve met a zero diagonal")
        return Cholesky._from_factor(out, self.flags & FLAG_EXACT)

    def l(self) -> np.ndarray:
        return np.tril(self.chol.to_numpy())

    def to_json(self) -> str:
        """nalgebra's serde JSON form of Cholesky (src/linalg/cholesky.rs:15-33)."""
        return factor_format.cholesky_to_json(self.chol.to_numpy())

    @classmethod
    def from_json(cls, s: str, flags: int = 0) -> "Cholesky":
        """A Cholesky from nalgebra's serde JSON form, its factor on the device."""
        return cls._from_factor(DeviceMatrix.from_numpy(factor_format.cholesky_from_json(s)), flags)


class DeviceBatch:
    """Many matrices on the GPU, packed back to back (each column-major), with a
    device offset table: a ragged batch when orders differ.

    ``ns`` are the row counts, ``ms`` the column counts (== ns for square)."""

    def __init__(self, data, nrows, ncols=None, offsets=None):
        self.nrows = np.asarray(nrows, dtype=np.int64)
        self.ncols = self.nrows.copy() if ncols is None else np.asarray(ncols, dtype=np.int64)
        sizes = self.nrows * self.ncols
        if offsets is None:
            offsets = np.concatenate([[0], np.cumsum(sizes)[:-1]]) if sizes.size else np.zeros(0, np.int64)
        self.offsets = np.asarray(offsets, dtype=np.int64)
        self.data = _dev_f64(data)
        self._d_rows = _dev.from_numpy(self.nrows.astype(np.int32))
        self._d_off = _dev.from_numpy(self.offsets)

    @classmethod
    def from_numpy(cls, mats) -> "DeviceBatch":
        """From a list of 2-D arrays, or a (batch, n, m) array."""
        mats = [np.asarray(m, dtype=np.float64).reshape(np.shape(m)[0], -1) for m in mats]
        flat = np.concatenate([np.asfortranarray(m).ravel(order="F") for m in mats]) if mats else np.zeros(0)
        return cls(flat, [m.shape[0] for m in mats], [m.shape[1] for m in mats])

    def __len__(self) -> int:
        return int(self.nrows.size)

    def to_numpy(self):
        host = self.data.to_numpy().reshape(-1)
        return [host[o:o + r * c].reshape(c, r).T.copy()
                for o, r, c in zip(self.offsets, self.nrows, self.ncols)]

    def clone_owned(self) -> "DeviceBatch":
        return DeviceBatch(self.data.clone(), self.nrows, self.ncols, self.offsets)

    def is_uniform(self) -> bool:
        return self.nrows.size > 0 and np.all(self.nrows == self.nrows[0]) and np.all(self.ncols == self.ncols[0])

    def lu(self, flags: int = 0) -> "LUBatch":
        return LUBatch(self, flags)

    def cholesky(self, flags: int = 0, substitute: float | None = None) -> "CholeskyBatch":
        return CholeskyBatch(self, flags, substitute)

    def qr(self) -> "QRBatch":
        return QRBatch(self)


class LUBatch:
    """Batched LU of equal-order square matrices (n <= 128).  Lazy: the first
    ``solve`` runs the fused factor + solve kernel."""

    def __init__(self, batch: DeviceBatch, flags: int = 0):
        if not batch.is_uniform() or batch.nrows[0] != batch.ncols[0]:
            raise ValueError("LUBatch needs equal-order square matrices")
        self.batch = batch
        self.n = int(batch.nrows[0])
        self.flags = flags
        self.ipiv = _i32(len(batch) * self.n)
        self.info = _dev.zeros(len(batch), np.int32)
        self.factored = False

    def factor(self) -> "LUBatch":
        if not self.factored:
            n = self.n
            _lib.call("nacu_dgetrf_batched", n, self.batch.data.data_ptr(), n * n, self.ipiv.data_ptr(),
                      self.info.data_ptr(), len(self.batch), self.flags, _stream_ptr())
            self.factored = True
        return self

    def solve_mut(self, b: DeviceBatch):
        """Solves every system in place; returns the device info array
        (0 = solved, k = U_kk == 0, nalgebra's ``false``)."""
        n = self.n
        if not (np.all(b.nrows == n) and b.is_uniform()):
            raise ValueError("right-hand sides must be n x nrhs each")
        nrhs = int(b.ncols[0])
        if self.factored:
            _lib.call("nacu_dgetrs_batched", n, nrhs, self.batch.data.data_ptr(), n * n, self.ipiv.data_ptr(),
                      b.data.data_ptr(), n * nrhs, self.info.data_ptr(), len(self.batch), self.flags, _stream_ptr())
        else:
            _lib.call("nacu_dgesv_batched", n, nrhs, self.batch.data.data_ptr(), n * n, self.ipiv.data_ptr(),
                      b.data.data_ptr(), n * nrhs, self.info.data_ptr(), len(self.batch), self.flags, _stream_ptr())
            self.factored = True
        return self.info

    def solve(self, b: DeviceBatch) -> DeviceBatch:
        res = b.clone_owned()
        self.solve_mut(res)
        return res

    def try_inverse(self):
        """LU::try_inverse (src/linalg/lu.rs:266-297) of every matrix: returns
        (inverses as a DeviceBatch, device info: 0 = invertible, k = U_kk == 0,
        nalgebra's None)."""
        self.factor()
        n, cnt = self.n, len(self.batch)
        data = _dev.empty(max(cnt * n * n, 1), np.float64)
        info = _dev.zeros(cnt, np.int32)
        _lib.call("nacu_dgetri_batched", n, self.batch.data.data_ptr(), n * n, self.ipiv.data_ptr(), data.data_ptr(),
                  n * n, info.data_ptr(), cnt, self.flags, _stream_ptr())
        nn = np.full(cnt, n, dtype=np.int32)
        return DeviceBatch(data, nn, nn, np.arange(cnt, dtype=np.int64) * n * n), info

    def pivots(self) -> np.ndarray:
        self.factor()
        return self.ipiv.to_numpy().reshape(len(self.batch), self.n)


class CholeskyBatch:
    """Ragged batched Cholesky (orders up to 512): persistent launches over the
    library's size-bucketed order, each bucket with its autotuned tile
    (``nalgebra_gb300.tuning``).  Lazy: ``solve`` runs factor + solve +
    log-determinant in one pass over the batch."""

    def __init__(self, batch: DeviceBatch, flags: int = 0, substitute: float | None = None):
        if np.any(batch.nrows != batch.ncols):
            raise ValueError("Cholesky needs square matrices")
        self.batch = batch
        self.flags = flags | (FLAG_SUBSTITUTE if substitute is not None else 0)
        self.substitute = 0.0 if substitute is None else float(substitute)
        count = len(batch)
        self.n_max = int(batch.nrows.max()) if count else 0
        self.info = _dev.zeros(count, np.int32)
        self.logdet = _dev.zeros(count, np.float64)
        order = np.argsort(-batch.nrows, kind="stable").astype(np.int32)  # largest first
        self._order = _dev.from_numpy(order)
        self._ws = _dev.zeros(_lib.load().nacu_ragged_workspace_bytes(count), np.uint8)
        self.factored = False

    def factor(self) -> "CholeskyBatch":
        if not self.factored:
            b = self.batch
            _lib.call("nacu_dpotrf_ragged", len(b), self.n_max, b._d_rows.data_ptr(), b._d_off.data_ptr(),
                      b.data.data_ptr(), self.info.data_ptr(), self.logdet.data_ptr(), None,
                      self._ws.data_ptr(), self._ws.numel(), self.substitute, self.flags, _stream_ptr())
            self.factored = True
        return self

    def solve_mut(self, rhs: DeviceBatch):
        """Solve in place; returns the device info array (0 = SPD and solved)."""
        b = self.batch
        if len(rhs) != len(b) or np.any(rhs.nrows != b.nrows):
            raise ValueError("one n x nrhs right-hand side block per matrix")
        nrhs = int(rhs.ncols[0]) if len(rhs) else 0
        if len(rhs) and np.any(rhs.ncols != nrhs):
            raise ValueError("every right-hand side block needs the same nrhs")
        if self.factored:
            _lib.call("nacu_dpotrs_ragged", len(b), self.n_max, b._d_rows.data_ptr(), b._d_off.data_ptr(),
                      b.data.data_ptr(), nrhs, rhs._d_off.data_ptr(), rhs.data.data_ptr(), None,
                      self._ws.data_ptr(), self._ws.numel(), self.flags, _stream_ptr())
        else:
            _lib.call("nacu_dposv_ragged", len(b), self.n_max, b._d_rows.data_ptr(), b._d_off.data_ptr(),
                      b.data.data_ptr(), nrhs, rhs._d_off.data_ptr(), rhs.data.data_ptr(), self.info.data_ptr(),
                      self.logdet.data_ptr(), None, self._ws.data_ptr(), self._ws.numel(),
                      self.substitute, self.flags, _stream_ptr())
            self.factored = True
        return self.info

    def solve(self, rhs: DeviceBatch) -> DeviceBatch:
        res = rhs.clone_owned()
        self.solve_mut(res)
        return res

    def capture(self, rhs: DeviceBatch) -> Graph:
        """Capture the fused factor + solve + log-det of this batch into a CUDA
        graph (``Graph``); ``graph.replay()`` re-runs it on the same device
        buffers (refill them between replays: the factorization is in place).
        The calls it captures neither synchronize nor allocate."""
        self.factored = False
        self.solve_mut(rhs)  # warm-up launch outside the graph (first-use set-up)
        g = Graph()
        with g.capture():
            self.factored = False
            self.solve_mut(rhs)
        return g

    def ln_determinant(self) -> np.ndarray:
        self.factor()
        return self.logdet.to_numpy()

    def solve_refined_into(self, rhs: DeviceBatch, out: DeviceBatch, tol_units: float = 1.0, max_iter: int = 0,
                           verify: bool = False):
        """The precision form (nacu_dposv_ragged_mixed): FP32 factor, FP64
        iterative refinement to backward error <= tol_units * n * eps64, FP64
        fallback per matrix.  The batch's matrices and ``rhs`` are left
        unchanged; solutions go to ``out`` (same layout as ``rhs``).  Returns the
        device per-matrix residual counts (negative: FP64 fallback used)."""
        b = self.batch
        nrhs = int(rhs.ncols[0]) if len(rhs) else 0
        if not hasattr(self, "_mws"):
            total = int(b.data.numel())
            self._mws = _bytes(_lib.load().nacu_mixed_workspace_bytes(len(b), total))
            self._iters = _i32(len(b))
        flags = self.flags & FLAG_SUBSTITUTE
        if verify:
            flags |= _lib.FLAG_VERIFY
        _lib.call("nacu_dposv_ragged_mixed", len(b), self.n_max, b._d_rows.data_ptr(), b._d_off.data_ptr(),
                  b.data.data_ptr(), nrhs, rhs._d_off.data_ptr(), rhs.data.data_ptr(), out.data.data_ptr(),
                  self.info.data_ptr(), self._iters.data_ptr(), self._order.data_ptr(), int(b.data.numel()),
                  self._mws.data_ptr(), self._mws.numel(), float(tol_units), int(max_iter), self.substitute, flags,
                  _stream_ptr())
        return self._iters

    def solve_refined(self, rhs: DeviceBatch, **kw) -> DeviceBatch:
        out = rhs.clone_owned()
        self.solve_refined_into(rhs, out, **kw)
        return out

    def is_ok(self) -> np.ndarray:
        """Per matrix: True where nalgebra's ``cholesky()`` returns Some."""
        self.factor()
        return self.info.to_numpy() == 0


class QRBatch:
    """Batched Householder QR of tall matrices (equal column count n <= 128,
    ragged row counts m >= n, m <= 2048), nalgebra's stored layout and sign
    convention (src/linalg/qr.rs:55-76).  Lazy: ``solve`` runs factor + Q^T b +
    least squares in one launch."""

    def __init__(self, batch: DeviceBatch):
        if len(batch) and not np.all(batch.ncols == batch.ncols[0]):
            raise ValueError("QRBatch needs the same column count in every matrix")
        self.batch = batch
        self.n = int(batch.ncols[0]) if len(batch) else 0
        if np.any(batch.nrows < self.n):
            raise ValueError("least squares needs m >= n (nalgebra-lapack Error::Underdetermined)")
        count = len(batch)
        self.m_max = int(batch.nrows.max()) if count else 0
        self.diag = _f64(count * self.n)
        self.info = _i32(count)
        order = np.argsort(-batch.nrows, kind="stable").astype(np.int32)
        self._order = _dev.from_numpy(order)
        self._ws = _dev.zeros(_lib.load().nacu_qr_workspace_bytes(count), np.uint8)
        self.factored = False

    def _launch(self, rhs: "DeviceBatch | None", x):
        b = self.batch
        _lib.call("nacu_dgels_batched", len(b), self.n, self.m_max, b._d_rows.data_ptr(), b._d_off.data_ptr(),
                  b.data.data_ptr(), rhs._d_off.data_ptr() if rhs is not None else 0,
                  rhs.data.data_ptr() if rhs is not None else 0, x.data_ptr() if x is not None else 0,
                  self.diag.data_ptr(), self.info.data_ptr(), self._order.data_ptr(), self._ws.data_ptr(),
                  self._ws.numel(), 0, _stream_ptr())
        self.factored = True

    def factor(self) -> "QRBatch":
        if not self.factored:
            self._launch(None, None)
        return self

    def solve_mut(self, rhs: DeviceBatch):
        """Least squares for one m x 1 right-hand side per matrix; rhs becomes
        Q^T b (as QR::q_tr_mul) and the n x 1 solutions are returned as a flat
        (count * n) device tensor.  Factor + solve run in one launch."""
        if self.factored:
            raise NotImplementedError("solve after a separate factor(): call solve on a fresh QRBatch")
        if len(rhs) != len(self.batch) or np.any(rhs.nrows != self.batch.nrows) or np.any(rhs.ncols != 1):
            raise ValueError("one m x 1 right-hand side per matrix")
        x = _f64(len(self.batch) * self.n)
        self._launch(rhs, x)
        return x

    def solve(self, rhs: DeviceBatch) -> np.ndarray:
        """nalgebra-lapack QR::solve (nalgebra-lapack/src/qr/abstraction.rs:48-77):
        the (count, n) least-squares solutions (host), rank-deficient rows NaN."""
        res = rhs.clone_owned()
        x = self.solve_mut(res).to_numpy()[: len(self.batch) * self.n].reshape(len(self.batch), self.n)
        bad = self.info.to_numpy()[: len(self.batch)] != 0
        x[bad] = np.nan
        return x

    def diag_host(self) -> np.ndarray:
        self.factor()
        return self.diag.to_numpy()[: len(self.batch) * self.n].reshape(len(self.batch), self.n)


class PosvLogdet:
    """The differentiation form (no nalgebra counterpart: nalgebra has no
    autodiff): a batch of equal-order SPD systems (n <= 128), f64 or f32,

        x_s = A_s^-1 b_s,   logdet_s = ln det A_s      (forward)

    and the reverse-mode adjoint

        (x_bar, logdet_bar) -> (A_bar, b_bar)          (backward)

    where A_bar is the gradient with respect to the lower-triangle entries
    nalgebra reads (off-diagonal entries count for A_ij and A_ji).  The
    store form keeps the Cholesky factor from the forward pass; the recompute
    form keeps nothing and refactors A in the backward pass (n^2 values per
    matrix saved for n^3/3 extra flops).  A is (batch, n*n) column-major rows,
    b (batch, n): host arrays (copied) or device arrays of the form's dtype
    (used in place); the results are DeviceBuffers."""

    def __init__(self, n: int, batch: int, dtype="float64", recompute: bool = False):
        _dev.require_gpu()
        self.n, self.batch = int(n), int(batch)
        self.tdt = np.dtype(np.float64 if str(dtype).endswith("64") else np.float32)
        self.pre = "d" if self.tdt == np.float64 else "s"
        self.recompute = bool(recompute)
        self.L = None if self.recompute else _dev.zeros((self.batch, self.n * self.n), self.tdt)
        self.info = _dev.zeros(max(self.batch, 1), np.int32)
        self._A = self._x = None

    def forward(self, A, b):
        A = _dev.as_device(A, self.tdt)
        b = _dev.as_device(b, self.tdt)
        if A.numel() != self.batch * self.n * self.n or b.numel() != self.batch * self.n:
            raise ValueError("PosvLogdet.forward: A is (batch, n*n) and b (batch, n)")
        x = _dev.empty((self.batch, self.n), self.tdt)
        logdet = _dev.empty(self.batch, self.tdt)
        _lib.call(f"nacu_{self.pre}posv_logdet_forward", self.n, A.data_ptr(), self.n * self.n, b.data_ptr(),
                  x.data_ptr(), None if self.L is None else self.L.data_ptr(), logdet.data_ptr(),
                  self.info.data_ptr(), self.batch, _stream_ptr())
        self._A, self._x = A, x
        return x, logdet

    def backward(self, x_bar, logdet_bar=None):
        """Returns (A_bar, b_bar); logdet_bar None means 1 for every system."""
        if self._x is None:
            raise RuntimeError("backward before forward")
        w = _dev.as_device(x_bar, self.tdt)
        g = None if logdet_bar is None else _dev.as_device(logdet_bar, self.tdt)
        if w.numel() != self.batch * self.n or (g is not None and g.numel() != self.batch):
            raise ValueError("PosvLogdet.backward: x_bar is (batch, n) and logdet_bar (batch,)")
        dA = _dev.empty((self.batch, self.n * self.n), self.tdt)
        db = _dev.empty((self.batch, self.n), self.tdt)
        src = self._A if self.recompute else self.L
        _lib.call(f"nacu_{self.pre}posv_logdet_backward", self.n, src.data_ptr(), self.n * self.n,
                  1 if self.recompute else 0, self._x.data_ptr(), w.data_ptr(), None if g is None else g.data_ptr(),
                  dA.data_ptr(), db.data_ptr(), self.info.data_ptr(), self.batch, _stream_ptr())
        return dA, db

    def is_ok(self) -> np.ndarray:
        return self.info.to_numpy() == 0
