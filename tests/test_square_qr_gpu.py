"""GPU parity of the batched square QR (nacu_dqr_batched, nacu_dqr_solve_batched)
against the oracle's restatement of src/linalg/qr.rs (QR::new :55-76,
QR::solve_mut :204-256, try_inverse :262-279).  With NACU_FLAG_EXACT the
factors (axes and R), the signed diagonal, info and the solutions are
bit-identical (NaN positions included).  The FMA form is held to the
reference's own properties (tests/linalg/qr.rs:15-22, 55-69, 87-99: Q R = A,
Q orthogonal, A x = b, A A^-1 = I).  Each batch mixes random matrices
(uniform in [-100, 100], the reference's proptest range) with the zero
matrix, a matrix with a zero column and a NaN at (0, 0)."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import FLAG_EXACT, NacuError, _lib

pytestmark = pytest.mark.gpu


def _batch(n, count, seed):
    rng = np.random.default_rng(seed)
    mats = [rng.uniform(-100, 100, size=(n, n)) for _ in range(count)]
    if n >= 2 and count >= 5:
        mats[1] = np.zeros((n, n))
        mats[2][:, n // 2] = 0.0
        mats[3][0, 0] = np.nan
    return mats


def _info_ref(diag):
    z = np.nonzero(diag == 0)[0]
    return 0 if len(z) == 0 else int(z[0]) + 1


def _dev(torch, mats):
    return torch.from_numpy(np.stack([np.asarray(m).ravel(order="F") for m in mats])).cuda()


def _factor(torch, mats, n, flags, rhs=None):
    count = len(mats)
    A = _dev(torch, mats)
    diag = torch.full((count * n,), -7.0, dtype=torch.float64, device="cuda")
    info = torch.full((count,), -7, dtype=torch.int32, device="cuda")
    nrhs, B, bp = 0, None, 0
    if rhs is not None:
        nrhs = rhs[0].shape[1]
        B = _dev(torch, rhs)
        bp = B.data_ptr()
    _lib.call("nacu_dqr_batched", n, nrhs, A.data_ptr(), n * n, diag.data_ptr(), bp, n * nrhs, info.data_ptr(),
              count, flags, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return (A.cpu().numpy(), diag.cpu().numpy().reshape(count, n), info.cpu().numpy(),
            B.cpu().numpy() if B is not None else None)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 20, 33, 64, 100, 128])
def test_factor_exact_bit_identical(cuda, n):
    mats = _batch(n, 5, 120 + n)
    A, diag, info, _ = _factor(cuda, mats, n, FLAG_EXACT)
    for k, m in enumerate(mats):
        qr, d = O.qr(m)
        assert np.array_equal(A[k].reshape(n, n).T, qr, equal_nan=True), (n, k)
        assert np.array_equal(diag[k], d, equal_nan=True), (n, k)
        assert info[k] == _info_ref(d), (n, k)
    if n >= 2:
        assert info[1] == 1


@pytest.mark.parametrize("n,nrhs", [(5, 1), (20, 20 % 16 or 16), (64, 3), (100, 1), (128, 16)])
def test_factor_and_solve_exact(cuda, n, nrhs):
    mats = _batch(n, 5, 140 + n)
    rng = np.random.default_rng(141 + n)
    rhs = [rng.standard_normal((n, nrhs)) for _ in mats]
    A, diag, info, B = _factor(cuda, mats, n, FLAG_EXACT, rhs)
    for k, m in enumerate(mats):
        qr, d = O.qr(m)
        x, ok = O.qr_solve(qr, d, rhs[k])
        assert (info[k] == 0) == ok, (n, k)
        assert np.array_equal(B[k].reshape(nrhs, n).T, x.reshape(n, nrhs), equal_nan=True), (n, k)


@pytest.mark.parametrize("n", [4, 15, 64, 128])
def test_solve_from_factors_and_try_inverse_exact(cuda, n):
    torch = cuda
    mats = _batch(n, 5, 160 + n)
    A, diag, info, _ = _factor(torch, mats, n, FLAG_EXACT)
    count = len(mats)
    QR = torch.from_numpy(A).cuda()
    D = torch.from_numpy(diag.reshape(-1).copy()).cuda()
    inv = torch.from_numpy(np.tile(np.eye(n).ravel(order="F"), (count, 1))).cuda()
    sinfo = torch.full((count,), -7, dtype=torch.int32, device="cuda")
    for c0 in range(0, n, 16):  # try_inverse: solve_mut on the identity, 16 columns per call
        k = min(16, n - c0)
        _lib.call("nacu_dqr_solve_batched", n, k, QR.data_ptr(), n * n, D.data_ptr(), inv.data_ptr() + c0 * n * 8,
                  n * n, sinfo.data_ptr(), count, FLAG_EXACT, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got, si = inv.cpu().numpy(), sinfo.cpu().numpy()
    for k in range(count):
        qr = A[k].reshape(n, n).T
        parts, ok = [], True
        for c0 in range(0, n, 16):  # the oracle per chunk, as the calls above
            x, okc = O.qr_solve(qr, diag[k], np.eye(n)[:, c0:c0 + 16])
            parts.append(x)
            ok = ok and okc
        ref = np.concatenate(parts, axis=1)
        assert (si[k] == 0) == ok, (n, k)
        assert np.array_equal(got[k].reshape(n, n).T, ref, equal_nan=True), (n, k)
        if ok and not np.isnan(mats[k]).any():  # tests/linalg/qr.rs:87-99
            assert np.allclose(mats[k] @ ref, np.eye(n), atol=1e-9 * n, rtol=0)
            assert np.allclose(ref @ mats[k], np.eye(n), atol=1e-9 * n, rtol=0)
    assert np.array_equal(QR.cpu().numpy(), A, equal_nan=True)  # the factors are read only


@pytest.mark.parametrize("n", [1, 16, 64, 128])
def test_fma_form_reconstructs_and_solves(cuda, n):
    rng = np.random.default_rng(180 + n)
    mats = [rng.uniform(-100, 100, size=(n, n)) for _ in range(8)]
    rhs = [rng.standard_normal((n, 2)) for _ in mats]
    A, diag, info, B = _factor(cuda, mats, n, 0, rhs)
    assert np.all(info == 0)
    for k, m in enumerate(mats):
        qr = A[k].reshape(n, n).T
        q, r = O.col_piv_qr_q_r(qr, diag[k])  # Q from q_tr_mul on I, the same for QR's layout
        assert np.abs(q @ r - m).max() <= 64 * n * np.finfo(float).eps * np.abs(m).max(), (n, k)
        assert np.abs(q.T @ q - np.eye(n)).max() <= 1e-7  # tests/linalg/qr.rs:21
        x = B[k].reshape(2, n).T
        berr = np.abs(m @ x - rhs[k]).max() / (np.abs(m).max() * np.abs(x).max() * n)
        assert berr <= 8 * np.finfo(float).eps, (n, k, berr)


@pytest.mark.parametrize("n", [1, 7, 64, 100, 128])
@pytest.mark.parametrize("nrhs", [0, 1])
def test_fma_single_rhs_form(cuda, n, nrhs):
    """The FMA form with at most one right-hand side (the compact-WY kernel of
    the least-squares path): nalgebra's stored layout and signs to rounding,
    info as QR::is_invertible, and b overwritten by the solution."""
    mats = _batch(n, 6, 200 + n)
    rng = np.random.default_rng(201 + n)
    rhs = [rng.standard_normal((n, 1)) for _ in mats] if nrhs else None
    A, diag, info, B = _factor(cuda, mats, n, 0, rhs)
    for k, m in enumerate(mats):
        qr_o, d_o = O.qr(m)
        assert info[k] == _info_ref(d_o), (n, k)
        if np.isnan(m).any() or info[k] != 0:
            continue
        scale = np.abs(m).max()
        assert np.abs(A[k].reshape(n, n).T - qr_o).max() <= 1e-10 * max(1.0, scale), (n, k)
        assert np.abs(diag[k] - d_o).max() <= 1e-10 * scale, (n, k)
        if nrhs:
            x = B[k].reshape(n)
            berr = np.abs(m @ x - rhs[k][:, 0]).max() / (scale * np.abs(x).max() * n)
            assert berr <= 8 * np.finfo(float).eps, (n, k, berr)
            x_o, ok = O.qr_solve(qr_o, d_o, rhs[k])
            assert ok and np.abs(x - x_o[:, 0]).max() <= 1e-9 * np.abs(x_o).max(), (n, k)


def test_mirror_qr(cuda):
    from nalgebra_gb300 import QR, DeviceMatrix

    a = np.array([[4.0, 1.0, 0.0], [1.0, 3.0, 1.0], [0.0, 1.0, 2.0]])
    qa = DeviceMatrix.from_numpy(a).qr(flags=FLAG_EXACT)
    ref_qr, ref_d = O.qr(a)
    assert np.array_equal(qa.qr.to_numpy(), ref_qr)
    assert np.array_equal(qa.r(), O.qr_r(ref_qr, ref_d))
    assert qa.is_invertible()
    b = np.array([[1.0], [2.0], [3.0]])
    x = qa.solve(DeviceMatrix.from_numpy(b)).to_numpy()
    assert np.array_equal(x, O.qr_solve(ref_qr, ref_d, b)[0])
    assert np.allclose(a @ qa.try_inverse().to_numpy(), np.eye(3), atol=1e-14, rtol=0)
    back = QR.from_json(qa.to_json(), flags=FLAG_EXACT)
    assert np.array_equal(back.solve(DeviceMatrix.from_numpy(b)).to_numpy(), x)
    z = DeviceMatrix.from_numpy(np.zeros((3, 3))).qr()
    assert not z.is_invertible() and z.try_inverse() is None
    tall = np.arange(12, dtype=np.float64).reshape(4, 3) ** 1.5  # any shape now: the one-matrix kernel
    qt = DeviceMatrix.from_numpy(tall).qr(flags=FLAG_EXACT)
    ref_qr, ref_d = O.qr(tall)
    assert np.array_equal(qt.r(), O.qr_r(ref_qr, ref_d)) and not qt.is_invertible()


def test_argument_errors(cuda):
    with pytest.raises(NacuError):
        _lib.call("nacu_dqr_batched", 129, 0, 1, 129 * 129, 1, 0, 0, 0, 1, 0, 0)
    with pytest.raises(NacuError):
        _lib.call("nacu_dqr_batched", 8, 17, 1, 64, 1, 1, 8 * 17, 0, 1, 0, 0)
    with pytest.raises(NacuError):
        _lib.call("nacu_dqr_solve_batched", 8, 2, 1, 63, 1, 1, 16, 0, 1, 0, 0)
