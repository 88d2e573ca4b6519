"""GPU parity of the batched LU with full pivoting (nacu_dfullpivlu_batched,
nacu_dfullpivlu_solve_batched) against the oracle's restatement of
src/linalg/full_piv_lu.rs: with NACU_FLAG_EXACT the factors, the row and
column pivots, info and the solutions are bit-identical (NaN positions
included); the FMA form reproduces P A Q = L U and solves to a small backward
error.  Each batch mixes random matrices (uniform in [-100, 100], the
reference's proptest range) with a rank-1 matrix of signed powers of two,
whose elimination is exact (the steps stop at the zero remainder), the zero
matrix, a NaN at (0, 0) (it wins the pivot search) and a NaN elsewhere (it
never does)."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import FLAG_EXACT, NacuError, _lib

pytestmark = pytest.mark.gpu


def _batch(n, count, seed):
    rng = np.random.default_rng(seed)
    mats = [rng.uniform(-100, 100, size=(n, n)) for _ in range(count)]
    if n >= 2 and count >= 6:
        signs = np.where(rng.random(n) < 0.5, -1.0, 1.0)
        mats[1] = np.outer(2.0 ** rng.integers(-3, 4, n), signs * 2.0 ** rng.integers(-2, 3, n))
        mats[2] = np.zeros((n, n))
        mats[3][0, 0] = np.nan
        mats[4][n - 1, n // 2] = np.nan
    return mats


def _info_ref(lu, steps):
    n = lu.shape[0]
    return 0 if (n == 0 or lu[n - 1, n - 1] != 0) else steps + 1


def _dev(torch, mats):
    return torch.from_numpy(np.stack([np.asarray(m).ravel(order="F") for m in mats])).cuda()


def _factor(torch, mats, n, flags, rhs=None):
    count = len(mats)
    A = _dev(torch, mats)
    ipiv = torch.full((count * n,), -1, dtype=torch.int32, device="cuda")
    jpiv = torch.full((count * n,), -1, dtype=torch.int32, device="cuda")
    info = torch.full((count,), -7, dtype=torch.int32, device="cuda")
    nrhs, B, bp = 0, None, 0
    if rhs is not None:
        nrhs = rhs[0].shape[1]
        B = _dev(torch, rhs)
        bp = B.data_ptr()
    _lib.call("nacu_dfullpivlu_batched", n, nrhs, A.data_ptr(), n * n, ipiv.data_ptr(), jpiv.data_ptr(), bp,
              n * nrhs, info.data_ptr(), count, flags, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    out = (A.cpu().numpy(), ipiv.cpu().numpy().reshape(count, n), jpiv.cpu().numpy().reshape(count, n),
           info.cpu().numpy())
    return out + ((B.cpu().numpy() if B is not None else None),)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 33, 64, 100, 128])
def test_factor_exact_bit_identical(cuda, n):
    mats = _batch(n, 6, 10 + n)
    A, ipiv, jpiv, info, _ = _factor(cuda, mats, n, FLAG_EXACT)
    for k, m in enumerate(mats):
        lu, ip, jp, steps = O.full_piv_lu(m)
        assert np.array_equal(A[k].reshape(n, n).T, lu, equal_nan=True), (n, k)
        assert np.array_equal(ipiv[k], ip) and np.array_equal(jpiv[k], jp), (n, k)
        assert info[k] == _info_ref(lu, steps), (n, k)
    if n >= 2:
        assert info[2] == 1 and info[1] >= 2  # the zero matrix stops at once, the rank-1 one after a step


@pytest.mark.parametrize("n,nrhs", [(5, 1), (64, 1), (64, 3), (128, 16)])
def test_factor_and_solve_exact(cuda, n, nrhs):
    mats = _batch(n, 6, 30 + n)
    rng = np.random.default_rng(31 + n)
    rhs = [rng.standard_normal((n, nrhs)) for _ in mats]
    A, ipiv, jpiv, info, B = _factor(cuda, mats, n, FLAG_EXACT, rhs)
    for k, m in enumerate(mats):
        lu, ip, jp, steps = O.full_piv_lu(m)
        x = O.full_piv_lu_solve(lu, ip, jp, rhs[k])
        got = B[k].reshape(nrhs, n).T
        if x is None:
            assert info[k] != 0 and np.array_equal(got, rhs[k]), (n, k)  # b untouched
        else:
            assert info[k] == 0 and np.array_equal(got, x.reshape(n, nrhs), equal_nan=True), (n, k)


@pytest.mark.parametrize("n", [4, 64, 128])
def test_solve_from_factors_and_try_inverse_exact(cuda, n):
    torch = cuda
    mats = _batch(n, 6, 50 + n)
    A, ipiv, jpiv, info, _ = _factor(torch, mats, n, FLAG_EXACT)
    count = len(mats)
    LU = torch.from_numpy(A).cuda()
    IP = torch.from_numpy(ipiv.reshape(-1).copy()).cuda()
    JP = torch.from_numpy(jpiv.reshape(-1).copy()).cuda()
    inv = torch.from_numpy(np.tile(np.eye(n).ravel(order="F"), (count, 1))).cuda()
    sinfo = torch.full((count,), -7, dtype=torch.int32, device="cuda")
    for c0 in range(0, n, 16):  # try_inverse: solve_mut on the identity, 16 columns per call
        k = min(16, n - c0)
        _lib.call("nacu_dfullpivlu_solve_batched", n, k, LU.data_ptr(), n * n, IP.data_ptr(), JP.data_ptr(),
                  inv.data_ptr() + c0 * n * 8, n * n, sinfo.data_ptr(), count, FLAG_EXACT,
                  torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got, si = inv.cpu().numpy(), sinfo.cpu().numpy()
    for k in range(count):
        lu = A[k].reshape(n, n).T
        ref = O.full_piv_lu_solve(lu, ipiv[k], jpiv[k], np.eye(n))
        if ref is None:
            assert si[k] != 0 and np.array_equal(got[k].reshape(n, n).T, np.eye(n)), (n, k)
        else:
            assert si[k] == 0 and np.array_equal(got[k].reshape(n, n).T, ref, equal_nan=True), (n, k)
            if not np.isnan(mats[k]).any():
                assert np.allclose(mats[k] @ ref, np.eye(n), atol=1e-9 * n, rtol=0)
    assert np.array_equal(LU.cpu().numpy(), A, equal_nan=True)  # the factors are read only


@pytest.mark.parametrize("n", [16, 64, 128])
def test_fma_form_reconstructs_and_solves(cuda, n):
    rng = np.random.default_rng(70 + n)
    mats = [rng.uniform(-100, 100, size=(n, n)) for _ in range(8)]
    rhs = [rng.standard_normal((n, 2)) for _ in mats]
    A, ipiv, jpiv, info, B = _factor(cuda, mats, n, 0, rhs)
    assert np.all(info == 0)
    for k, m in enumerate(mats):
        lu = A[k].reshape(n, n).T
        l, u = np.tril(lu, -1) + np.eye(n), np.triu(lu)
        rec = l @ u
        for i in reversed(range(n)):  # P^T (L U) Q^T
            if ipiv[k][i] != i:
                rec[[i, ipiv[k][i]]] = rec[[ipiv[k][i], i]]
        for i in reversed(range(n)):
            if jpiv[k][i] != i:
                rec[:, [i, jpiv[k][i]]] = rec[:, [jpiv[k][i], i]]
        assert np.abs(rec - m).max() <= 64 * n * np.finfo(float).eps * np.abs(m).max(), (n, k)
        assert np.all(np.abs(np.tril(lu, -1)) <= 1.0)
        x = B[k].reshape(2, n).T
        berr = np.abs(m @ x - rhs[k]).max() / (np.abs(m).max() * np.abs(x).max() * n)
        assert berr <= 4 * np.finfo(float).eps, (n, k, berr)


def test_mirror_full_piv_lu(cuda):
    from nalgebra_gb300 import DeviceMatrix

    m = np.array([[0.0, -1.0, 2.0], [-1.0, 2.0, -1.0], [2.0, -1.0, 0.0]])  # tests/linalg/full_piv_lu.rs:23-40
    lu = DeviceMatrix.from_numpy(m).full_piv_lu(flags=FLAG_EXACT)
    assert lu.determinant() == -4.0
    assert lu.is_invertible()
    x = lu.solve(DeviceMatrix.from_numpy(np.array([[1.0], [2.0], [3.0]])))
    assert np.array_equal(x.to_numpy()[:, 0], O.full_piv_lu_solve(*O.full_piv_lu(m)[:3], np.array([1.0, 2.0, 3.0])))
    inv = lu.try_inverse().to_numpy()
    assert np.allclose(m @ inv, np.eye(3), atol=1e-14, rtol=0)
    z = DeviceMatrix.from_numpy(np.zeros((4, 4))).full_piv_lu()
    assert not z.is_invertible() and z.determinant() == 0.0 and z.try_inverse() is None


def test_argument_errors(cuda):
    with pytest.raises(NacuError):
        _lib.call("nacu_dfullpivlu_batched", 129, 0, 1, 129 * 129, 1, 1, 0, 0, 0, 1, 0, 0)
    with pytest.raises(NacuError):
        _lib.call("nacu_dfullpivlu_batched", 8, 17, 1, 64, 1, 1, 1, 8 * 17, 0, 1, 0, 0)
    with pytest.raises(NacuError):
        _lib.call("nacu_dfullpivlu_solve_batched", 8, 2, 1, 63, 1, 1, 1, 16, 0, 1, 0, 0)
