"""GPU parity of the one-matrix Householder QR (nacu_dqr, nacu_dqr_solve)
against the oracle's restatement of nalgebra's QR::new (src/linalg/qr.rs:55-76,
householder.rs:19-85, reflection.rs:70-83), q_tr_mul (qr.rs:157-171) and
solve_mut (qr.rs:204-256).  NACU_FLAG_EXACT: the factors and the signed
diagonal are bit-identical for tall, square and wide shapes, zero columns and
NaN included.  The FMA form is held to the reference's QR properties
(tests/linalg/qr.rs:15-22, 55-69: Q R = A, Q orthogonal, A x = b) and to the
oracle's factors within rounding."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import FLAG_EXACT, NacuError, _lib

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def _mat(m, n, seed, special=True):
    rng = np.random.default_rng(seed)
    a = rng.uniform(-100, 100, size=(m, n))  # the reference's proptest range
    if special and min(m, n) >= 8:
        a[:, 3] = 0.0  # a zero column: no reflection at step 3
        a[:, 6] = 1e-170  # squares underflow: a zero norm over a nonzero column at step 6
    return a


def _factor(torch, a, flags):
    m, n = a.shape
    A = torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).cuda()
    diag = torch.full((max(min(m, n), 1),), -7.0, dtype=torch.float64, device="cuda")
    _lib.call("nacu_dqr", m, n, A.data_ptr(), m, diag.data_ptr(), flags, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return A.cpu().numpy().reshape(n, m).T, diag.cpu().numpy()[: min(m, n)]


@pytest.mark.parametrize("m,n", [(1, 1), (1, 7), (7, 1), (129, 129), (200, 130), (300, 200), (100, 500),
                                 (500, 100), (257, 260), (64, 700)])
def test_factor_exact_bit_identical(cuda, m, n):
    a = _mat(m, n, 300 + m + n)
    got, d = _factor(cuda, a, FLAG_EXACT)
    ref, rd = O.qr(a)
    assert np.array_equal(got, ref, equal_nan=True), (m, n)
    assert np.array_equal(d, rd, equal_nan=True), (m, n)
    if min(m, n) >= 8:
        assert rd[3] == 0.0 and d[3] == 0.0


def test_factor_exact_nan_and_zero_matrix(cuda):
    a = _mat(150, 140, 7)
    a[10, 20] = np.nan
    got, d = _factor(cuda, a, FLAG_EXACT)
    ref, rd = O.qr(a)
    assert np.array_equal(got, ref, equal_nan=True) and np.array_equal(d, rd, equal_nan=True)
    z = np.zeros((160, 150))
    got, d = _factor(cuda, z, FLAG_EXACT)
    ref, rd = O.qr(z)
    assert np.array_equal(got, ref) and np.array_equal(d, rd) and not d.any()


@pytest.mark.parametrize("m,n", [(1000, 1000), (2000, 300), (300, 900), (4096, 64)])
def test_factor_fma_matches_oracle(cuda, m, n):
    a = _mat(m, n, 400 + m + n, special=False)
    got, d = _factor(cuda, a, 0)
    ref, rd = O.qr(a)
    k = min(m, n)
    # rounding differences grow with the conditioning (about 2n for these matrices)
    assert np.abs(d - rd).max() <= 1e-8 * np.abs(rd).max(), (m, n)
    axes_g, axes_r = np.tril(got[:, :k]), np.tril(ref[:, :k])
    assert np.abs(axes_g - axes_r).max() <= 1e-8, (m, n)  # unit axes
    assert np.abs(np.triu(got[:k], 1) - np.triu(ref[:k], 1)).max() <= 1e-8 * np.abs(rd).max(), (m, n)


@pytest.mark.parametrize("m,n", [(600, 400), (300, 700)])
def test_fma_factor_reconstructs(cuda, m, n):
    """Q R = A and Q^T Q = I (tests/linalg/qr.rs:15-22), Q from the oracle's
    q_tr_mul on the identity applied to the GPU's factors."""
    a = _mat(m, n, 500 + m, special=False)
    got, d = _factor(cuda, a, 0)
    q, r = O.col_piv_qr_q_r(got, d)
    assert np.abs(q @ r - a).max() <= 64 * max(m, n) * EPS * np.abs(a).max(), (m, n)
    assert np.abs(q.T @ q - np.eye(q.shape[1])).max() <= 1e-7


def _solve(torch, qr, d, b, flags=0):
    m, n = qr.shape
    nrhs = b.shape[1]
    QR = torch.from_numpy(np.asfortranarray(qr).ravel(order="F").copy()).cuda()
    D = torch.from_numpy(np.ascontiguousarray(d)).cuda()
    B = torch.from_numpy(np.asfortranarray(b).ravel(order="F").copy()).cuda()
    info = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    ws = torch.empty(_lib.load().nacu_qr_solve_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    _lib.call("nacu_dqr_solve", m, n, nrhs, QR.data_ptr(), m, D.data_ptr(), B.data_ptr(), m, info.data_ptr(),
              ws.data_ptr(), ws.numel(), flags, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return B.cpu().numpy().reshape(nrhs, m).T, int(info.item())


@pytest.mark.parametrize("n,nrhs", [(130, 1), (1000, 3), (2500, 1)])
def test_square_solve(cuda, n, nrhs):
    """QR::solve_mut: backward error at the n eps64 level, and the oracle's
    solution within the conditioning."""
    a = _mat(n, n, 600 + n, special=False)
    b = np.random.default_rng(601 + n).standard_normal((n, nrhs))
    qr, d = _factor(cuda, a, 0)
    x, info = _solve(cuda, qr, d, b)
    assert info == 0
    berr = np.abs(a @ x - b).max() / (np.abs(a).max() * np.abs(x).max() * n)
    assert berr <= 8 * EPS, (n, berr)
    if n <= 1000:
        ref_qr, ref_d = O.qr(a)
        xo, ok = O.qr_solve(ref_qr, ref_d, b)
        assert ok and np.abs(x - xo).max() <= 1e-8 * np.abs(xo).max()


def test_square_solve_stops_where_nalgebra_does(cuda):
    """A zero column j makes diag[j] zero; the backward substitution stops
    there (qr.rs:238-242): info = j + 1, nalgebra's false."""
    n, j = 300, 111
    a = _mat(n, n, 17, special=False)
    a[:, j] = 0.0
    qr, d = _factor(cuda, a, 0)
    assert d[j] == 0.0
    _, info = _solve(cuda, qr, d, np.ones((n, 1)))
    assert info == j + 1
    ref_qr, ref_d = O.qr(a)
    assert not O.qr_solve(ref_qr, ref_d, np.ones((n, 1)))[1]


@pytest.mark.parametrize("m,n", [(3000, 400), (700, 129)])
def test_least_squares(cuda, m, n):
    """A tall factor: the least-squares solution in the top n rows, as the
    oracle's (nalgebra-lapack qr_util.rs:167-239), with the normal equations
    of nalgebra-lapack's test (tests/linalg/qr.rs:53-61)."""
    a = _mat(m, n, 700 + m, special=False)
    b = np.random.default_rng(701 + m).standard_normal((m, 2))
    qr, d = _factor(cuda, a, 0)
    y, info = _solve(cuda, qr, d, b)
    x = y[:n]
    assert info == 0
    ref_qr, ref_d = O.qr(a)
    xo, info_o = O.qr_ls_solve(ref_qr, ref_d, b)
    assert info_o == 0 and np.abs(x - xo).max() <= 1e-9 * np.abs(xo).max()
    ne = a.T @ (a @ x - b)
    assert np.abs(ne).max() <= 1e-7 * np.abs(a.T @ b).max()


def test_mirror_large_and_wide(cuda):
    from nalgebra_gb300 import QR, DeviceMatrix

    a = _mat(100, 500, 11)  # benches/linalg/qr.rs: qr_decompose_100x500
    q = DeviceMatrix.from_numpy(a).qr(flags=FLAG_EXACT)
    ref_qr, ref_d = O.qr(a)
    assert q.large and np.array_equal(q.r(), O.qr_r(ref_qr, ref_d)) and not q.is_invertible()
    back = QR.from_json(q.to_json())
    assert np.array_equal(back.qr.to_numpy(), ref_qr)
    n = 200
    s = _mat(n, n, 12, special=False)
    qs = DeviceMatrix.from_numpy(s).qr()
    assert qs.large and qs.is_invertible()
    inv = qs.try_inverse().to_numpy()
    assert np.abs(s @ inv - np.eye(n)).max() <= 1e-10
    b = np.random.default_rng(13).standard_normal((n, 1))
    x = qs.solve(DeviceMatrix.from_numpy(b)).to_numpy()
    assert np.abs(s @ x - b).max() <= 1e-10 * np.abs(b).max() * n
    t = _mat(400, 60, 14, special=False)
    bt = np.random.default_rng(15).standard_normal((400, 1))
    xt = DeviceMatrix.from_numpy(t).qr().solve_least_squares(DeviceMatrix.from_numpy(bt)).to_numpy()
    assert np.allclose(xt, np.linalg.lstsq(t, bt, rcond=None)[0], rtol=1e-9, atol=1e-12)


def test_argument_errors(cuda):
    torch = cuda
    A = torch.zeros(16, dtype=torch.float64, device="cuda")
    with pytest.raises(NacuError):
        _lib.call("nacu_dqr", 4, 4, A.data_ptr(), 3, A.data_ptr(), 0, 0)  # lda < m
    with pytest.raises(NacuError):  # the large solve is FMA arithmetic only
        _lib.call("nacu_dqr_solve", 4, 4, 1, A.data_ptr(), 4, A.data_ptr(), A.data_ptr(), 4, A.data_ptr(),
                  A.data_ptr(), 128, FLAG_EXACT, 0)
