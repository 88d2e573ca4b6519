"""GPU parity of the batched Cholesky factor updates against the oracle's
restatement of src/linalg/cholesky.rs:277-449: rank_one_update (update and
downdate), remove_column and insert_column, bit-identical with
NACU_FLAG_EXACT (the factors' strict upper parts included, copied as nalgebra
copies its views); the FMA form reproduces the updated matrix."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import FLAG_EXACT, _lib

pytestmark = pytest.mark.gpu


def _factors(n, count, seed):
    rng = np.random.default_rng(seed)
    mats, facs = [], []
    for _ in range(count):
        b = rng.standard_normal((n, n))
        a = b @ b.T + n * np.eye(n)
        l, info = O.cholesky(a)
        assert info == 0
        mats.append(a)
        facs.append(np.asfortranarray(l))
    return mats, facs, rng


def _dev(cuda, arrs):
    return cuda.from_numpy(np.stack([np.asarray(a).ravel(order="F") for a in arrs])).cuda()


@pytest.mark.parametrize("n", [1, 5, 33, 64, 128])
@pytest.mark.parametrize("flags", [FLAG_EXACT, 0])
def test_rank_one_update(cuda, n, flags):
    torch = cuda
    mats, facs, rng = _factors(n, 4, 40 + n)
    xs = [rng.standard_normal(n) for _ in range(4)]
    sig = np.array([1.0, 2.5, -0.3 / max(1.0, float(np.dot(xs[2], xs[2])) / n), 0.0])
    L = _dev(torch, facs)
    X = _dev(torch, xs)
    S = torch.from_numpy(sig).cuda()
    _lib.call("nacu_dchol_rank1_update_batched", n, L.data_ptr(), n * n, X.data_ptr(), n, S.data_ptr(), 4, flags,
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = L.cpu().numpy()
    for k in range(4):
        g = got[k].reshape(n, n).T
        ref = O.cholesky_rank_one_update(facs[k], xs[k], sig[k])
        if flags == FLAG_EXACT:
            assert np.array_equal(g, ref), (n, k)
        else:
            lo = np.tril(g)
            target = mats[k] + sig[k] * np.outer(xs[k], xs[k])
            assert np.allclose(lo @ lo.T, target, rtol=1e-12, atol=1e-12 * np.abs(target).max()), (n, k)


@pytest.mark.parametrize("n,j", [(2, 0), (9, 0), (9, 4), (9, 8), (64, 31), (128, 127)])
def test_remove_column_exact(cuda, n, j):
    torch = cuda
    mats, facs, _ = _factors(n, 3, 70 + n + j)
    L = _dev(torch, facs)
    out = torch.full((3, (n - 1) * (n - 1)), np.nan, dtype=torch.float64, device="cuda")
    _lib.call("nacu_dchol_remove_column_batched", n, L.data_ptr(), n * n, j, out.data_ptr(), (n - 1) * (n - 1), 3,
              FLAG_EXACT, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    for k in range(3):
        assert np.array_equal(got[k].reshape(n - 1, n - 1).T, O.cholesky_remove_column(facs[k], j)), (n, j, k)


@pytest.mark.parametrize("n,j", [(0, 0), (1, 0), (1, 1), (8, 0), (8, 3), (8, 8), (63, 20), (127, 127)])
def test_insert_column_exact(cuda, n, j):
    torch = cuda
    mats, facs, rng = _factors(n, 3, 90 + n + j) if n else ([], [np.zeros((0, 0))] * 3, np.random.default_rng(0))
    cols = []
    for k in range(3):
        c = rng.standard_normal(n + 1)
        c[j] = float(np.dot(c, c)) + n + 1.0  # keeps the bordered matrix SPD
        cols.append(c)
    L = _dev(torch, facs) if n else torch.zeros((3, 1), dtype=torch.float64, device="cuda")
    C = _dev(torch, cols)
    out = torch.full((3, (n + 1) * (n + 1)), np.nan, dtype=torch.float64, device="cuda")
    info = torch.full((3,), -7, dtype=torch.int32, device="cuda")
    _lib.call("nacu_dchol_insert_column_batched", n, L.data_ptr(), n * n, j, C.data_ptr(), n + 1, out.data_ptr(),
              (n + 1) * (n + 1), info.data_ptr(), 3, FLAG_EXACT, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.all(info.cpu().numpy() == 0)
    got = out.cpu().numpy()
    for k in range(3):
        ref = O.cholesky_insert_column(facs[k], j, cols[k])
        assert np.array_equal(got[k].reshape(n + 1, n + 1).T, ref), (n, j, k)


def test_insert_column_zero_diagonal_reports_info(cuda):
    torch = cuda
    n, j = 6, 4
    _, facs, rng = _factors(n, 1, 5)
    f = facs[0].copy()
    f[2, 2] = 0.0
    L = _dev(torch, [f])
    C = _dev(torch, [rng.standard_normal(n + 1)])
    out = torch.zeros((1, (n + 1) ** 2), dtype=torch.float64, device="cuda")
    info = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    _lib.call("nacu_dchol_insert_column_batched", n, L.data_ptr(), n * n, j, C.data_ptr(), n + 1, out.data_ptr(),
              (n + 1) ** 2, info.data_ptr(), 1, FLAG_EXACT, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(info.item()) == 1
    assert O.cholesky_insert_column(f, j, np.ones(n + 1)) is None
