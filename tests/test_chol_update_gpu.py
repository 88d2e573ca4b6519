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


# From 1024 factors up, rank_one_update runs 8 lanes per factor (4 factors per
# warp); 1030 leaves the last CTA and its last warp partly empty.  The same
# batch covers remove_column and insert_column at full size.  16 distinct
# factors and 37 distinct vectors are tiled over the batch; the oracle checks
# every 29th factor and the last six.
GROUP_BATCH = 1030


def _group_sample():
    return sorted(set(range(0, GROUP_BATCH, 29)) | set(range(GROUP_BATCH - 6, GROUP_BATCH)))


@pytest.mark.parametrize("n", [7, 64, 128])
@pytest.mark.parametrize("flags", [FLAG_EXACT, 0])
def test_rank_one_update_group_form(cuda, n, flags):
    torch = cuda
    mats, facs, rng = _factors(n, 16, 140 + n)
    xs = rng.standard_normal((37, n))
    sig = np.array([1.0, 0.5, 2.0, -0.2 / n])  # the downdate keeps A + sigma x x^T >= (n - 0.2 |x|^2 / n) I
    L = _dev(torch, [facs[k % 16] for k in range(GROUP_BATCH)])
    X = torch.from_numpy(np.stack([xs[k % 37] for k in range(GROUP_BATCH)])).cuda()
    S = torch.from_numpy(np.array([sig[k % 4] for k in range(GROUP_BATCH)])).cuda()
    _lib.call("nacu_dchol_rank1_update_batched", n, L.data_ptr(), n * n, X.data_ptr(), n, S.data_ptr(), GROUP_BATCH,
              flags, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = L.cpu().numpy()
    for k in _group_sample():
        g = got[k].reshape(n, n).T
        f, x, sg = facs[k % 16], xs[k % 37], sig[k % 4]
        if flags == FLAG_EXACT:
            assert np.array_equal(g, O.cholesky_rank_one_update(f, x, sg)), (n, k)
        else:
            lo = np.tril(g)
            target = mats[k % 16] + sg * np.outer(x, x)
            assert np.allclose(lo @ lo.T, target, rtol=1e-12, atol=1e-12 * np.abs(target).max()), (n, k)


@pytest.mark.parametrize("n,j", [(40, 39), (128, 5)])
def test_remove_column_group_form_exact(cuda, n, j):
    torch = cuda
    _, facs, _ = _factors(n, 16, 170 + n)
    L = _dev(torch, [facs[k % 16] for k in range(GROUP_BATCH)])
    out = torch.full((GROUP_BATCH, (n - 1) * (n - 1)), np.nan, dtype=torch.float64, device="cuda")
    _lib.call("nacu_dchol_remove_column_batched", n, L.data_ptr(), n * n, j, out.data_ptr(), (n - 1) * (n - 1),
              GROUP_BATCH, FLAG_EXACT, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    refs = [O.cholesky_remove_column(f, j) for f in facs]
    for k in _group_sample():
        assert np.array_equal(got[k].reshape(n - 1, n - 1).T, refs[k % 16]), (n, j, k)


@pytest.mark.parametrize("n,j", [(20, 0), (20, 20), (127, 60)])
@pytest.mark.parametrize("flags", [FLAG_EXACT, 0])
def test_insert_column_group_form(cuda, n, j, flags):
    torch = cuda
    mats, facs, rng = _factors(n, 16, 190 + n + j)
    cols = rng.standard_normal((37, n + 1))
    cols[:, j] = (cols * cols).sum(axis=1) + n + 1.0
    bad = facs[3].copy()
    if j > 2:
        bad[2, 2] = 0.0  # the lower solve meets it: info = 1 for the last factor only
    fl = [facs[k % 16] for k in range(GROUP_BATCH - 1)] + [bad]
    L = _dev(torch, fl)
    C = torch.from_numpy(np.stack([cols[k % 37] for k in range(GROUP_BATCH)])).cuda()
    out = torch.full((GROUP_BATCH, (n + 1) * (n + 1)), np.nan, dtype=torch.float64, device="cuda")
    info = torch.full((GROUP_BATCH,), -7, dtype=torch.int32, device="cuda")
    _lib.call("nacu_dchol_insert_column_batched", n, L.data_ptr(), n * n, j, C.data_ptr(), n + 1, out.data_ptr(),
              (n + 1) * (n + 1), info.data_ptr(), GROUP_BATCH, flags, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    inf = info.cpu().numpy()
    assert np.all(inf[:-1] == 0)
    assert inf[-1] == (1 if j > 2 else 0)
    got = out.cpu().numpy()
    for k in _group_sample():
        if k == GROUP_BATCH - 1 and j > 2:
            continue
        g = got[k].reshape(n + 1, n + 1).T
        ref = O.cholesky_insert_column(fl[k], j, cols[k % 37])
        if flags == FLAG_EXACT:
            assert np.array_equal(g, ref), (n, j, k)
        else:
            lo = np.tril(g)
            a = np.tril(fl[k]) @ np.tril(fl[k]).T
            target = np.insert(np.insert(a, j, 0.0, axis=0), j, 0.0, axis=1)
            target[:, j] = cols[k % 37]
            target[j, :] = cols[k % 37]
            assert np.allclose(lo @ lo.T, target, rtol=1e-12, atol=1e-12 * np.abs(target).max()), (n, j, k)


def test_mirror_cholesky_updates(cuda):
    """Cholesky.rank_one_update / remove_column / insert_column on the mirror's
    one-matrix Cholesky, against the oracle applied to the same factor."""
    from nalgebra_gb300 import DeviceMatrix

    n, j = 24, 7
    rng = np.random.default_rng(77)
    b = rng.standard_normal((n, n))
    a = b @ b.T + n * np.eye(n)
    ch = DeviceMatrix.from_numpy(a).cholesky(flags=FLAG_EXACT)
    f0 = ch.chol.to_numpy()
    x = rng.standard_normal(n)
    ch.rank_one_update(DeviceMatrix.from_numpy(x.reshape(n, 1)), 0.75)
    f1 = O.cholesky_rank_one_update(f0, x, 0.75)
    np.testing.assert_array_equal(ch.chol.to_numpy(), f1)
    ref_logdet = 0.0
    for v in np.diag(f1):
        ref_logdet += float(np.log(abs(v)))
    assert ch.ln_determinant() == ref_logdet * 2.0
    rm = ch.remove_column(j)
    np.testing.assert_array_equal(rm.chol.to_numpy(), O.cholesky_remove_column(f1, j))
    col = rng.standard_normal(n)
    col[j] = float(col @ col) + 2.0 * n
    ins = rm.insert_column(j, DeviceMatrix.from_numpy(col.reshape(n, 1)))
    np.testing.assert_array_equal(ins.chol.to_numpy(), O.cholesky_insert_column(rm.chol.to_numpy(), j, col))
    # the round trip reproduces the updated matrix with column j replaced
    a1 = np.tril(f1) @ np.tril(f1).T
    a1[:, j] = col
    a1[j, :] = col
    lo = np.tril(ins.chol.to_numpy())
    assert np.abs(lo @ lo.T - a1).max() <= 1e-12 * np.abs(a1).max()
