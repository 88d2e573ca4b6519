"""GPU parity of the large triangular solve (nacu_dtrsv, one matrix of any
order) against the oracle's restatement of src/linalg/solve.rs:55-442, for
every variant (lower / upper, plain / transposed, with_diag): the FMA form
solves to 1e-12 relative of the oracle, only the named triangle is read (the
other holds NaN), a zero diagonal reports the index nalgebra stops at, and a
residual check covers n = 8192 (a 64-row block count that is not a multiple of
anything in the kernel, and a ragged last block at n = 4100)."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import FLAG_EXACT, NacuError, _lib

pytestmark = pytest.mark.gpu
VARIANTS = [(False, False, None), (True, False, None), (False, True, None), (True, True, None),
            (False, False, 1.0), (False, False, -2.5)]


def _tri(n, upper, seed):
    rng = np.random.default_rng(seed)
    t = rng.standard_normal((n, n)) / np.sqrt(n) + np.diag(rng.uniform(1.0, 2.0, n) * np.sign(rng.standard_normal(n)))
    keep = np.triu(np.ones((n, n), bool)) if upper else np.tril(np.ones((n, n), bool))
    return np.where(keep, t, np.nan)  # the other triangle must never be read


def _solve(torch, t, b, upper, trans, diag, flags=0):
    n, nrhs = b.shape
    T = torch.from_numpy(np.asfortranarray(t).ravel(order="F")).cuda()
    B = torch.from_numpy(np.asfortranarray(b).ravel(order="F")).cuda()
    info = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    ws = torch.empty(_lib.load().nacu_trsv_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    _lib.call("nacu_dtrsv", n, nrhs, int(upper), int(trans), int(diag is not None),
              float(diag if diag is not None else 0.0), T.data_ptr(), n, B.data_ptr(), n, info.data_ptr(),
              ws.data_ptr(), ws.numel(), flags, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return B.cpu().numpy().reshape(nrhs, n).T, int(info.item())


@pytest.mark.parametrize("n,nrhs", [(129, 1), (1000, 1), (1000, 3), (4100, 2)])
@pytest.mark.parametrize("variant", VARIANTS)
def test_matches_oracle(cuda, n, nrhs, variant):
    upper, trans, diag = variant
    t = _tri(n, upper, 300 + n + 7 * nrhs)
    b = np.random.default_rng(n + nrhs).standard_normal((n, nrhs))
    x, info = _solve(cuda, t, b, upper, trans, diag)
    ref = O.triangular_solve(np.nan_to_num(t, nan=0.0), b, upper=upper, trans=trans, diag=diag)
    assert info == 0 and ref is not None
    err = np.abs(x - ref).max() / np.abs(ref).max()
    assert err <= 1e-12, (n, nrhs, variant, err)


@pytest.mark.parametrize("variant", VARIANTS[:4])
def test_residual_8192(cuda, variant):
    torch = cuda
    upper, trans, _ = variant
    n = 8192
    t = np.nan_to_num(_tri(n, upper, 77), nan=0.0)
    b = np.random.default_rng(78).standard_normal((n, 1))
    x, info = _solve(torch, t, b, upper, trans, None)
    assert info == 0
    m = t.T if trans else t
    r = m @ x - b
    berr = np.abs(r).max() / (np.abs(m).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max())
    assert berr <= n * np.finfo(float).eps, (variant, berr)


@pytest.mark.parametrize("upper,trans", [(False, False), (True, False), (False, True), (True, True)])
def test_zero_diagonal_info(cuda, upper, trans):
    n = 700
    t = np.nan_to_num(_tri(n, upper, 91), nan=0.0)
    t[100, 100] = 0.0
    t[600, 600] = 0.0
    b = np.ones((n, 1))
    _, info = _solve(cuda, t, b, upper, trans, None)
    fwd = (not upper) != trans
    assert info == (101 if fwd else 601)  # nalgebra stops at the first zero in its solve order
    assert O.triangular_solve(t, b, upper=upper, trans=trans) is None


@pytest.mark.parametrize("upper,trans", [(False, False), (True, False), (False, True), (True, True)])
def test_short_last_block_after_a_zero_diagonal_solve(cuda, upper, trans):
    """A solve that meets a zero diagonal leaves inf and NaN in the kernel's
    shared memory; the next solve with a short last block (n = 129: one row)
    must not pick them up where the tile is zero (NaN * 0)."""
    n0 = 2000
    t0 = np.nan_to_num(_tri(n0, upper, 93), nan=0.0)
    t0[np.arange(0, n0, 50), np.arange(0, n0, 50)] = 0.0
    _, info = _solve(cuda, t0, np.ones((n0, 1)), upper, trans, None)
    assert info != 0
    n = 129
    t = _tri(n, upper, 94)
    b = np.random.default_rng(95).standard_normal((n, 2))
    x, info = _solve(cuda, t, b, upper, trans, None)
    ref = O.triangular_solve(np.nan_to_num(t, nan=0.0), b, upper=upper, trans=trans)
    assert info == 0 and np.isfinite(x).all()
    assert np.abs(x - ref).max() <= 1e-12 * np.abs(ref).max()


def test_with_diag_zero_leaves_b(cuda):
    n = 300
    t = np.nan_to_num(_tri(n, False, 5), nan=0.0)
    b = np.arange(n, dtype=np.float64).reshape(n, 1)
    x, info = _solve(cuda, t, b, False, False, 0.0)
    assert info == 1 and np.array_equal(x, b)  # solve.rs:115-117


def test_argument_errors(cuda):
    torch = cuda
    n = 200
    T = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    B = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = torch.empty(_lib.load().nacu_trsv_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    with pytest.raises(NacuError):  # EXACT is the batched form's
        _lib.call("nacu_dtrsv", n, 1, 0, 0, 0, 0.0, T.data_ptr(), n, B.data_ptr(), n, info.data_ptr(),
                  ws.data_ptr(), ws.numel(), FLAG_EXACT, s)
    with pytest.raises(NacuError):  # with_diag is lower, not transposed
        _lib.call("nacu_dtrsv", n, 1, 1, 0, 1, 1.0, T.data_ptr(), n, B.data_ptr(), n, info.data_ptr(),
                  ws.data_ptr(), ws.numel(), 0, s)
    with pytest.raises(NacuError):  # workspace too small
        _lib.call("nacu_dtrsv", n, 1, 0, 0, 0, 0.0, T.data_ptr(), n, B.data_ptr(), n, info.data_ptr(),
                  ws.data_ptr(), 4, 0, s)


def test_mirror_routes_large(cuda):
    from nalgebra_gb300 import DeviceMatrix

    n = 1000  # benches/linalg/solve.rs: solve_l_triangular_1000x1000
    t = np.nan_to_num(_tri(n, False, 13), nan=0.0)
    b = np.random.default_rng(14).standard_normal((n, 1))
    td = DeviceMatrix.from_numpy(t)
    x = td.solve_lower_triangular(DeviceMatrix.from_numpy(b)).to_numpy()
    assert np.abs(x - O.triangular_solve(t, b)).max() <= 1e-12 * np.abs(x).max()
    y = td.tr_solve_lower_triangular(DeviceMatrix.from_numpy(b)).to_numpy()
    assert np.abs(y - O.triangular_solve(t, b, trans=True)).max() <= 1e-12 * np.abs(y).max()
