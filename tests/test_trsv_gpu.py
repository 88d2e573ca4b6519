"""GPU parity of the batched triangular solves (nacu_dtrsv_batched) against
the oracle's restatement of src/linalg/solve.rs: with NACU_FLAG_EXACT every
variant (lower / upper, plain / transposed, the with_diag form) is
bit-identical; the FMA form solves to 1e-12 relative; a zero diagonal reports
the index nalgebra stops at (its `false`)."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import FLAG_EXACT, _lib

pytestmark = pytest.mark.gpu
VARIANTS = [(False, False, None), (True, False, None), (False, True, None), (True, True, None),
            (False, False, 1.0), (False, False, -2.5)]


def _trsv(cuda, ts, bs, upper, trans, diag, flags):
    torch = cuda
    batch, n = len(ts), ts[0].shape[0]
    nrhs = bs[0].shape[1]
    T = torch.from_numpy(np.stack([t.ravel(order="F") for t in ts])).cuda()
    B = torch.from_numpy(np.stack([b.ravel(order="F") for b in bs])).cuda()
    info = torch.full((batch,), -7, dtype=torch.int32, device="cuda")
    _lib.call("nacu_dtrsv_batched", n, nrhs, int(upper), int(trans), int(diag is not None),
              float(diag if diag is not None else 0.0), T.data_ptr(), n * n, B.data_ptr(), n * nrhs, info.data_ptr(),
              batch, flags, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    x = B.cpu().numpy()
    return [x[k].reshape(nrhs, n).T for k in range(batch)], info.cpu().numpy()


def _mats(n, count, nrhs, seed):
    rng = np.random.default_rng(seed)
    ts = [rng.standard_normal((n, n)) + (n / 2) * np.diag(np.sign(rng.standard_normal(n)) + 2.0) for _ in range(count)]
    bs = [rng.standard_normal((n, nrhs)) for _ in range(count)]
    return ts, bs


@pytest.mark.parametrize("n", [1, 7, 8, 33, 64, 100, 128])
@pytest.mark.parametrize("variant", VARIANTS)
def test_exact_bit_identical_to_oracle(cuda, n, variant):
    upper, trans, diag = variant
    ts, bs = _mats(n, 3, 3, 1000 + n)
    xs, info = _trsv(cuda, ts, bs, upper, trans, diag, FLAG_EXACT)
    assert np.all(info == 0)
    for t, b, x in zip(ts, bs, xs):
        ref = O.triangular_solve(t, b, upper=upper, trans=trans, diag=diag)
        assert np.array_equal(x, ref), (n, variant)


@pytest.mark.parametrize("variant", VARIANTS[:5])
def test_fma_form_solves(cuda, variant):
    upper, trans, diag = variant
    n = 96
    ts, bs = _mats(n, 4, 2, 77)
    xs, info = _trsv(cuda, ts, bs, upper, trans, diag, 0)
    assert np.all(info == 0)
    for t, b, x in zip(ts, bs, xs):
        tri = np.triu(t) if upper else np.tril(t)
        if diag is not None:
            tri = np.tril(t, -1) + diag * np.eye(n)
        m = tri.T if trans else tri
        assert np.abs(m @ x - b).max() <= 1e-12 * np.abs(m).max() * max(1.0, np.abs(x).max()) * n


@pytest.mark.parametrize("upper,trans", [(False, False), (True, False), (False, True), (True, True)])
def test_zero_diagonal_reports_the_stopping_index(cuda, upper, trans):
    n = 40
    ts, bs = _mats(n, 2, 2, 5)
    ts[1][17, 17] = 0.0
    ts[1][31, 31] = -0.0
    _, info = _trsv(cuda, ts, bs, upper, trans, None, FLAG_EXACT)
    first = 31 if (upper != trans) else 17  # the sweep order: descending for upper / tr-lower
    assert info[0] == 0 and info[1] == first + 1
    assert O.triangular_solve(ts[1], bs[1], upper=upper, trans=trans) is None


def test_mirror_methods(cuda):
    """DeviceMatrix.{solve,tr_solve,ad_solve}_{lower,upper}_triangular: the
    oracle's results bit for bit in the EXACT form; None at a zero diagonal."""
    from nalgebra_gb300 import DeviceMatrix
    ts, bs = _mats(50, 1, 2, 9)
    t, b = ts[0], bs[0]
    m = DeviceMatrix.from_numpy(t)
    for meth, upper, trans in (("solve_lower_triangular", False, False), ("solve_upper_triangular", True, False),
                               ("tr_solve_lower_triangular", False, True), ("ad_solve_upper_triangular", True, True)):
        x = getattr(m, meth)(DeviceMatrix.from_numpy(b), FLAG_EXACT)
        assert np.array_equal(x.to_numpy(), O.triangular_solve(t, b, upper=upper, trans=trans)), meth
    z = t.copy()
    z[10, 10] = 0.0
    assert DeviceMatrix.from_numpy(z).solve_lower_triangular(DeviceMatrix.from_numpy(b)) is None
