"""GPU parity of the blocked multi-SM LU (one large matrix) against the CPU
oracle (nalgebra's unblocked LU::new and LU::solve): identical pivot
sequences on N(0,1) matrices (well-separated pivots), ||PA - LU||_F /
(||A||_F n eps) <= 10, backward error <= 10 n eps64, and the zero-column /
singular reporting."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import _lib
from tests.conftest import EPS64

pytestmark = pytest.mark.gpu


def _getrf(cuda, a, b=None):
    torch = cuda
    n = a.shape[0]
    A = torch.from_numpy(np.asfortranarray(a).ravel(order="F")).cuda()
    ipiv = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    info = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    L = _lib.load()
    ws = torch.empty(L.nacu_getrf_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    _lib.call("nacu_dgetrf", n, A.data_ptr(), n, ipiv.data_ptr(), info.data_ptr(), ws.data_ptr(), ws.numel(), s)
    x = None
    info2 = None
    if b is not None:
        X = torch.from_numpy(np.ascontiguousarray(b)).cuda()
        i2 = torch.full((1,), -7, dtype=torch.int32, device="cuda")
        _lib.call("nacu_dgetrs", n, A.data_ptr(), n, ipiv.data_ptr(), X.data_ptr(), i2.data_ptr(), ws.data_ptr(),
                  ws.numel(), s)
        torch.cuda.synchronize()
        x = X.cpu().numpy()
        info2 = int(i2.item())
    torch.cuda.synchronize()
    return A.cpu().numpy().reshape(n, n).T, ipiv.cpu().numpy()[:n], int(info.item()), x, info2


@pytest.mark.parametrize("n", [1, 2, 63, 64, 65, 200, 513, 1000])
def test_pivots_factors_and_solve_match_oracle(cuda, n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n))
    b = rng.standard_normal(n)
    lu, ipiv, info, x, info2 = _getrf(cuda, a, b)
    lu_o, ipiv_o, _ = O.lu(a)
    assert info == 0 and info2 == 0
    assert np.array_equal(ipiv, ipiv_o)
    assert O.lu_reconstruction(a, lu, ipiv) <= 10.0
    assert O.backward_error(a, x, b) <= 10 * n * EPS64
    x_o = O.lu_solve(lu_o, ipiv_o, b)
    cond = np.linalg.cond(a)
    assert np.linalg.norm(x - x_o) <= 1e3 * cond * EPS64 * np.linalg.norm(x_o)


def test_diagonally_dominant_large(cuda):
    n = 1500
    rng = np.random.default_rng(7)
    a = rng.standard_normal((n, n)) + n * np.eye(n)
    b = rng.standard_normal(n)
    lu, ipiv, info, x, _ = _getrf(cuda, a, b)
    assert info == 0 and np.array_equal(ipiv, np.arange(n))
    assert O.backward_error(a, x, b) <= n * EPS64


def test_zero_column_and_singular(cuda):
    n = 150
    rng = np.random.default_rng(3)
    a = rng.standard_normal((n, n))
    a[:, 70] = 0.0  # zero column: skipped (lu.rs:107-110), info = 71
    lu, ipiv, info, x, info2 = _getrf(cuda, a, rng.standard_normal(n))
    lu_o, ipiv_o, _ = O.lu(a)
    assert info == 71
    assert np.array_equal(ipiv, ipiv_o)
    assert info2 == 71  # U_70,70 == 0: the solve reports it


def test_grid_form_panels_large_n(cuda):
    """n = 6600: the first panels (rows above what a 16-CTA cluster holds in
    shared memory) take the grid-barrier form, the rest the cluster form.
    Pivots against LAPACK's partial pivoting (same rule: largest |x|, first
    on ties) and the backward error."""
    sla = pytest.importorskip("scipy.linalg")
    n = 6600
    rng = np.random.default_rng(66)
    a = rng.standard_normal((n, n))
    b = rng.standard_normal(n)
    lu, ipiv, info, x, info2 = _getrf(cuda, a, b)
    assert info == 0 and info2 == 0
    _, piv_ref = sla.lu_factor(a, check_finite=False)
    assert np.array_equal(ipiv, piv_ref)
    r = b - a @ x
    berr = np.abs(r).max() / (np.abs(a).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max())
    assert berr <= 10 * n * EPS64


def test_flag_wait_runs_out_and_reports(cuda):
    """The triangular solve's bounded flag wait (one CTA per 64-row block,
    each waiting on the ready flags of the blocks before it): with block 3's
    flag never raised and a short poll limit, the later blocks give up, info
    is -1000, the call returns, and the same factors then solve correctly on
    the same context -- the failure path, without faulting or hanging the GPU."""
    torch = cuda
    n = 1000  # 16 row blocks, all resident at once
    rng = np.random.default_rng(17)
    a = rng.standard_normal((n, n))
    b = rng.standard_normal(n)
    lu, ipiv, info, _, _ = _getrf(cuda, a)
    assert info == 0
    L = _lib.load()
    LU = torch.from_numpy(np.asfortranarray(lu).ravel(order="F")).cuda()
    P = torch.from_numpy(ipiv.astype(np.int32)).cuda()
    ws = torch.zeros(L.nacu_getrf_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    X = torch.from_numpy(b.copy()).cuda()
    inf = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    _lib.call("nacu_test_dgetrs_flag_timeout", n, LU.data_ptr(), n, P.data_ptr(), X.data_ptr(), inf.data_ptr(), 3,
              4096, ws.data_ptr(), ws.numel(), s)
    torch.cuda.synchronize()
    assert int(inf.item()) == -1000
    with pytest.raises(_lib.NacuError):  # a skip_block outside the row blocks is an argument error
        _lib.call("nacu_test_dgetrs_flag_timeout", n, LU.data_ptr(), n, P.data_ptr(), X.data_ptr(), inf.data_ptr(),
                  16, 4096, ws.data_ptr(), ws.numel(), s)
    X.copy_(torch.from_numpy(b))
    _lib.call("nacu_dgetrs", n, LU.data_ptr(), n, P.data_ptr(), X.data_ptr(), inf.data_ptr(), ws.data_ptr(),
              ws.numel(), s)
    torch.cuda.synchronize()
    assert int(inf.item()) == 0
    assert O.backward_error(a, X.cpu().numpy(), b) <= 10 * n * EPS64
