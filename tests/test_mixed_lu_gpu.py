"""GPU checks of the mixed-precision large solve (FP32 LU with BF16-split
tensor-core trailing updates, FP64 iterative refinement, FP64 fallback) on
A = U diag(s) V^T systems of prescribed condition: backward error
||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= n eps64 (recomputed
on the host), forward error against the oracle's FP64 LU solve within
cond * n * eps64, GMRES-IR where classical refinement stalls (u32 * cond >
1), and the FP64 fallback where FP32 cannot factor at all."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import _lib, workloads
from tests.conftest import EPS64

pytestmark = pytest.mark.gpu


def _berr(a, x, b):
    r = b - a @ x
    return np.abs(r).max() / (np.abs(a).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max())


def _solve(cuda, a, b, tol_units=1.0, max_iter=30):
    import ctypes as C

    torch = cuda
    n = a.shape[0]
    A = torch.from_numpy(np.asfortranarray(a).ravel(order="F")).cuda()
    B = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    X = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
    L = _lib.load()
    ws = torch.empty(L.nacu_gesv_mixed_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    it, berr, fb = C.c_int(-1), C.c_double(-1.0), C.c_int(-1)
    s = torch.cuda.current_stream().cuda_stream
    _lib.call("nacu_dgesv_mixed_ir", n, A.data_ptr(), n, B.data_ptr(), X.data_ptr(), tol_units, max_iter,
              C.byref(it), C.byref(berr), C.byref(fb), ws.data_ptr(), ws.numel(), s)
    torch.cuda.synchronize()
    assert np.array_equal(A.cpu().numpy(), np.asfortranarray(a).ravel(order="F")), "A must stay unchanged"
    return X.cpu().numpy(), it.value, berr.value, fb.value


@pytest.mark.parametrize("n,cond", [(256, 1e2), (640, 1e2), (1000, 1e5), (1536, 1e5), (777, 1e3), (778, 1e4),
                                    (128, 1e2), (132, 1e3)])
def test_refined_solution_meets_backward_error(cuda, n, cond):
    a, b = workloads.conditioned(n, cond, seed=n)
    x, iters, berr, fb = _solve(cuda, a, b)
    assert fb == 0, "FP32 refinement should converge at u32 * cond < 1"
    assert 1 <= iters <= 10
    host_berr = _berr(a, x, b)
    assert host_berr <= n * EPS64
    assert berr <= n * EPS64
    lu_o, ipiv_o, _ = O.lu(a)
    x_o = O.lu_solve(lu_o, ipiv_o, b)
    assert np.abs(x - x_o).max() <= cond * n * EPS64 * np.abs(x_o).max()


def test_ill_conditioned_reaches_fp64_target(cuda):
    """u32 * cond > 1: classical refinement cannot converge; GMRES-IR or the
    FP64 refactorization still delivers backward error <= n eps64."""
    n, cond = 512, 1e8
    a, b = workloads.conditioned(n, cond, seed=5)
    x, iters, berr, fb = _solve(cuda, a, b)
    assert fb in (1, 2)
    assert _berr(a, x, b) <= n * EPS64 and berr <= n * EPS64


def test_fp32_singular_matrix_falls_back(cuda):
    # entries below FP32's smallest subnormal in one column: FP32 sees a zero
    # column (info > 0) while FP64 factors the matrix
    n = 300
    rng = np.random.default_rng(11)
    a = rng.standard_normal((n, n))
    a[:, 17] *= 1e-60
    b = rng.standard_normal(n)
    x, iters, berr, fb = _solve(cuda, a, b)
    assert fb == 1 and iters == 0
    assert _berr(a, x, b) <= n * EPS64


def test_tolerance_and_iteration_cap(cuda):
    n = 400
    a, b = workloads.conditioned(n, 1e4, seed=3)
    # one classical step cannot reach 1e-3 n eps: with max_iter = 1 the driver
    # goes on with GMRES-IR, and to FP64 where that cannot reach it either
    x, iters, berr, fb = _solve(cuda, a, b, tol_units=1e-3, max_iter=1)
    assert iters >= 1 and fb in (1, 2)
    assert fb == 1 or berr <= 1e-3 * n * EPS64
    x2, iters2, berr2, fb2 = _solve(cuda, a, b, tol_units=100.0)
    assert fb2 == 0 and berr2 <= 100 * n * EPS64


def test_argument_errors(cuda):
    L = _lib.load()
    assert L.nacu_dgesv_mixed_ir(-1, None, 1, None, None, 1.0, 5, None, None, None, None, 0, None) == -1
    torch = cuda
    A = torch.zeros(16, dtype=torch.float64, device="cuda")
    ws = torch.empty(16, dtype=torch.uint8, device="cuda")
    rc = L.nacu_dgesv_mixed_ir(4, A.data_ptr(), 4, A.data_ptr(), A.data_ptr(), 1.0, 5, None, None, None,
                               ws.data_ptr(), ws.numel(), None)
    assert rc == -11


def test_mirror_large_lu_and_refined_solve(cuda):
    from nalgebra_gb300 import DeviceMatrix, gemm, solve_refined

    n = 300
    a, b = workloads.conditioned(n, 1e3, seed=21)
    lu = DeviceMatrix.from_numpy(a).lu()
    assert lu.large and lu.is_invertible()
    lu_o, ipiv_o, _ = O.lu(a)
    assert [p for p in lu.p()] == [(i, int(p)) for i, p in enumerate(ipiv_o) if p != i]
    x = lu.solve(DeviceMatrix.from_numpy(b.reshape(-1, 1))).to_numpy().ravel()
    assert _berr(a, x, b) <= 10 * n * EPS64
    xr, st = solve_refined(DeviceMatrix.from_numpy(a), DeviceMatrix.from_numpy(b.reshape(-1, 1)))
    assert not st["fallback"] and st["berr"] <= n * EPS64
    assert _berr(a, xr.to_numpy().ravel(), b) <= n * EPS64
    c = DeviceMatrix.from_numpy(np.zeros((n, 1)))
    gemm(c, 1.0, DeviceMatrix.from_numpy(a), xr, 0.0)
    assert np.allclose(c.to_numpy().ravel(), b, rtol=0, atol=1e-10 * np.abs(b).max())


@pytest.fixture(scope="module")
def config3_systems(cuda):
    """The mixed-LU workload at n = 4096: A = U diag(s) V^T with U, V from the
    QR of N(0,1) matrices and s log-uniform, cond 1e2 / 1e5 / 1e8, one RHS."""
    out = {}
    for cond in (1e2, 1e5, 1e8):
        A, b = workloads.conditioned_torch(4096, cond, seed=int(np.log10(cond)) + 4096)
        a = A.cpu().numpy().reshape(4096, 4096).T  # the device buffer is column-major
        out[cond] = (np.asfortranarray(a), b.cpu().numpy())
        del A, b
    return out


@pytest.mark.parametrize("cond", [1e2, 1e5, 1e8])
def test_config3_size_backward_error_and_fallback(cuda, config3_systems, cond):
    """n = 4096 at the three configured condition numbers: the backward error
    (residual by Dot2 on the host) is <= n eps64 for every condition number,
    FP32 refinement converges at 1e2 and 1e5 (u32 * cond < 1), and exactly the
    1e8 system (u32 * cond > 1, classical refinement diverges, too far for the
    FP32 preconditioner of GMRES-IR) takes the FP64 refactorization."""
    a, b = config3_systems[cond]
    n = a.shape[0]
    x, iters, berr, fb = _solve(cuda, a, b)
    assert fb == (1 if cond == 1e8 else 0)
    assert np.all(np.isfinite(x))
    host_berr = O.dense_backward_error(a.ravel(order="F"), n, x, b)
    assert host_berr <= n * EPS64
    assert berr <= n * EPS64


def test_config3_size_fp64_pivots_match_lapack(cuda, config3_systems):
    """The plain FP64 form at n = 4096 (nacu_dgetrf + nacu_dgetrs) on the
    cond-1e5 system: the same pivot sequence as LAPACK's partial pivoting
    (largest |x|, first on ties: nalgebra's icamax rule), ||PA - LU|| <=
    10 n eps and backward error <= 10 n eps64."""
    sla = pytest.importorskip("scipy.linalg")
    from tests.test_getrf_large_gpu import _getrf

    a, b = config3_systems[1e5]
    n = a.shape[0]
    lu, ipiv, info, x, info2 = _getrf(cuda, a, b)
    assert info == 0 and info2 == 0
    _, piv_ref = sla.lu_factor(a, check_finite=False)
    assert np.array_equal(ipiv, piv_ref)
    assert O.dense_backward_error(a.ravel(order="F"), n, x, b) <= 10 * n * EPS64


def test_gmres_ir_between_the_regimes(cuda):
    """n = 4096 at cond 1e7 (u32 * cond ~ 0.6): classical refinement stalls,
    GMRES-IR with the FP32 LU factors as the preconditioner (Carson & Higham
    2018) converges to backward error <= n eps64 without an FP64
    refactorization."""
    n, cond = 4096, 1e7
    A, bb = workloads.conditioned_torch(n, cond, seed=int(np.log10(cond)) + n)
    a = np.asfortranarray(A.cpu().numpy().reshape(n, n).T)
    b = bb.cpu().numpy()
    x, iters, berr, fb = _solve(cuda, a, b)
    assert fb == 2
    assert O.dense_backward_error(a.ravel(order="F"), n, x, b) <= n * EPS64 and berr <= n * EPS64
