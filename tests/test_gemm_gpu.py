"""GPU checks of the GEMM entry points against the compensated FP64 oracle.

nalgebra's Dyn f64 GEMM runs in the third-party matrixmultiply crate, whose
summation order is not pinned (no lockfile), so parity is tolerance-based
(an unpinned oracle: Dot2 compensated products, Ogita-Rump-Oishi 2005):
  FP64 form:  |C - C_ref| <= 2 k eps64 (|alpha| |A||B| + |beta| |C|) elementwise;
  split BF16 form (3 slices, FP32 accumulation): <= 1e-5 of (|A||B|) elementwise,
  1 slice <= 1e-2; and the beta == 0 rule (C never read) for both."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import _lib

pytestmark = pytest.mark.gpu
EPS64 = 2.220446049250313e-16


def _mats(m, n, k, scaled, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((m, k))
    b = rng.standard_normal((k, n))
    c = rng.standard_normal((m, n))
    if scaled:  # entries N(0,1) 2^k, k uniform in [-20, 20] per row of A / column of B
        a *= 2.0 ** rng.integers(-20, 21, size=(m, 1))
        b *= 2.0 ** rng.integers(-20, 21, size=(1, n))
    return a, b, c


def _run(cuda, kind, a, b, c, alpha, beta, slices=3):
    torch = cuda
    m, k = a.shape
    n = b.shape[1]
    d = lambda x: torch.from_numpy(np.asfortranarray(x).ravel(order="F")).cuda()
    A, B, Cm = d(a) if k else torch.zeros(1, dtype=torch.float64, device="cuda"), d(b) if k else torch.zeros(
        1, dtype=torch.float64, device="cuda"), d(c)
    s = torch.cuda.current_stream().cuda_stream
    if kind == "fp64":
        _lib.call("nacu_dgemm", m, n, k, alpha, A.data_ptr(), max(m, 1), B.data_ptr(), max(k, 1), beta,
                  Cm.data_ptr(), max(m, 1), s)
    else:
        L = _lib.load()
        wsb = L.nacu_gemm_split_workspace_bytes(m, n, k)
        ws = torch.empty(wsb + 1024, dtype=torch.uint8, device="cuda")
        wp = (ws.data_ptr() + 1023) // 1024 * 1024
        _lib.call("nacu_dgemm_split_bf16", m, n, k, alpha, A.data_ptr(), max(m, 1), B.data_ptr(), max(k, 1), beta,
                  Cm.data_ptr(), max(m, 1), slices, wp, wsb, s)
    torch.cuda.synchronize()
    if kind != "fp64":
        flag = C.c_int(0)
        _lib.load().nacu_split_gemm_error(C.byref(flag))
        assert flag.value == 0
    return Cm.cpu().numpy().reshape(n, m).T


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (37, 53, 71), (64, 64, 16), (256, 256, 256), (300, 129, 1000)])
@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (-0.5, 2.0)])
def test_dgemm_fp64(cuda, m, n, k, alpha, beta):
    a, b, c = _mats(m, n, k, True, m + n + k)
    got = _run(cuda, "fp64", a, b, c, alpha, beta)
    ref = O.gemm_dot2(alpha, a, b, beta, c)
    bound = 2 * k * EPS64 * (abs(alpha) * (np.abs(a) @ np.abs(b)) + abs(beta) * np.abs(c)) + 1e-300
    assert np.all(np.abs(got - ref) <= bound)


@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (300, 700, 500), (1, 3, 5), (256, 256, 1000)])
@pytest.mark.parametrize("scaled", [False, True])
def test_split_bf16_three_slices(cuda, m, n, k, scaled):
    a, b, c = _mats(m, n, k, scaled, 7 * m + n)
    got = _run(cuda, "split", a, b, c, 1.0, 0.0, 3)
    ref = O.gemm_dot2(1.0, a, b)
    scale = np.abs(a) @ np.abs(b)
    assert np.all(np.abs(got - ref) <= 1e-5 * scale)


def test_split_bf16_one_slice_and_alpha_beta(cuda):
    a, b, c = _mats(200, 300, 400, True, 3)
    got = _run(cuda, "split", a, b, c, 1.0, 0.0, 1)
    ref = O.gemm_dot2(1.0, a, b)
    assert np.all(np.abs(got - ref) <= 1e-2 * (np.abs(a) @ np.abs(b)))
    got = _run(cuda, "split", a, b, c, 2.0, -1.0, 3)
    ref = O.gemm_dot2(2.0, a, b, -1.0, c)
    assert np.all(np.abs(got - ref) <= 2e-5 * (np.abs(a) @ np.abs(b)) + 1e-15 * np.abs(c))


@pytest.mark.parametrize("kind", ["fp64", "split"])
def test_beta_zero_never_reads_c_and_k_zero(cuda, kind):
    """blas.rs:729-746: with beta == 0, C is not read (NaN in C stays out)."""
    a, b, c = _mats(70, 90, 33, False, 1)
    c[:] = np.nan
    got = _run(cuda, kind, a, b, c, 1.5, 0.0)
    assert np.all(np.isfinite(got))
    a0, b0, c0 = _mats(5, 6, 0, False, 2)
    got = _run(cuda, kind, a0, b0, c0, 1.0, 3.0)
    assert np.allclose(got, 3.0 * c0)


def test_split_extreme_scales_and_zero_rows(cuda):
    """Row/column scales far outside FP32's range (2^-600 .. 2^600 per row of A,
    2^-400 .. 2^400 per column of B) and an all-zero row: the epilogue rebuilds
    the FP64 result exactly from the FP32 accumulator and the two exponents."""
    rng = np.random.default_rng(12)
    m, n, k = 160, 272, 96
    a = rng.standard_normal((m, k)) * 2.0 ** rng.integers(-600, 601, size=(m, 1))
    b = rng.standard_normal((k, n)) * 2.0 ** rng.integers(-400, 401, size=(1, n))
    a[7, :] = 0.0
    got = _run(cuda, "split", a, b, np.zeros((m, n)), 1.0, 0.0, 3)
    ref = O.gemm_dot2(1.0, a, b)
    scale = np.abs(a) @ np.abs(b)
    assert np.all(np.abs(got - ref) <= 1e-5 * scale)
    assert np.all(got[7, :] == 0.0)
