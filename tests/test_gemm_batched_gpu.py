"""GPU parity of the batched GEMM (nacu_dgemm_batched), the batched form of
nalgebra's `&a * &b` (src/base/ops.rs:566-570) and `Matrix::gemm`
(src/base/blas.rs:729-746): NACU_FLAG_EXACT bit-identical to the oracle's
restatement of gemm_uninit's gemv order (src/base/blas_uninit.rs:127-176,
320-332), which nalgebra itself uses when a dimension is <= 5 or the sizes are
static; the FMA form within k * eps64 * (|alpha||A||B| + |beta||C|) of the
compensated (Dot2) oracle; the reference's gemm example (blas.rs:713-727)."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import FLAG_EXACT, _lib
from tests.conftest import EPS64

pytestmark = pytest.mark.gpu


def _run(cuda, a, b, c, alpha, beta, flags):
    """a: (batch, m, k), b: (batch, k, n), c: (batch, m, n) row-major numpy;
    the device holds each product column-major."""
    torch = cuda
    batch, m, k = a.shape
    n = b.shape[2]
    cm = lambda x: torch.from_numpy(np.ascontiguousarray(np.transpose(x, (0, 2, 1)))).cuda()
    A, B, C = cm(a), cm(b), cm(c)
    _lib.call("nacu_dgemm_batched", m, n, k, float(alpha), A.data_ptr(), max(m, 1), m * k, B.data_ptr(), max(k, 1),
              k * n, float(beta), C.data_ptr(), max(m, 1), m * n, batch, flags, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return np.transpose(C.cpu().numpy(), (0, 2, 1))


SHAPES = [(1, 1, 1), (3, 4, 5), (5, 5, 5), (7, 3, 9), (2, 300, 5), (64, 64, 64), (65, 130, 17), (100, 100, 100),
          (13, 1, 70), (129, 3, 4)]


@pytest.mark.parametrize("m,n,k", SHAPES)
@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (1.5, -0.25), (-2.0, 1.0)])
def test_exact_form_is_nalgebras_gemv_order(cuda, m, n, k, alpha, beta):
    rng = np.random.default_rng(m * 1000 + n * 10 + k)
    batch = 5
    a = rng.standard_normal((batch, m, k))
    b = rng.standard_normal((batch, k, n))
    c = rng.standard_normal((batch, m, n))
    got = _run(cuda, a, b, c, alpha, beta, FLAG_EXACT)
    ref = O.gemm_gemv_order(alpha, a, b, beta, c)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("m,n,k", SHAPES)
def test_fma_form_against_dot2(cuda, m, n, k):
    rng = np.random.default_rng(7 + m + n + k)
    batch = 4
    alpha, beta = 0.75, 0.5
    a = rng.standard_normal((batch, m, k)) * 2.0 ** rng.integers(-20, 21, size=(batch, m, 1))
    b = rng.standard_normal((batch, k, n)) * 2.0 ** rng.integers(-20, 21, size=(batch, 1, n))
    c = rng.standard_normal((batch, m, n))
    got = _run(cuda, a, b, c, alpha, beta, 0)
    for s in range(batch):
        ref = O.gemm_dot2(alpha, a[s], b[s], beta, c[s])
        bound = (k + 2) * EPS64 * (abs(alpha) * np.abs(a[s]) @ np.abs(b[s]) + abs(beta) * np.abs(c[s]))
        assert np.all(np.abs(got[s] - ref) <= bound)


def test_zero_depth_beta_and_special_values(cuda):
    rng = np.random.default_rng(3)
    c = rng.standard_normal((2, 4, 3))
    a = np.zeros((2, 4, 0))
    b = np.zeros((2, 0, 3))
    for flags in (0, FLAG_EXACT):
        # gemv_uninit with ncols == 0: y = 0 when beta == 0, else y *= beta
        assert np.array_equal(_run(cuda, a, b, c, 1.0, 0.0, flags), np.zeros_like(c))
        assert np.array_equal(_run(cuda, a, b, c, 1.0, 0.5, flags), c * 0.5)
    # beta == 0: C is never read (NaN there does not leak); signed zeros and NaN in A follow nalgebra
    a = np.array([[[-0.0, 1.0], [np.nan, 2.0], [3.0, -0.0]]])
    b = np.array([[[0.0, 1.0], [-0.0, 2.0]]])
    cn = np.full((1, 3, 2), np.nan)
    got = _run(cuda, a, b, cn, 1.0, 0.0, FLAG_EXACT)
    ref = O.gemm_gemv_order(1.0, a, b, 0.0, np.zeros((1, 3, 2)))
    assert np.array_equal(np.signbit(got), np.signbit(ref)) and np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.array_equal(np.nan_to_num(got), np.nan_to_num(ref))


def test_reference_gemm_example(cuda):
    """src/base/blas.rs:713-727: mat1 = Matrix2x4::identity(); mat1.gemm(10.0,
    &mat2, &mat3, 5.0) equals mat2 * mat3 * 10 + mat1 * 5 (relative_eq).  The
    static sizes take the gemv order: the exact form matches the oracle bit
    for bit."""
    mat1 = np.eye(2, 4)[None]
    mat2 = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]])[None]
    mat3 = np.array([[0.1, 0.2, 0.3, 0.4], [0.5, 0.6, 0.7, 0.8], [0.9, 1.0, 1.1, 1.2]])[None]
    expected = mat2[0] @ mat3[0] * 10.0 + mat1[0] * 5.0
    got = _run(cuda, mat2, mat3, mat1, 10.0, 5.0, FLAG_EXACT)
    assert np.array_equal(got, O.gemm_gemv_order(10.0, mat2, mat3, 5.0, mat1))
    assert np.allclose(got[0], expected, rtol=1e-12, atol=0)


def test_argument_errors_and_mirror(cuda):
    torch = cuda
    L = _lib.load()
    assert L.nacu_dgemm_batched(-1, 1, 1, 1.0, None, 1, 1, None, 1, 1, 0.0, None, 1, 1, 1, 0, None) == -1
    assert L.nacu_dgemm_batched(2, 2, 2, 1.0, None, 2, 4, None, 2, 4, 0.0, None, 2, 4, -1, 0, None) == -15
    A = torch.zeros(8, dtype=torch.float64, device="cuda")
    assert L.nacu_dgemm_batched(2, 2, 2, 1.0, A.data_ptr(), 2, 3, A.data_ptr(), 2, 4, 0.0, A.data_ptr(), 2, 4, 2, 0,
                                None) == -7
    from nalgebra_gb300 import gemm_batched

    rng = np.random.default_rng(11)
    a = rng.standard_normal((6, 10, 12))
    b = rng.standard_normal((6, 12, 9))
    ta = torch.from_numpy(np.ascontiguousarray(np.transpose(a, (0, 2, 1)))).cuda()
    tb = torch.from_numpy(np.ascontiguousarray(np.transpose(b, (0, 2, 1)))).cuda()
    tc = torch.zeros((6, 9, 10), dtype=torch.float64, device="cuda")
    gemm_batched(tc, 1.0, ta, tb, 0.0, FLAG_EXACT)
    torch.cuda.synchronize()
    assert np.array_equal(np.transpose(tc.cpu().numpy(), (0, 2, 1)), O.gemm_gemv_order(1.0, a, b))
