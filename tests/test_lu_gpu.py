"""GPU parity of the batched LU (factor, pivots, fused solve) against the CPU
oracle, through the C ABI.

Bar (from the workload definition): identical pivot sequences; with
NACU_FLAG_EXACT the factors and solutions are bit-identical to nalgebra's
arithmetic; in the default FMA form ||PA - LU||_F / (||A||_F n eps) <= 10 and
backward error <= 10 n eps64."""
import os

import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import FLAG_EXACT, DeviceBatch, DeviceMatrix, _lib
from nalgebra_gb300 import workloads as W
from tests.conftest import EPS64

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz")


def _gesv(cuda, a_colmaj, b_colmaj, n, nrhs, flags=0, mode="gesv"):
    torch = cuda
    batch = a_colmaj.shape[0]
    A = torch.from_numpy(np.ascontiguousarray(a_colmaj)).cuda()
    B = torch.from_numpy(np.ascontiguousarray(b_colmaj)).cuda()
    ipiv = torch.full((batch * max(n, 1),), -7, dtype=torch.int32, device="cuda")
    info = torch.full((batch,), -7, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    if mode == "gesv":
        _lib.call("nacu_dgesv_batched", n, nrhs, A.data_ptr(), n * n, ipiv.data_ptr(), B.data_ptr(), n * nrhs,
                  info.data_ptr(), batch, flags, s)
    else:
        _lib.call("nacu_dgetrf_batched", n, A.data_ptr(), n * n, ipiv.data_ptr(), info.data_ptr(), batch, flags, s)
        _lib.call("nacu_dgetrs_batched", n, nrhs, A.data_ptr(), n * n, ipiv.data_ptr(), B.data_ptr(), n * nrhs,
                  info.data_ptr(), batch, flags, s)
    torch.cuda.synchronize()
    return (A.cpu().numpy(), ipiv.cpu().numpy().reshape(batch, max(n, 1))[:, :n], B.cpu().numpy(),
            info.cpu().numpy())


@pytest.mark.parametrize("mode", ["gesv", "getrf+getrs"])
def test_exact_mode_bit_identical_to_oracle_golden(cuda, mode):
    with np.load(GOLD) as z:
        for n in [1, 2, 5, 6, 16, 33, 64]:
            for kind in ("dom", "piv"):
                key = f"lu_n{n}_{kind}"
                a = z[key + "_a"]
                b = z[key + "_b"]
                lu, ipiv, x, info = _gesv(cuda, a.ravel(order="F")[None], b.ravel(order="F")[None], n, 2,
                                          FLAG_EXACT, mode)
                assert info[0] == 0
                assert np.array_equal(ipiv[0], z[key + "_ipiv"]), key
                assert np.array_equal(lu[0].reshape(n, n).T, z[key + "_lu"]), key
                assert np.array_equal(x[0].reshape(2, n).T, z[key + "_x"]), key


def test_dominant_workload_parity_fma(cuda):
    """The 64 x 64, A + 64 I workload (a slice of the 4096-system batch)."""
    n = 64
    a, b = W.dense_lu(512, n, 1, seed=0)
    lu, ipiv, x, info = _gesv(cuda, a, b, n, 1)
    lu_o, ipiv_o, x_o, info_o = O.gesv_batched(a, b, n)
    assert np.all(info == 0) and np.all(info_o == 0)
    assert np.array_equal(ipiv, ipiv_o)
    worst_rec, worst_be = 0.0, 0.0
    for s in range(0, 512, 7):
        m = W.dense_lu_matrix(a[s], n)
        worst_rec = max(worst_rec, O.lu_reconstruction(m, lu[s].reshape(n, n).T, ipiv[s]))
        worst_be = max(worst_be, O.backward_error(m, x[s], b[s]))
    assert worst_rec <= 10.0
    assert worst_be <= 10 * n * EPS64
    assert np.allclose(x, x_o, rtol=1e-11, atol=1e-13)


def test_pivoting_inputs_pivots_match(cuda):
    """Non-dominant N(0,1) matrices: swaps on most steps.  With FMA the
    elimination values can differ in the last bits, so pivots could only
    differ on near-ties; with these well-separated seeded inputs they must match
    exactly, and in EXACT form always."""
    n = 48
    a, b = W.dense_lu(256, n, 3, shift=0.0, seed=11)
    lu_o, ipiv_o, x_o, _ = O.gesv_batched(a, b, n)
    for flags in (0, FLAG_EXACT):
        lu, ipiv, x, info = _gesv(cuda, a, b, n, 3, flags)
        assert np.all(info == 0)
        assert np.array_equal(ipiv, ipiv_o)
        if flags:
            assert np.array_equal(lu, lu_o) and np.array_equal(x, x_o)
        else:
            for s in range(0, 256, 9):
                m = W.dense_lu_matrix(a[s], n)
                assert O.lu_reconstruction(m, lu[s].reshape(n, n).T, ipiv[s]) <= 10.0
                assert O.backward_error(m, x[s], b[s]) <= 10 * n * EPS64


@pytest.mark.parametrize("n", [1, 2, 5, 6, 7, 31, 32, 33, 100, 128])
def test_sizes_and_many_rhs(cuda, n):
    a, b = W.dense_lu(20, n, 16, shift=0.5 * n, seed=n)
    lu, ipiv, x, info = _gesv(cuda, a, b, n, 16, FLAG_EXACT)
    lu_o, ipiv_o, x_o, info_o = O.gesv_batched(a, b, n)
    assert np.array_equal(info, info_o)
    assert np.array_equal(ipiv, ipiv_o)
    assert np.array_equal(lu, lu_o)
    assert np.array_equal(x, x_o)


def test_singular_and_nan_edge_cases(cuda):
    n = 6
    rng = np.random.default_rng(9)
    mats = []
    m0 = rng.standard_normal((n, n)); m0[:, 2] = 0.0  # zero column: skipped, info = 3
    m1 = np.zeros((n, n))                              # all zero: info = 1
    m2 = rng.standard_normal((n, n)); m2[0, 0] = np.nan  # NaN at the first pivot position
    m3 = rng.standard_normal((n, n)); m3[3, 0] = np.nan  # NaN below: ignored by icamax
    m4 = np.ones((n, n)); m4[np.arange(n), np.arange(n)] = 2.0  # exact ties in |x|
    mats = [m0, m1, m2, m3, m4]
    a = np.stack([m.ravel(order="F") for m in mats])
    b = rng.standard_normal((len(mats), n))
    for flags in (0, FLAG_EXACT):
        lu, ipiv, x, info = _gesv(cuda, a, b, n, 1, flags)
        for s, m in enumerate(mats):
            lu_o, ipiv_o, _ = O.lu(m)
            assert np.array_equal(ipiv[s], ipiv_o), s
            diag = np.diag(lu_o)
            expect = int(np.argmax(diag == 0) + 1) if np.any(diag == 0) else 0
            assert info[s] == expect, s
            if flags:
                assert np.array_equal(lu[s].reshape(n, n).T, lu_o, equal_nan=True), s
    assert info[0] == 3 and info[1] == 1


def test_device_matrix_api_mirrors_nalgebra(cuda):
    """m.lu(), lu.solve(&b), lu.determinant(), lu.p() on the known answers
    (tests/linalg/lu.rs:5-39)."""
    m = np.array([[0.0, -1.0, 2.0], [-1.0, 2.0, -1.0], [2.0, -1.0, 0.0]])
    lu = DeviceMatrix.from_numpy(m).lu(flags=FLAG_EXACT)
    assert lu.determinant() == -4.0
    assert lu.p() == [(0, 2)]
    b = DeviceMatrix.from_numpy(np.array([1.0, 2.0, 3.0]))
    x = lu.solve(b)
    assert x is not None and np.allclose(m @ x.to_numpy()[:, 0], [1, 2, 3], atol=1e-12)
    lu2 = DeviceMatrix.from_numpy(np.array([[2.0, -1, 0], [-1, 2, -1], [0, -1, 2]])).lu()
    assert lu2.determinant() == 4.0
    sing = DeviceMatrix.from_numpy(np.zeros((3, 3))).lu()
    assert lu2.is_invertible() and not sing.is_invertible()
    assert sing.solve(b) is None


def test_device_batch_lazy_fused(cuda):
    n = 32
    a, b = W.dense_lu(64, n, 2, seed=5)
    batch = DeviceBatch.from_numpy([W.dense_lu_matrix(r, n) for r in a])
    rhs = DeviceBatch.from_numpy([r.reshape(2, n).T for r in b])
    lub = batch.lu(flags=FLAG_EXACT)
    x = lub.solve(rhs)
    lu_o, ipiv_o, x_o, _ = O.gesv_batched(a, b, n)
    got = np.stack([xx.T.ravel() for xx in x.to_numpy()])
    assert np.array_equal(got, x_o)
    assert np.array_equal(lub.pivots(), ipiv_o)
    x2 = lub.solve(rhs)  # second solve uses the stored factors
    assert np.array_equal(np.stack([xx.T.ravel() for xx in x2.to_numpy()]), x_o)


def _getri(cuda, a_colmaj, n, flags=0):
    torch = cuda
    batch = a_colmaj.shape[0]
    A = torch.from_numpy(np.ascontiguousarray(a_colmaj)).cuda()
    inv = torch.full((batch, n * n), np.nan, dtype=torch.float64, device="cuda")
    ipiv = torch.full((batch * max(n, 1),), -7, dtype=torch.int32, device="cuda")
    info = torch.full((batch,), -7, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    _lib.call("nacu_dgetrf_batched", n, A.data_ptr(), n * n, ipiv.data_ptr(), info.data_ptr(), batch, flags, s)
    _lib.call("nacu_dgetri_batched", n, A.data_ptr(), n * n, ipiv.data_ptr(), inv.data_ptr(), n * n, info.data_ptr(),
              batch, flags, s)
    torch.cuda.synchronize()
    return inv.cpu().numpy(), info.cpu().numpy()


@pytest.mark.parametrize("n", [5, 17, 33, 64, 100, 128])
def test_try_inverse_exact_bit_identical_to_oracle(cuda, n):
    """nacu_dgetri_batched (LU::try_inverse, lu.rs:266-297) in EXACT form
    equals the oracle's identity-then-solve_mut bit for bit."""
    rng = np.random.default_rng(300 + n)
    mats = [rng.standard_normal((n, n)) + (float(n) if k % 2 else 0.0) * np.eye(n) for k in range(3)]
    inv, info = _getri(cuda, np.stack([m.ravel(order="F") for m in mats]), n, FLAG_EXACT)
    assert np.all(info == 0)
    for k, m in enumerate(mats):
        lu, ipiv, _ = O.lu(m)
        ref = O.lu_try_inverse(lu, ipiv)
        assert np.array_equal(inv[k].reshape(n, n).T, ref), (n, k)


def test_try_inverse_known_answer_and_singular(cuda):
    """tests/linalg/inverse.rs:62-81 (relative 1e-4) through the GPU path, in
    the FMA form; a singular matrix reports info (nalgebra's None)."""
    import json
    with open(os.path.join(os.path.dirname(__file__), "golden", "reference_known_answers.json")) as f:
        k = json.load(f)["inverse_matrix5"]
    m = np.array(k["rows"], dtype=np.float64)
    sing = np.array([[1.0, 2.0, 3.0, 0.0, 1.0], [2.0, 4.0, 6.0, 0.0, 2.0], [0.0, 1.0, 1.0, 1.0, 0.0],
                     [1.0, 0.0, 2.0, 3.0, 1.0], [0.0, 0.0, 1.0, 1.0, 1.0]])
    sing[:, 3] = 0.0  # an exactly zero column: skipped by the LU (lu.rs:107-110), U_33 = 0
    inv, info = _getri(cuda, np.stack([m.ravel(order="F"), sing.ravel(order="F")]), 5)
    exp = np.array(k["expected_inverse_rows"])
    got = inv[0].reshape(5, 5).T
    d = np.abs(got - exp)
    assert np.all((d <= np.finfo(np.float64).eps) | (d <= k["max_relative"] * np.maximum(np.abs(got), np.abs(exp))))
    assert info[0] == 0 and info[1] > 0


def test_try_inverse_fma_workload(cuda):
    """The 64 x 64 workload matrices: A Ainv = I to 1e-12 relative (FMA form)."""
    n = 64
    a, _ = W.dense_lu(16, n, 1, seed=9)
    inv, info = _getri(cuda, a, n)
    assert np.all(info == 0)
    for k in range(16):
        m = a[k].reshape(n, n).T
        r = m @ inv[k].reshape(n, n).T - np.eye(n)
        assert np.abs(r).max() <= 1e-12 * n, k


def test_mirror_try_inverse(cuda):
    """LU.try_inverse / LUBatch.try_inverse in the mirror."""
    rng = np.random.default_rng(77)
    m = rng.standard_normal((20, 20)) + 20 * np.eye(20)
    inv = DeviceMatrix.from_numpy(m).lu().try_inverse()
    assert inv is not None and np.abs(m @ inv.to_numpy() - np.eye(20)).max() < 1e-12
    z = m.copy()
    z[:, 5] = 0.0
    assert DeviceMatrix.from_numpy(z).lu().try_inverse() is None
    mats = [rng.standard_normal((9, 9)) + 9 * np.eye(9) for _ in range(5)]
    invs, info = DeviceBatch.from_numpy(mats).lu().try_inverse()
    assert np.all(info.to_numpy() == 0)
    for a, x in zip(mats, invs.to_numpy()):
        assert np.abs(a @ x - np.eye(9)).max() < 1e-12
