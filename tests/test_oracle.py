"""The CPU oracle (C++ restatement of nalgebra's loops) pinned against the
reference's own known-answer tests and property tests, and cross-checked with
scipy's LAPACK.  Runs without a GPU."""
import json
import os

import numpy as np
import pytest
import scipy.linalg as sl

import oracle as O
from tests.conftest import EPS64

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _known():
    with open(os.path.join(GOLD, "reference_known_answers.json")) as f:
        return json.load(f)


def _rows(rows):
    return np.array([[np.nan if v == "nan" else v for v in r] for r in rows], dtype=np.float64)


def _unpack(lu, ipiv):
    n = lu.shape[0]
    l = np.tril(lu, -1) + np.eye(n)
    u = np.triu(lu)
    return l, u


def _inv_permute_rows(m, ipiv):
    """PermutationSequence::inv_permute_rows (permutation_sequence.rs:108-116)."""
    m = m.copy()
    for i in reversed(range(len(ipiv))):
        p = ipiv[i]
        if p != i:
            m[[i, p]] = m[[p, i]]
    return m


@pytest.mark.parametrize("case", ["lu_simple", "lu_simple_with_pivot"])
def test_lu_known_answers(case):
    k = _known()[case]
    m = _rows(k["rows"])
    lu, ipiv, ln = O.lu(m)
    assert O.lu_determinant(lu, ln) == k["determinant"]  # exact, as assert_eq! in the reference
    l, u = _unpack(lu, ipiv)
    rec = _inv_permute_rows(l @ u, ipiv)
    assert np.allclose(rec, m, atol=k["reconstruction_epsilon"], rtol=0)
    if case == "lu_simple_with_pivot":
        assert ln == 1 and list(ipiv) == [2, 1, 2]


def test_cholesky_with_substitute_known_answer():
    k = _known()["cholesky_with_substitute"]
    m = _rows(k["rows"])
    _, info = O.cholesky(m)
    assert info != 0  # None
    _, info2 = O.cholesky(m, substitute=k["substitute"])
    assert info2 == 0  # Some


def test_dot_eight_accumulators():
    """blas.rs:96-165: blocks of 8 into 8 accumulators, combined (0+4),(1+5),
    (2+6),(3+7), then the tail."""
    rng = np.random.default_rng(3)
    for n in [0, 1, 7, 8, 9, 16, 23, 64, 100]:
        x = rng.standard_normal(n)
        y = rng.standard_normal(n)
        acc = [0.0] * 8
        i = 0
        while n - i >= 8:
            for k in range(8):
                acc[k] += x[i + k] * y[i + k]
            i += 8
        res = 0.0
        res += acc[0] + acc[4]
        res += acc[1] + acc[5]
        res += acc[2] + acc[6]
        res += acc[3] + acc[7]
        for k in range(i, n):
            res += x[k] * y[k]
        assert O.dot(x, y) == res


def _pure_python_lu(a):
    """Independent pure-Python restatement of LU::new for tiny matrices."""
    a = [list(map(float, r)) for r in a]
    n = len(a)
    ipiv = list(range(n))
    for i in range(n):
        piv, best = i, abs(a[i][i])
        for r in range(i + 1, n):
            if abs(a[r][i]) > best:
                best, piv = abs(a[r][i]), r
        diag = a[piv][i]
        if diag == 0.0:
            continue
        ipiv[i] = piv
        a[i], a[piv] = a[piv], a[i]
        inv = 1.0 / diag
        for r in range(i + 1, n):
            a[r][i] = a[r][i] * inv
        for c in range(i + 1, n):
            p = a[i][c]
            for r in range(i + 1, n):
                a[r][c] = (-p) * a[r][i] + a[r][c]
    return np.array(a), np.array(ipiv)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 6, 9])
def test_lu_matches_pure_python_restatement_bitwise(n):
    rng = np.random.default_rng(n)
    a = rng.uniform(-100, 100, size=(n, n))  # PROPTEST_F64 range, tests/proptest/mod.rs:19-20
    lu, ipiv, _ = O.lu(a)
    lu2, ipiv2 = _pure_python_lu(a)
    assert np.array_equal(ipiv, ipiv2)
    assert np.array_equal(lu, lu2)


@pytest.mark.parametrize("n", [1, 4, 13, 20])
def test_lu_properties(n):
    """tests/linalg/lu.rs:54-105: reconstruction 1e-7, solve residual 1e-6,
    and scipy's partial pivoting picks the same rows."""
    rng = np.random.default_rng(100 + n)
    a = rng.uniform(-100, 100, size=(n, n))
    lu, ipiv, _ = O.lu(a)
    l, u = _unpack(lu, ipiv)
    assert np.allclose(_inv_permute_rows(l @ u, ipiv), a, atol=1e-7 * np.abs(a).max())
    b = rng.uniform(-100, 100, size=(n, 3))
    x = O.lu_solve(lu, ipiv, b)
    assert np.allclose(a @ x, b, atol=1e-6 * max(1.0, np.abs(b).max()))
    _, piv_scipy = sl.lu_factor(a)
    assert np.array_equal(piv_scipy, ipiv)
    assert O.lu_reconstruction(a, lu, ipiv) <= 10.0


def test_lu_zero_column_is_skipped_and_solve_fails():
    a = np.array([[0.0, 1.0, 2.0], [0.0, 3.0, 4.0], [0.0, 5.0, 7.0]])
    lu, ipiv, _ = O.lu(a)
    assert ipiv[0] == 0 and lu[0, 0] == 0.0  # lu.rs:107-110
    assert O.lu_solve(lu, ipiv, np.ones(3)) is None


@pytest.mark.parametrize("n", [1, 2, 8, 20, 37])
def test_cholesky_properties(n):
    """tests/linalg/cholesky.rs:35-77 and the log-determinant."""
    rng = np.random.default_rng(200 + n)
    b = rng.standard_normal((n, n))
    a = b @ b.T + n * np.eye(n)
    l, info = O.cholesky(a)
    assert info == 0
    L = np.tril(l)
    assert np.allclose(L @ L.T, a, atol=1e-7 * np.abs(a).max())
    assert np.array_equal(np.triu(l, 1), np.triu(a, 1))  # upper triangle untouched
    rhs = rng.standard_normal((n, 4))
    x = O.cholesky_solve(l, rhs)
    assert np.allclose(a @ x, rhs, atol=1e-7 * max(1, np.abs(rhs).max()))
    assert O.backward_error(a, x, rhs) <= n * EPS64
    assert abs(O.cholesky_ln_determinant(l) - np.linalg.slogdet(a)[1]) <= 1e-12 * max(1, abs(np.linalg.slogdet(a)[1]))
    assert np.allclose(L, np.linalg.cholesky(a), rtol=1e-12, atol=1e-12)


def test_cholesky_not_spd():
    a = np.array([[1.0, 2.0], [2.0, 1.0]])
    _, info = O.cholesky(a)
    assert info == 2
    _, info = O.cholesky(np.array([[-1.0]]))
    assert info == 1
    _, info = O.cholesky(np.array([[np.nan]]))
    assert info == 1


@pytest.mark.parametrize("m,n", [(3, 3), (5, 3), (3, 5), (40, 7), (300, 64)])
def test_qr_properties(m, n):
    """tests/linalg/qr.rs:15-52: Q R = A and Q orthogonal within 1e-7."""
    rng = np.random.default_rng(300 + m + n)
    a = rng.uniform(-100, 100, size=(m, n))
    qr, diag = O.qr(a)
    r = O.qr_r(qr, diag)
    qt = O.qr_q_tr_mul(qr, diag, np.eye(m))  # Q^T
    q = qt.T[:, : min(m, n)]
    assert np.allclose(q @ r, a, atol=1e-7 * np.abs(a).max())
    assert np.allclose(q.T @ q, np.eye(min(m, n)), atol=1e-7)
    assert np.all(np.diag(r) >= 0)


@pytest.mark.parametrize("m,n", [(5, 3), (20, 20), (128, 64), (512, 64)])
def test_qr_least_squares_normal_equations(m, n):
    """nalgebra-lapack/tests/linalg/qr.rs:46-61: A^T A x = A^T b within 1e-5."""
    rng = np.random.default_rng(400 + m)
    a = rng.standard_normal((m, n))
    b = rng.standard_normal(m)
    qr, diag = O.qr(a)
    x, info = O.qr_ls_solve(qr, diag, b)
    assert info == 0
    x = x[:, 0]
    assert np.allclose(a.T @ a @ x, a.T @ b, atol=1e-5)
    assert np.allclose(x, np.linalg.lstsq(a, b, rcond=None)[0], atol=1e-10)


def test_qr_rank_deficient_reports_info():
    a = np.zeros((6, 3))
    a[:, 0] = 1.0
    qr, diag = O.qr(a)
    _, info = O.qr_ls_solve(qr, diag, np.ones(6))
    assert info > 0


def test_gemm_dot2_is_accurate():
    rng = np.random.default_rng(5)
    a = rng.standard_normal((30, 40)) * 2.0 ** rng.integers(-20, 21, size=(30, 1))
    b = rng.standard_normal((40, 20)) * 2.0 ** rng.integers(-20, 21, size=(1, 20))
    c = O.gemm_dot2(1.0, a, b)
    from fractions import Fraction

    i, j = 7, 11
    exact = sum(Fraction(a[i, k]) * Fraction(b[k, j]) for k in range(40))
    assert abs(Fraction(c[i, j]) - exact) <= abs(exact) * Fraction(2 * EPS64)
    c2 = O.gemm_dot2(2.0, a, b, beta=-1.0, c=np.ones((30, 20)))
    assert np.allclose(c2, 2 * (a @ b) - 1, rtol=1e-12, atol=1e-6)


def test_golden_fixtures_reproduce():
    """The committed oracle fixtures (tests/golden/make_golden.py) are
    reproduced bit for bit by the oracle built here."""
    from tests.golden.make_golden import make

    fresh = make()
    with np.load(os.path.join(GOLD, "oracle_small.npz")) as z:
        for key in z.files:
            ref = z[key]
            got = fresh[key]
            if key.endswith("logdet"):
                assert np.allclose(got, ref, rtol=1e-14, atol=0), key
            else:
                assert np.array_equal(got, ref, equal_nan=True), key


def _relative_eq(a, b, max_relative, epsilon=np.finfo(np.float64).eps):
    """approx's relative_eq per entry: equal, or |a-b| <= epsilon (absolute,
    f64::EPSILON by default), or |a-b| <= max_relative * max(|a|, |b|)."""
    a, b = np.asarray(a), np.asarray(b)
    d = np.abs(a - b)
    return bool(np.all((a == b) | (d <= epsilon) | (d <= max_relative * np.maximum(np.abs(a), np.abs(b)))))


def test_try_inverse_known_answers():
    """tests/linalg/inverse.rs:62-81 and 126-142 (the n = 5 Gaussian-elimination
    inverse, lu::try_invert_to), restated through the oracle's LU::try_inverse."""
    k = _known()["inverse_matrix5"]
    m = _rows(k["rows"])
    lu, ipiv, _ = O.lu(m)
    inv = O.lu_try_inverse(lu, ipiv)
    exp = _rows(k["expected_inverse_rows"])
    assert _relative_eq(inv, exp, k["max_relative"])
    k = _known()["inverse_matrix5_scaled_identity"]
    m = k["diagonal"] * np.eye(k["n"])
    lu, ipiv, _ = O.lu(m)
    inv = O.lu_try_inverse(lu, ipiv)
    assert _relative_eq(inv, k["expected_inverse_diagonal"] * np.eye(k["n"]), k["max_relative"])


def test_try_inverse_singular_is_none():
    a = np.array([[1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [0.0, 1.0, 1.0]])
    lu, ipiv, _ = O.lu(a)
    assert O.lu_try_inverse(lu, ipiv) is None


@pytest.mark.parametrize("seed", range(6))
def test_triangular_solve_properties(seed):
    """tests/linalg/solve.rs:20-60: 4x4 matrices with near-zero diagonals set to
    1 (unzero_diagonal), 4x5 right-hand sides, tri * x == b to 1e-7 for the
    lower / upper / tr_ forms."""
    rng = np.random.default_rng(500 + seed)
    a = rng.uniform(-1, 1, size=(4, 4))
    d = np.diag(a).copy()
    d[np.abs(d) < 1e-7] = 1.0
    a[np.arange(4), np.arange(4)] = d
    b = rng.uniform(-1, 1, size=(4, 5))
    for upper, trans in ((False, False), (True, False), (False, True), (True, True)):
        tri = np.triu(a) if upper else np.tril(a)
        x = O.triangular_solve(a, b, upper=upper, trans=trans)
        assert np.allclose((tri.T if trans else tri) @ x, b, atol=1e-7, rtol=0)
    x = O.triangular_solve(a, b, diag=1.0)
    assert np.allclose((np.tril(a, -1) + np.eye(4)) @ x, b, atol=1e-7, rtol=0)


def _inv_permute_columns(m, jpiv):
    """PermutationSequence::inv_permute_columns (permutation_sequence.rs:131-140)."""
    m = m.copy()
    for i in reversed(range(len(jpiv))):
        q = jpiv[i]
        if q != i:
            m[:, [i, q]] = m[:, [q, i]]
    return m


@pytest.mark.parametrize("case", ["full_piv_lu_simple", "full_piv_lu_simple_with_pivot"])
def test_full_piv_lu_known_answers(case):
    """tests/linalg/full_piv_lu.rs:3-40: the exact determinant and P, L, U, Q
    reconstructing m."""
    k = _known()[case]
    m = _rows(k["rows"])
    lu, ipiv, jpiv, steps = O.full_piv_lu(m)
    assert steps == 3
    assert O.full_piv_lu_determinant(lu, ipiv, jpiv) == k["determinant"]
    l, u = _unpack(lu, ipiv)
    rec = _inv_permute_columns(_inv_permute_rows(l @ u, ipiv), jpiv)
    assert np.allclose(rec, m, atol=k["reconstruction_epsilon"], rtol=0)


@pytest.mark.parametrize("n", [1, 2, 5, 17, 40])
def test_full_piv_lu_properties(n):
    """The reference's property tests (tests/linalg/full_piv_lu.rs:62-100):
    P L U Q reconstructs m, |L| <= 1, solve gives m x = b, the determinant."""
    rng = np.random.default_rng(900 + n)
    m = rng.standard_normal((n, n))
    lu, ipiv, jpiv, steps = O.full_piv_lu(m)
    assert steps == n
    l, u = _unpack(lu, ipiv)
    rec = _inv_permute_columns(_inv_permute_rows(l @ u, ipiv), jpiv)
    assert np.allclose(rec, m, atol=1e-12 * n, rtol=0)
    assert np.all(np.abs(np.tril(lu, -1)) <= 1.0)
    b = rng.standard_normal((n, 3))
    x = O.full_piv_lu_solve(lu, ipiv, jpiv, b)
    assert np.allclose(m @ x, b, atol=1e-10, rtol=0)
    det = O.full_piv_lu_determinant(lu, ipiv, jpiv)
    assert np.isclose(det, np.linalg.det(m), rtol=1e-10, atol=0)


def test_full_piv_lu_rank_deficient_stops():
    """A rank-1 4x4 matrix: one step, then the remaining submatrix is zero
    (full_piv_lu.rs:73-76), so the solve returns None."""
    m = np.outer([1.0, 2.0, 4.0, 0.5], [3.0, -1.0, 2.0, 5.0])  # rank 1, every elimination exact
    lu, ipiv, jpiv, steps = O.full_piv_lu(m)
    assert steps == 1 and ipiv[0] == 2 and jpiv[0] == 3
    assert list(ipiv[steps:]) == list(range(steps, 4)) and list(jpiv[steps:]) == list(range(steps, 4))
    assert O.full_piv_lu_solve(lu, ipiv, jpiv, np.ones(4)) is None
    assert O.full_piv_lu_determinant(lu, ipiv, jpiv) == 0.0
    lz, _, _, sz = O.full_piv_lu(np.zeros((3, 3)))
    assert sz == 0 and np.all(lz == 0)


def test_full_piv_lu_pivot_rule_ties_and_nan():
    """icamax_full (min_max.rs:146-167): the first maximum in column-major order;
    a NaN wins only at (0, 0)."""
    m = np.array([[1.0, 4.0], [4.0, 2.0]])  # equal maxima at (1, 0) and (0, 1): (1, 0) first
    _, ipiv, jpiv, _ = O.full_piv_lu(m)
    assert ipiv[0] == 1 and jpiv[0] == 0
    m = np.array([[np.nan, 5.0], [1.0, 2.0]])
    _, ipiv, jpiv, _ = O.full_piv_lu(m)
    assert ipiv[0] == 0 and jpiv[0] == 0
    m = np.array([[1.0, np.nan], [3.0, 2.0]])
    _, ipiv, jpiv, _ = O.full_piv_lu(m)
    assert ipiv[0] == 1 and jpiv[0] == 0


def _pure_python_full_piv_lu(a):
    """Independent pure-Python restatement of FullPivLU::new for tiny matrices."""
    a = [list(map(float, r)) for r in a]
    n = len(a)
    ipiv, jpiv, steps = list(range(n)), list(range(n)), n
    for i in range(n):
        best, br, bc = abs(a[i][i]), i, i
        for c in range(i, n):
            for r in range(i, n):
                if abs(a[r][c]) > best:
                    best, br, bc = abs(a[r][c]), r, c
        diag = a[br][bc]
        if diag == 0.0:
            steps = i
            break
        for r in range(n):
            a[r][i], a[r][bc] = a[r][bc], a[r][i]
        jpiv[i], ipiv[i] = bc, br
        a[i], a[br] = a[br], a[i]
        inv = 1.0 / diag
        for r in range(i + 1, n):
            a[r][i] = a[r][i] * inv
        for c in range(i + 1, n):
            p = a[i][c]
            for r in range(i + 1, n):
                a[r][c] = (-p) * a[r][i] + a[r][c]
    return np.array(a), np.array(ipiv), np.array(jpiv), steps


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8])
def test_full_piv_lu_matches_pure_python_restatement_bitwise(n):
    rng = np.random.default_rng(40 + n)
    a = rng.uniform(-100, 100, size=(n, n))
    lu, ipiv, jpiv, steps = O.full_piv_lu(a)
    lu2, ipiv2, jpiv2, steps2 = _pure_python_full_piv_lu(a)
    assert steps == steps2
    assert np.array_equal(ipiv, ipiv2) and np.array_equal(jpiv, jpiv2)
    assert np.array_equal(lu, lu2)


def _colpiv_reconstruct(qr, diag, jpiv):
    q, r = O.col_piv_qr_q_r(qr, diag)
    return q, _inv_permute_columns(q @ r, jpiv)


def test_col_piv_qr_known_answer():
    """tests/linalg/col_piv_qr.rs:5-21: the (singular) 4x4 matrix has a zero
    determinant to 1e-7 and Q R P^-1 reconstructs it."""
    k = _known()["col_piv_qr"]
    m = _rows(k["rows"])
    qr, diag, jpiv = O.col_piv_qr(m)
    det = float(np.prod(diag)) * (-1.0 if int(np.sum(jpiv != np.arange(4))) % 2 else 1.0)
    assert abs(det - k["determinant"]) <= k["determinant_epsilon"]
    q, rec = _colpiv_reconstruct(qr, diag, jpiv)
    assert np.allclose(rec, m, atol=k["reconstruction_epsilon"], rtol=0)
    assert np.allclose(q.T @ q, np.eye(4), atol=1e-7, rtol=0)


@pytest.mark.parametrize("m,n", [(1, 1), (5, 5), (9, 4), (4, 9), (30, 30)])
def test_col_piv_qr_properties(m, n):
    """tests/linalg/col_piv_qr.rs:40-80: Q R P^-1 = m and Q orthogonal (1e-7);
    for square systems solve gives m x = b."""
    rng = np.random.default_rng(600 + 7 * m + n)
    a = rng.uniform(-100, 100, size=(m, n))
    qr, diag, jpiv = O.col_piv_qr(a)
    q, rec = _colpiv_reconstruct(qr, diag, jpiv)
    assert np.allclose(rec, a, atol=1e-7, rtol=0)
    assert np.allclose(q.T @ q, np.eye(min(m, n)), atol=1e-7, rtol=0)
    if m == n:
        b = rng.standard_normal((n, 2))
        x, ok = O.col_piv_qr_solve(qr, diag, jpiv, b)
        assert ok and np.allclose(a @ x, b, atol=1e-9, rtol=0)


def test_col_piv_qr_pivots_on_the_largest_entry():
    """The pivot column holds the trailing submatrix's largest |a| (icamax_full),
    not the largest column norm: column 1 has the larger norm, column 0 the
    larger entry."""
    a = np.array([[5.0, 3.0], [0.0, 3.0]])
    _, _, jpiv = O.col_piv_qr(a)
    assert jpiv[0] == 0
    a = np.array([[1.0, 3.0], [1.0, 3.0]])
    _, _, jpiv = O.col_piv_qr(a)
    assert jpiv[0] == 1


def test_col_piv_qr_zero_column_and_failed_solve():
    """A zero matrix: no reflection (diag = +/-0), the solve returns false after
    q_tr_mul and the inverse permutation, with b still overwritten."""
    qr, diag, jpiv = O.col_piv_qr(np.zeros((3, 3)))
    assert np.all(diag == 0)
    x, ok = O.col_piv_qr_solve(qr, diag, jpiv, np.array([1.0, 2.0, 3.0]))
    assert not ok


def _pure_python_rank_one_update(l, x, sigma):
    """Independent pure-Python restatement of xx_rank_one_update
    (src/linalg/cholesky.rs:404-449) on the lower part of l."""
    import math

    n = len(x)
    l = [[float(l[r][c]) for c in range(n)] for r in range(n)]
    x = [float(v) for v in x]
    beta = 1.0
    for j in range(n):
        diag = l[j][j]
        diag2 = diag * diag
        xj = x[j]
        sigma_xj2 = sigma * (xj * xj)
        gamma = diag2 * beta + sigma_xj2
        new_diag = math.sqrt(diag2 + sigma_xj2 / beta)
        l[j][j] = new_diag
        beta += sigma_xj2 / diag2
        a1 = -xj / diag
        for r in range(j + 1, n):
            x[r] = a1 * l[r][j] + x[r]
        if gamma != 0.0:
            a2 = new_diag * sigma / gamma * xj
            b2 = new_diag / diag
            for r in range(j + 1, n):
                l[r][j] = a2 * x[r] + b2 * l[r][j]
    return np.array(l)


@pytest.mark.parametrize("n", [1, 3, 8, 13])
@pytest.mark.parametrize("sigma", [0.7, -0.2])
def test_rank_one_update_matches_pure_python_restatement_bitwise(n, sigma):
    rng = np.random.default_rng(70 + n)
    b = rng.standard_normal((n, n))
    l, info = O.cholesky(b @ b.T + n * np.eye(n))
    assert info == 0
    x = rng.standard_normal(n) / np.sqrt(n)
    got = O.cholesky_rank_one_update(l, x, sigma)
    ref = _pure_python_rank_one_update(l, x, sigma)
    assert np.array_equal(np.tril(got), np.tril(ref))
    assert np.array_equal(np.triu(got, 1), np.triu(l, 1))  # the strict upper part is not touched


def _random_sdp(rng, n):
    b = rng.standard_normal((n, n))
    return b @ b.T + n * np.eye(n)


@pytest.mark.parametrize("seed", range(5))
def test_cholesky_update_properties(seed):
    """tests/linalg/cholesky.rs:120-173: rank_one_update with sigma in [0, 1),
    insert_column and remove_column (n <= 10, random j) rebuild the updated
    matrix to 1e-7."""
    rng = np.random.default_rng(800 + seed)
    m = _random_sdp(rng, 4)
    x = rng.uniform(-1, 1, 4)
    sigma = float(rng.random())
    l, _ = O.cholesky(m)
    lu = np.tril(O.cholesky_rank_one_update(l, x, sigma))
    assert np.allclose(lu @ lu.T, m + sigma * np.outer(x, x), atol=1e-7, rtol=0)
    n = int(rng.integers(1, 11))
    j = int(rng.integers(0, n))
    m_updated = _random_sdp(rng, n)
    m_small = np.delete(np.delete(m_updated, j, axis=0), j, axis=1)
    l_small, _ = O.cholesky(m_small) if n > 1 else (np.zeros((0, 0)), 0)
    li = np.tril(O.cholesky_insert_column(l_small, j, m_updated[:, j]))
    assert np.allclose(li @ li.T, m_updated, atol=1e-7, rtol=0)
    l_full, _ = O.cholesky(m_updated)
    lr = np.tril(O.cholesky_remove_column(l_full, j))
    assert np.allclose(lr @ lr.T, m_small, atol=1e-7, rtol=0)


def _py_dotx(x, y):
    """Matrix::dotx (src/base/blas.rs:96-165) in pure Python."""
    n = len(x)
    acc = [0.0] * 8
    i = 0
    while n - i >= 8:
        for q in range(8):
            acc[q] += x[i + q] * y[i + q]
        i += 8
    res = 0.0
    for q in range(4):
        res += acc[q] + acc[q + 4]
    for k in range(i, n):
        res += x[k] * y[k]
    return res


def _pure_python_col_piv_qr(a):
    """Independent pure-Python restatement of ColPivQR::new
    (src/linalg/col_piv_qr.rs:59-92, householder.rs:19-85, reflection.rs:70-83)
    for tiny square matrices; columns as lists."""
    import math

    n = len(a)
    cols = [[float(a[r][c]) for r in range(n)] for c in range(n)]
    diag, jpiv = [0.0] * n, list(range(n))
    for i in range(n):
        best, bc = abs(cols[i][i]), i
        for c in range(i, n):
            for r in range(i, n):
                if abs(cols[c][r]) > best:
                    best, bc = abs(cols[c][r]), c
        cols[i], cols[bc] = cols[bc], cols[i]
        jpiv[i] = bc
        x = cols[i][i:]
        sq = 0.0 + _py_dotx(x, x)
        nrm = math.sqrt(sq)
        modulus, sign = (x[0], 1.0) if x[0] >= 0 else (-x[0], -1.0)
        signed_norm = sign * nrm
        factor = (sq + modulus * nrm) * 2.0
        x[0] += signed_norm
        if factor != 0.0:
            sf = math.sqrt(factor)
            x = [v / sf for v in x]
            n2 = math.sqrt(0.0 + _py_dotx(x, x))
            x = [v / n2 for v in x]
            rnorm = -signed_norm
            sgn = math.copysign(1.0, rnorm)
            for c in range(i + 1, n):
                y = cols[c][i:]
                f = (_py_dotx(x, y) - 0.0) * (sgn * -2.0)
                cols[c][i:] = [f * x[k] + sgn * y[k] for k in range(len(y))]
        else:
            rnorm = signed_norm
        cols[i][i:] = x
        diag[i] = rnorm
    return np.array(cols).T, np.array(diag), np.array(jpiv)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 9])
def test_col_piv_qr_matches_pure_python_restatement_bitwise(n):
    rng = np.random.default_rng(90 + n)
    a = rng.uniform(-100, 100, size=(n, n))
    qr, diag, jpiv = O.col_piv_qr(a)
    qr2, diag2, jpiv2 = _pure_python_col_piv_qr(a)
    assert np.array_equal(jpiv, jpiv2)
    assert np.array_equal(diag, diag2)
    assert np.array_equal(qr, qr2)


def _pure_python_trsv(t, b, upper, trans, diag=None):
    """Independent pure-Python restatement of the vector loops of
    src/linalg/solve.rs (:74-101, :106-133, :156-182, :374-442) for one column."""
    n = len(b)
    x = [float(v) for v in b]
    if diag is not None:  # solve_lower_triangular_with_diag_mut: b_i is never rewritten
        if diag == 0.0:
            return None
        for i in range(n - 1):
            coeff = x[i] / diag
            for r in range(i + 1, n):
                x[r] = -coeff * t[r][i] + x[r]
        return x
    if not trans:
        order = reversed(range(n)) if upper else range(n)
        for i in order:
            d = t[i][i]
            if d == 0.0:
                return None
            coeff = x[i] / d
            x[i] = coeff
            rows = range(i) if upper else range(i + 1, n)
            for r in rows:
                x[r] = -coeff * t[r][i] + x[r]
        return x
    order = range(n) if upper else reversed(range(n))
    for i in order:
        rows = list(range(i)) if upper else list(range(i + 1, n))
        dot = _py_dotx([t[r][i] for r in rows], [x[r] for r in rows])
        d = t[i][i]
        if d == 0.0:
            return None
        x[i] = (x[i] - dot) / d
    return x


@pytest.mark.parametrize("n", [1, 7, 8, 9, 17])
def test_triangular_solves_match_pure_python_restatement_bitwise(n):
    rng = np.random.default_rng(120 + n)
    t = rng.uniform(-1, 1, size=(n, n)) + 2 * np.eye(n)
    b = rng.uniform(-1, 1, size=n)
    for upper in (False, True):
        for trans in (False, True):
            got = O.triangular_solve(t, b, upper=upper, trans=trans)
            ref = _pure_python_trsv(t, b, upper, trans)
            assert np.array_equal(np.asarray(got).ravel(), np.array(ref)), (upper, trans)
    got = O.triangular_solve(t, b, diag=2.5)
    assert np.array_equal(np.asarray(got).ravel(), np.array(_pure_python_trsv(t, b, False, False, diag=2.5)))


def test_batch_backward_error_helpers_match_per_system_metric():
    """The batch checkers the bench and the GPU tests use (Dot2 residuals,
    per system; one large dense system) agree with the per-system
    backward_error on the symmetric matrix of the lower triangle, and with
    numpy's extended-precision residual."""
    from nalgebra_gb300 import workloads as W

    w = W.ragged_spd(40, 1, 40, nrhs=3, seed=9)
    ns, aoff, boff = w["ns"], w["a_offsets"], w["b_offsets"]
    a_flat = w["a_flat"].copy()
    for s in range(ns.size):  # garbage in the strict upper part: only the lower triangle counts
        n = int(ns[s])
        m = a_flat[aoff[s]:aoff[s] + n * n].reshape(n, n)
        m[np.tril_indices(n, -1)] = 1e3
    _, x, _, _ = O.posv_ragged(ns, aoff, w["a_flat"], boff, w["b_flat"], 3)
    x = x + 1e-9  # a visible error
    be = O.ragged_backward_errors(ns, aoff, a_flat, boff, w["b_flat"], x, 3)
    for s in range(ns.size):
        n = int(ns[s])
        a = w["a_flat"][aoff[s]:aoff[s] + n * n].reshape(n, n).T
        a = np.tril(a) + np.tril(a, -1).T
        xs = x[boff[s]:boff[s] + 3 * n].reshape(3, n).T
        bs = w["b_flat"][boff[s]:boff[s] + 3 * n].reshape(3, n).T
        assert be[s] == pytest.approx(O.backward_error(a, xs, bs), rel=1e-12)
    rng = np.random.default_rng(4)
    n = 300
    a = rng.standard_normal((n, n))
    xx = rng.standard_normal(n)
    bb = a @ xx
    ref = O.backward_error(a, xx, bb)
    assert O.dense_backward_error(a.ravel(order="F"), n, xx, bb) == pytest.approx(ref, rel=1e-12)


def test_gemm_gemv_order_restatement_bit_for_bit():
    """The oracle's gemm in nalgebra's gemv order (blas_uninit.rs:32-78,
    127-176, 320-332) against a pure-Python transcription of the same loops,
    with beta zero and non-zero and k = 0; and the reference's gemm example
    (blas.rs:713-727) to relative accuracy."""
    rng = np.random.default_rng(12)

    def loops(alpha, a, b, beta, c):
        m, k = a.shape
        n = b.shape[1]
        y = c.copy()
        for j in range(n):
            if k == 0:
                for i in range(m):
                    y[i, j] = 0.0 if beta == 0.0 else y[i, j] * beta
                continue
            for l in range(k):
                bb = beta if l == 0 else 1.0
                for i in range(m):
                    t = alpha * a[i, l] * b[l, j]
                    y[i, j] = t if bb == 0.0 else t + bb * y[i, j]
        return y

    for (m, n, k) in [(3, 4, 5), (1, 1, 1), (6, 2, 0), (5, 7, 3)]:
        for alpha, beta in [(1.0, 0.0), (1.3, 0.7), (-0.5, 1.0)]:
            a = rng.standard_normal((m, k))
            b = rng.standard_normal((k, n))
            c = rng.standard_normal((m, n))
            assert np.array_equal(O.gemm_gemv_order(alpha, a, b, beta, c), loops(alpha, a, b, beta, c))
    mat1 = np.eye(2, 4)
    mat2 = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]])
    mat3 = np.array([[0.1, 0.2, 0.3, 0.4], [0.5, 0.6, 0.7, 0.8], [0.9, 1.0, 1.1, 1.2]])
    assert np.allclose(O.gemm_gemv_order(10.0, mat2, mat3, 5.0, mat1), mat2 @ mat3 * 10.0 + mat1 * 5.0, rtol=1e-12)


@pytest.mark.parametrize("n", [1, 4, 10, 20])
def test_qr_solve_properties(n):
    """tests/linalg/qr.rs:55-69, 87-99: for invertible square m, QR::solve gives
    m x = b (1e-6; here far tighter) and solve_mut on the identity gives the
    inverse (m m^-1 = I to 1e-5)."""
    rng = np.random.default_rng(700 + n)
    a = rng.uniform(-100, 100, size=(n, n))
    qr, diag = O.qr(a)
    b = rng.standard_normal((n, 3))
    x, ok = O.qr_solve(qr, diag, b)
    assert ok and np.allclose(a @ x, b, atol=1e-9, rtol=0)
    inv, ok = O.qr_solve(qr, diag, np.eye(n))
    assert ok and np.allclose(a @ inv, np.eye(n), atol=1e-9, rtol=0)
    assert np.allclose(inv @ a, np.eye(n), atol=1e-9, rtol=0)


def test_qr_solve_equals_col_piv_solve_without_pivots():
    """QR::solve_mut and ColPivQR::solve_mut run the same q_tr_mul and upper
    solve; with an identity permutation their restatements agree bit for bit
    (the one difference is the inverse permutation)."""
    rng = np.random.default_rng(711)
    a = rng.uniform(-100, 100, size=(12, 12))
    qr, diag = O.qr(a)
    b = rng.standard_normal((12, 2))
    x, ok = O.qr_solve(qr, diag, b)
    y, ok2 = O.col_piv_qr_solve(qr, diag, np.arange(12, dtype=np.int32), b)
    assert ok and ok2 and np.array_equal(x, y)


def test_qr_solve_zero_diagonal_returns_false():
    """A zero |diag_i| stops the upper solve (qr.rs:238-242): false."""
    qr, diag = O.qr(np.zeros((3, 3)))
    _, ok = O.qr_solve(qr, diag, np.array([1.0, 2.0, 3.0]))
    assert not ok


def _pure_python_qr(a):
    """Independent pure-Python restatement of QR::new (src/linalg/qr.rs:55-76:
    clear_column_unchecked per column, householder.rs:19-85, reflection.rs:70-83)
    for small m x n matrices of any shape; columns as lists."""
    import math

    m, n = len(a), len(a[0])
    cols = [[float(a[r][c]) for r in range(m)] for c in range(n)]
    diag = [0.0] * min(m, n)
    for i in range(min(m, n)):
        x = cols[i][i:]
        sq = 0.0 + _py_dotx(x, x)
        nrm = math.sqrt(sq)
        modulus, sign = (x[0], 1.0) if x[0] >= 0 else (-x[0], -1.0)
        signed_norm = sign * nrm
        factor = (sq + modulus * nrm) * 2.0
        x[0] += signed_norm
        if factor != 0.0:
            sf = math.sqrt(factor)
            x = [v / sf for v in x]
            n2 = math.sqrt(0.0 + _py_dotx(x, x))
            x = [v / n2 for v in x]
            rnorm = -signed_norm
            sgn = math.copysign(1.0, rnorm)
            for c in range(i + 1, n):
                y = cols[c][i:]
                f = (_py_dotx(x, y) - 0.0) * (sgn * -2.0)
                cols[c][i:] = [f * x[k] + sgn * y[k] for k in range(len(y))]
        else:
            rnorm = signed_norm
        cols[i][i:] = x
        diag[i] = rnorm
    return np.array(cols).T, np.array(diag)


@pytest.mark.parametrize("m,n", [(1, 1), (1, 6), (6, 1), (9, 9), (12, 5), (5, 12), (17, 11)])
def test_qr_matches_pure_python_restatement_bitwise(m, n):
    """The oracle's QR::new for tall, square and wide shapes (the one-matrix GPU
    kernel's checker), with a zero column and a column whose squares underflow
    (a zero norm over nonzero entries: no reflection, x[0] += 0)."""
    rng = np.random.default_rng(800 + 13 * m + n)
    a = rng.uniform(-100, 100, size=(m, n))
    if min(m, n) >= 5:
        a[:, 2] = 0.0
        a[:, 4] = 1e-170
    qr, diag = O.qr(a)
    qr2, diag2 = _pure_python_qr(a)
    assert np.array_equal(diag, diag2) and np.array_equal(qr, qr2)
    if min(m, n) >= 5:
        assert diag[2] == 0.0 and diag[4] == 0.0
