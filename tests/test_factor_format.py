"""nalgebra's serde JSON form of the factor objects (nalgebra_gb300.factor_format):
the reference's own serde strings (tests/core/serde.rs:25-55), the layouts of
PermutationSequence and of the decompositions, and exact round trips of
factors computed by the oracle."""
import json

import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import factor_format as F


def test_reference_dmatrix_strings():
    """tests/core/serde.rs:25-47: "[[1.0, ..., 6.0],2,3]" is the 2x3 matrix of
    that column slice; five components for a 2x3 matrix are refused."""
    m = F.matrix_from_obj(json.loads("[[1.0, 2.0, 3.0, 4.0, 5.0, 6.0],2,3]"))
    assert np.array_equal(m, np.array([[1.0, 3.0, 5.0], [2.0, 4.0, 6.0]]))
    assert F.matrix_to_obj(m) == [[1.0, 2.0, 3.0, 4.0, 5.0, 6.0], 2, 3]
    with pytest.raises(ValueError, match="Expected 6 components, found 5"):
        F.matrix_from_obj(json.loads("[[1.0, 2.0, 3.0, 4.0, 5.0],2,3]"))


def test_permutation_sequence_layout():
    """lu_simple_with_pivot (tests/linalg/lu.rs:24-39) swaps rows 0 and 2 once:
    len 1, the swap first, identity_generic's (0, 0) after it."""
    m = np.array([[0.0, -1.0, 2.0], [-1.0, 2.0, -1.0], [2.0, -1.0, 0.0]])
    lu, ipiv, ln = O.lu(m)
    o = json.loads(F.lu_to_json(lu, ipiv))
    assert list(o) == ["lu", "p"]
    assert o["p"] == {"len": ln, "ipiv": [[[0, 2], [0, 0], [0, 0]], 3, 1]}
    assert o["lu"][1:] == [3, 3]
    lu2, ipiv2 = F.lu_from_json(json.dumps(o))
    assert np.array_equal(lu2, lu) and np.array_equal(ipiv2, ipiv)


@pytest.mark.parametrize("n", [1, 5, 17])
def test_round_trips_are_exact(n):
    rng = np.random.default_rng(300 + n)
    a = rng.uniform(-100, 100, size=(n, n))
    a[0, 0] = 5e-324  # a subnormal survives the text form
    lu, ipiv, _ = O.lu(a)
    l2, p2 = F.lu_from_json(F.lu_to_json(lu, ipiv))
    assert np.array_equal(l2, lu) and np.array_equal(p2, ipiv)
    flu, fp, fq, _ = O.full_piv_lu(a)
    o = json.loads(F.full_piv_lu_to_json(flu, fp, fq))
    assert list(o) == ["lu", "p", "q"]
    f2 = F.full_piv_lu_from_json(json.dumps(o))
    assert np.array_equal(f2[0], flu) and np.array_equal(f2[1], fp) and np.array_equal(f2[2], fq)
    qr, diag, jp = O.col_piv_qr(a)
    o = json.loads(F.col_piv_qr_to_json(qr, jp, diag))
    assert list(o) == ["col_piv_qr", "p", "diag"] and o["diag"][1:] == [n, 1]
    c2 = F.col_piv_qr_from_json(json.dumps(o))
    assert np.array_equal(c2[0], qr) and np.array_equal(c2[1], jp) and np.array_equal(c2[2], diag)
    spd = a @ a.T + n * np.eye(n)
    l, info = O.cholesky(spd)
    assert info == 0
    assert np.array_equal(F.cholesky_from_json(F.cholesky_to_json(l)), l)


def test_qr_layout():
    rng = np.random.default_rng(5)
    a = rng.standard_normal((6, 4))
    qr = np.asfortranarray(a.copy())
    o = json.loads(F.qr_to_json(qr, np.arange(4.0)))
    assert list(o) == ["qr", "diag"] and o["qr"][1:] == [6, 4] and o["diag"] == [[0.0, 1.0, 2.0, 3.0], 4, 1]
    q2, d2 = F.qr_from_json(json.dumps(o))
    assert np.array_equal(q2, qr) and np.array_equal(d2, np.arange(4.0))


def test_non_finite_values_follow_serde_json():
    """serde_json writes NaN and infinities as null and refuses null for an f64."""
    s = F.cholesky_to_json(np.array([[np.nan, 0.0], [np.inf, 1.0]]))
    assert json.loads(s)["chol"][0] == [None, None, 0.0, 1.0]
    with pytest.raises(ValueError, match="expected f64"):
        F.cholesky_from_json(s)


def test_empty_and_malformed_objects():
    """A 0 x 0 factor round-trips; a permutation whose len exceeds its vector,
    or a vector that is not n x 1, is refused."""
    lu, ipiv = F.lu_from_json(F.lu_to_json(np.zeros((0, 0)), np.zeros(0, dtype=np.int32)))
    assert lu.shape == (0, 0) and ipiv.shape == (0,)
    with pytest.raises(ValueError, match="exceeds"):
        F.permutation_from_obj({"len": 3, "ipiv": [[[0, 1], [0, 0]], 2, 1]})
    with pytest.raises(ValueError, match="components"):
        F.permutation_from_obj({"len": 1, "ipiv": [[[0, 1], [0, 0]], 2, 2]})
    with pytest.raises(ValueError, match="expected"):
        F.matrix_from_obj({"data": [1.0], "nrows": 1, "ncols": 1})


def test_out_of_range_swaps_are_refused():
    """A swap pair outside [0, dim), with i2 < i, out of step order, or a
    negative len would index outside the device factor: refused."""
    def perm(pairs, dim, k=None):
        pad = [[0, 0]] * (dim - len(pairs))
        return {"len": len(pairs) if k is None else k, "ipiv": [pairs + pad, dim, 1]}

    assert list(F.permutation_from_obj(perm([[0, 2], [1, 2]], 3))) == [2, 2, 2]
    for bad in (perm([[-1, 2]], 3), perm([[0, 3]], 3), perm([[2, 1]], 3), perm([[1, 2], [0, 1]], 3),
                perm([[1, 2], [1, 2]], 3), perm([[0, -3]], 3)):
        with pytest.raises(ValueError, match="out of"):
            F.permutation_from_obj(bad)
    with pytest.raises(ValueError, match="negative len"):
        F.permutation_from_obj(perm([[0, 1]], 3, k=-1))


def test_factor_shapes_are_checked():
    """A tall factor, or a permutation / diag of another dimension than the
    factor's order, is refused before anything reaches the device."""
    tall = np.arange(12.0).reshape(4, 3)
    with pytest.raises(ValueError, match="square"):
        F.lu_from_json(F.lu_to_json(tall, np.arange(3, dtype=np.int32)))
    with pytest.raises(ValueError, match="square"):
        F.cholesky_from_json(F.cholesky_to_json(tall))
    with pytest.raises(ValueError, match="square"):
        F.col_piv_qr_from_json(F.col_piv_qr_to_json(tall, np.arange(3), np.ones(3)))
    sq = np.eye(3)
    with pytest.raises(ValueError, match="does not match"):
        F.lu_from_json(F.lu_to_json(sq, np.arange(2, dtype=np.int32)))
    with pytest.raises(ValueError, match="does not match"):
        F.full_piv_lu_from_json(F.full_piv_lu_to_json(sq, np.arange(3), np.arange(4)))
    with pytest.raises(ValueError, match="does not match"):
        F.col_piv_qr_from_json(F.col_piv_qr_to_json(sq, np.arange(3), np.ones(2)))
    with pytest.raises(ValueError, match="does not match"):
        F.qr_from_json(F.qr_to_json(tall, np.ones(4)))
    q, d = F.qr_from_json(F.qr_to_json(tall, np.ones(3)))
    assert q.shape == (4, 3) and d.shape == (3,)
