"""Generates tests/golden/oracle_small.npz: seeded small inputs of every path
with the CPU oracle's outputs (bit-exact nalgebra arithmetic).  The GPU tests
compare the EXACT kernels against these bit for bit, and test_oracle checks
that the oracle built on any machine still reproduces them.

    python -m tests.golden.make_golden
"""
import os

import numpy as np

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
LU_SIZES = [1, 2, 5, 6, 16, 33, 64]
CHOL_SIZES = [1, 3, 8, 17, 33, 64, 100]
QR_SHAPES = [(7, 3), (128, 64), (200, 64)]


def make():
    out = {}
    rng = np.random.default_rng(2024)
    for n in LU_SIZES:
        for kind, shift in (("dom", float(n)), ("piv", 0.0)):
            a = rng.standard_normal((n, n)) + shift * np.eye(n)
            b = rng.standard_normal((n, 2))
            lu, ipiv, _ = O.lu(a)
            x = O.lu_solve(lu, ipiv, b)
            key = f"lu_n{n}_{kind}"
            out[key + "_a"] = a
            out[key + "_b"] = b
            out[key + "_lu"] = lu
            out[key + "_ipiv"] = ipiv
            out[key + "_x"] = x
    for n in CHOL_SIZES:
        bm = rng.standard_normal((n, n))
        a = bm @ bm.T + n * np.eye(n)
        rhs = rng.standard_normal((n, 4))
        l, info = O.cholesky(a)
        assert info == 0
        key = f"chol_n{n}"
        out[key + "_a"] = a
        out[key + "_b"] = rhs
        out[key + "_l"] = l
        out[key + "_x"] = O.cholesky_solve(l, rhs)
        out[key + "_logdet"] = np.array([O.cholesky_ln_determinant(l)])
    for m, n in QR_SHAPES:
        a = rng.standard_normal((m, n))
        b = rng.standard_normal(m)
        qr, diag = O.qr(a)
        x, info = O.qr_ls_solve(qr, diag, b)
        assert info == 0
        key = f"qr_m{m}_n{n}"
        out[key + "_a"] = a
        out[key + "_b"] = b
        out[key + "_qr"] = qr
        out[key + "_diag"] = diag
        out[key + "_x"] = x[:, 0]
    # the next rows: try_inverse, triangular solves, Cholesky factor updates,
    # FullPivLU and ColPivQR (drawn after the inputs above, which stay as they were)
    for n in (4, 16, 33):
        a = rng.standard_normal((n, n)) + n * np.eye(n)
        lu, ipiv, _ = O.lu(a)
        out[f"inv_n{n}_a"] = a
        out[f"inv_n{n}_inv"] = O.lu_try_inverse(lu, ipiv)
    for n in (7, 33, 100):
        t = rng.random((n, n)) + n * np.eye(n)
        b = rng.random((n, 2))
        out[f"trsv_n{n}_t"] = t
        out[f"trsv_n{n}_b"] = b
        for name, upper, trans in (("l", False, False), ("u", True, False), ("tl", False, True), ("tu", True, True)):
            out[f"trsv_n{n}_{name}_x"] = O.triangular_solve(t, b, upper=upper, trans=trans)
        out[f"trsv_n{n}_diag_x"] = O.triangular_solve(t, b, diag=2.5)
    for n in (5, 33):
        bm = rng.standard_normal((n, n))
        l, info = O.cholesky(bm @ bm.T + n * np.eye(n))
        assert info == 0
        x = rng.standard_normal(n)
        col = rng.standard_normal(n + 1)
        j = n // 2
        col[j] = float(col @ col) + n + 1.0
        key = f"cholupd_n{n}"
        out[key + "_l"] = l
        out[key + "_x"] = x
        out[key + "_col"] = col
        out[key + "_rank1"] = O.cholesky_rank_one_update(l, x, 0.7)
        out[key + "_remove"] = O.cholesky_remove_column(l, j)
        out[key + "_insert"] = O.cholesky_insert_column(l, j, col)
    for n in (5, 17, 64):
        a = rng.uniform(-100, 100, size=(n, n))
        b = rng.standard_normal((n, 2))
        lu, ipiv, jpiv, steps = O.full_piv_lu(a)
        key = f"fplu_n{n}"
        out[key + "_a"] = a
        out[key + "_b"] = b
        out[key + "_lu"] = lu
        out[key + "_ipiv"] = ipiv
        out[key + "_jpiv"] = jpiv
        out[key + "_x"] = O.full_piv_lu_solve(lu, ipiv, jpiv, b)
        qr, diag, qpiv = O.col_piv_qr(a)
        key = f"cpqr_n{n}"
        out[key + "_qr"] = qr
        out[key + "_diag"] = diag
        out[key + "_jpiv"] = qpiv
        out[key + "_x"] = O.col_piv_qr_solve(qr, diag, qpiv, b)[0]
    return out


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), **make())
    print("wrote", os.path.join(HERE, "oracle_small.npz"))
