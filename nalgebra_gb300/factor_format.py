"""nalgebra's serde JSON form of the factor objects, for the factors this
library computes on the device (host side, numpy arrays in and out).

The layouts follow the reference's Serialize impls, which serde_json writes
as follows:
  - a dynamic matrix (Matrix -> VecStorage, src/base/matrix.rs:239-252,
    src/base/vec_storage.rs:75-87, Dyn as a bare usize,
    src/base/dimension.rs:40-48): ``[[column-major data], nrows, ncols]``;
  - PermutationSequence (derived, src/linalg/permutation_sequence.rs:15-34):
    ``{"len": k, "ipiv": [[[i, i2], ...], dim, 1]}``, the k recorded swaps
    first and the rest of the vector holding identity_generic's (0, 0)
    (:72-79);
  - the decompositions (derived, field order kept): LU ``{"lu", "p"}``
    (src/linalg/lu.rs:32-38), FullPivLU ``{"lu", "p", "q"}``
    (full_piv_lu.rs:32-39), QR ``{"qr", "diag"}`` (qr.rs:34-40), ColPivQR
    ``{"col_piv_qr", "p", "diag"}`` (col_piv_qr.rs:36-43), Cholesky
    ``{"chol"}`` (cholesky.rs:28-33).
serde_json writes a non-finite f64 as ``null`` and refuses ``null`` for an
f64 when reading; both are kept.  Numbers are written in Python's shortest
round-trip form, which serde_json reads back to the same f64 (its own writer
may spell exponents differently, e.g. ``1e-7`` for ``1e-07``).

The device side stores a permutation as ``ipiv[i]`` (the index swapped with
i at step i, i when none); the pairs with ``ipiv[i] != i``, in order, are
the PermutationSequence's swaps.
"""
from __future__ import annotations

import json
import math

import numpy as np


def _num(x: float):
    x = float(x)
    return x if math.isfinite(x) else None


def _f64(v, where: str) -> float:
    if v is None or isinstance(v, bool) or not isinstance(v, (int, float)):
        raise ValueError(f"{where}: invalid type: {v!r}, expected f64")
    return float(v)


def matrix_to_obj(a) -> list:
    """A dynamic matrix as serde writes it: [[column-major data], nrows, ncols]."""
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    return [[_num(x) for x in a.ravel(order="F")], int(a.shape[0]), int(a.shape[1])]


def matrix_from_obj(o, where: str = "matrix") -> np.ndarray:
    """VecStorage's Deserialize (vec_storage.rs:89-114): the component count must
    be nrows * ncols."""
    if not (isinstance(o, list) and len(o) == 3 and isinstance(o[0], list)):
        raise ValueError(f"{where}: expected [data, nrows, ncols]")
    data, nrows, ncols = o
    nrows, ncols = int(nrows), int(ncols)
    if nrows * ncols != len(data):
        raise ValueError(f"{where}: Expected {nrows * ncols} components, found {len(data)}")
    vals = np.array([_f64(v, where) for v in data], dtype=np.float64)
    return vals.reshape(ncols, nrows).T.copy(order="F") if nrows * ncols else np.zeros((nrows, ncols))


def permutation_to_obj(ipiv, dim: int | None = None) -> dict:
    """PermutationSequence from the device form ipiv[i]."""
    ipiv = [int(p) for p in np.asarray(ipiv).ravel()]
    dim = len(ipiv) if dim is None else int(dim)
    pairs = [[i, p] for i, p in enumerate(ipiv) if p != i]
    pad = [[0, 0]] * (dim - len(pairs))
    return {"len": len(pairs), "ipiv": [pairs + pad, dim, 1]}


def permutation_from_obj(o, where: str = "permutation") -> np.ndarray:
    """The device form ipiv[i] (int32) of a PermutationSequence."""
    if not (isinstance(o, dict) and "len" in o and "ipiv" in o):
        raise ValueError(f"{where}: expected {{len, ipiv}}")
    k = int(o["len"])
    data, nrows, ncols = o["ipiv"]
    dim = int(nrows)
    if dim * int(ncols) != len(data) or int(ncols) != 1:
        raise ValueError(f"{where}: Expected {dim * int(ncols)} components, found {len(data)}")
    if k > dim:
        raise ValueError(f"{where}: len {k} exceeds the dimension {dim}")
    if k < 0:
        raise ValueError(f"{where}: negative len {k}")
    ipiv = np.arange(dim, dtype=np.int32)
    prev = -1
    for pair in data[:k]:
        if not (isinstance(pair, list) and len(pair) == 2):
            raise ValueError(f"{where}: expected [i, i2] pairs")
        i, i2 = int(pair[0]), int(pair[1])
        # The factorizations append (i, piv) at step i with i < piv < dim
        # (lu.rs:103-113, full_piv_lu.rs:79-82, col_piv_qr.rs:74-78,
        # append_permutation skipping i == piv); only such sequences have the
        # per-step device form.
        if not (0 <= i < dim and i <= i2 < dim):
            raise ValueError(f"{where}: swap ({i}, {i2}) out of range for dimension {dim}")
        if i <= prev:
            raise ValueError(f"{where}: swap ({i}, {i2}) out of step order")
        prev = i
        ipiv[i] = i2
    return ipiv


def _square(m: np.ndarray, where: str) -> int:
    if m.shape[0] != m.shape[1]:
        raise ValueError(f"{where}: the factor is {m.shape[0]} x {m.shape[1]}, expected a square matrix")
    return int(m.shape[0])


def _dim(v: np.ndarray, n: int, where: str) -> None:
    if v.shape[0] != n:
        raise ValueError(f"{where}: dimension {v.shape[0]} does not match the factor's order {n}")


def _dump(obj: dict) -> str:
    return json.dumps(obj, separators=(",", ":"), allow_nan=False)


def lu_to_json(lu, ipiv) -> str:
    """LU { lu, p } (src/linalg/lu.rs:32-38)."""
    return _dump({"lu": matrix_to_obj(lu), "p": permutation_to_obj(ipiv)})


def lu_from_json(s: str):
    """(lu, ipiv) of a square LU; a non-square factor or a permutation of
    another dimension is refused."""
    o = json.loads(s)
    lu, p = matrix_from_obj(o["lu"], "lu"), permutation_from_obj(o["p"], "p")
    _dim(p, _square(lu, "lu"), "p")
    return lu, p


def full_piv_lu_to_json(lu, ipiv, jpiv) -> str:
    """FullPivLU { lu, p, q } (src/linalg/full_piv_lu.rs:32-39)."""
    return _dump({"lu": matrix_to_obj(lu), "p": permutation_to_obj(ipiv), "q": permutation_to_obj(jpiv)})


def full_piv_lu_from_json(s: str):
    o = json.loads(s)
    lu, p, q = (matrix_from_obj(o["lu"], "lu"), permutation_from_obj(o["p"], "p"),
                permutation_from_obj(o["q"], "q"))
    n = _square(lu, "lu")
    _dim(p, n, "p")
    _dim(q, n, "q")
    return lu, p, q


def qr_to_json(qr, diag) -> str:
    """QR { qr, diag } (src/linalg/qr.rs:34-40)."""
    return _dump({"qr": matrix_to_obj(qr), "diag": matrix_to_obj(np.asarray(diag).reshape(-1, 1))})


def qr_from_json(s: str):
    """(qr, diag) of an m x n QR; diag holds min(m, n) entries (qr.rs:60-62)."""
    o = json.loads(s)
    qr, diag = matrix_from_obj(o["qr"], "qr"), matrix_from_obj(o["diag"], "diag")
    if diag.shape[1] != 1:
        raise ValueError("diag: expected a column vector")
    _dim(diag, min(qr.shape), "diag")
    return qr, diag[:, 0].copy()


def col_piv_qr_to_json(qr, jpiv, diag) -> str:
    """ColPivQR { col_piv_qr, p, diag } (src/linalg/col_piv_qr.rs:36-43)."""
    return _dump({"col_piv_qr": matrix_to_obj(qr), "p": permutation_to_obj(jpiv),
                  "diag": matrix_to_obj(np.asarray(diag).reshape(-1, 1))})


def col_piv_qr_from_json(s: str):
    o = json.loads(s)
    qr, p, diag = (matrix_from_obj(o["col_piv_qr"], "col_piv_qr"), permutation_from_obj(o["p"], "p"),
                   matrix_from_obj(o["diag"], "diag"))
    n = _square(qr, "col_piv_qr")
    if diag.shape[1] != 1:
        raise ValueError("diag: expected a column vector")
    _dim(p, n, "p")
    _dim(diag, n, "diag")
    return qr, p, diag[:, 0].copy()


def cholesky_to_json(chol) -> str:
    """Cholesky { chol } (src/linalg/cholesky.rs:28-33): the factor with its
    strict upper part as stored."""
    return _dump({"chol": matrix_to_obj(chol)})


def cholesky_from_json(s: str) -> np.ndarray:
    chol = matrix_from_obj(json.loads(s)["chol"], "chol")
    _square(chol, "chol")
    return chol
