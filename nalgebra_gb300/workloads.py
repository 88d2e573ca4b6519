"""Seeded synthetic inputs for the dense-solve workloads.

nalgebra publishes no benchmark data set; these generators produce the shapes,
sizes and value distributions the workloads are defined by, from a fixed seed,
so the oracle and the GPU always see identical inputs.  Matrices are returned
column-major (each one packed as nalgebra's VecStorage would hold it).

  dense_lu      : `count` n x n systems, A_ij ~ N(0,1) + shift*I, b ~ N(0,1)
                  (shift = n gives the diagonally dominant LU workload: 4096 x 64)
  ragged_spd    : SPD matrices with n ~ U{n_lo..n_hi}, A = B B^T + n I,
                  B ~ N(0,1), nrhs right-hand sides ~ N(0,1)
                  (20000 matrices, n in [8, 256], 4 RHS)
  conditioned   : one dense system A = U diag(s) V^T, U, V orthogonal (QR of
                  N(0,1)), s log-uniform between 1 and 1/cond (cond 1e2, 1e5,
                  1e8; n = 4096, 8192), b ~ N(0,1)
"""
from __future__ import annotations

import numpy as np


def dense_lu(count: int, n: int, nrhs: int = 1, shift: float | None = None, seed: int = 0):
    """Returns (a, b): a is (count, n*n), row s the column-major image of
    system s (element (r, c) at a[s, c*n + r]); b is (count, n*nrhs), also
    column-major per system."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((count, n, n))
    if shift is None:
        shift = float(n)
    a[:, np.arange(n), np.arange(n)] += shift
    b = rng.standard_normal((count, nrhs, n))
    colmaj = np.ascontiguousarray(np.transpose(a, (0, 2, 1))).reshape(count, n * n)
    return colmaj, b.reshape(count, n * nrhs).copy()


def dense_lu_matrix(colmaj_row: np.ndarray, n: int) -> np.ndarray:
    """The n x n matrix held column-major in one row of dense_lu's output."""
    return colmaj_row.reshape(n, n).T


def ragged_sizes(count: int, n_lo: int, n_hi: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.integers(n_lo, n_hi + 1, size=count).astype(np.int32)


def ragged_spd(count: int, n_lo: int, n_hi: int, nrhs: int = 4, seed: int = 0):
    """Host generation (numpy).  Returns dict with ns, a_offsets, a_flat,
    b_offsets, b_flat."""
    ns = ragged_sizes(count, n_lo, n_hi, seed)
    rng = np.random.default_rng(seed + 1)
    sizes = ns.astype(np.int64) ** 2
    aoff = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    boff = np.concatenate([[0], np.cumsum(ns.astype(np.int64) * nrhs)[:-1]]).astype(np.int64)
    a_flat = np.empty(int(sizes.sum()), dtype=np.float64)
    b_flat = rng.standard_normal(int(ns.astype(np.int64).sum() * nrhs))
    for s, n in enumerate(ns):
        B = rng.standard_normal((n, n))
        A = B @ B.T + n * np.eye(n)
        a_flat[aoff[s]:aoff[s] + n * n] = A.ravel(order="F")
    return dict(ns=ns, a_offsets=aoff, a_flat=a_flat, b_offsets=boff, b_flat=b_flat, nrhs=nrhs)


def ragged_spd_torch(count: int, n_lo: int, n_hi: int, nrhs: int = 4, seed: int = 0, device="cuda"):
    """The same distribution generated on the GPU with PyTorch (input
    preparation only, for the large timed workloads).  Returns host numpy
    ns/offsets and device tensors for the packed data."""
    import torch

    ns = ragged_sizes(count, n_lo, n_hi, seed)
    sizes = ns.astype(np.int64) ** 2
    aoff = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    boff = np.concatenate([[0], np.cumsum(ns.astype(np.int64) * nrhs)[:-1]]).astype(np.int64)
    g = torch.Generator(device=device)
    g.manual_seed(seed + 1)
    a_flat = torch.empty(int(sizes.sum()), dtype=torch.float64, device=device)
    b_flat = torch.randn(int(ns.astype(np.int64).sum() * nrhs), dtype=torch.float64, device=device, generator=g)
    for n in np.unique(ns):
        idx = np.nonzero(ns == n)[0]
        n = int(n)
        chunk = max(1, (8 << 20) // (n * n))
        for c0 in range(0, idx.size, chunk):
            sel = idx[c0:c0 + chunk]
            B = torch.randn((sel.size, n, n), dtype=torch.float64, device=device, generator=g)
            A = torch.bmm(B, B.transpose(1, 2))
            A.diagonal(dim1=1, dim2=2).add_(float(n))
            # A is symmetric, so its row-major image is its column-major image
            dst = torch.from_numpy(aoff[sel]).to(device)
            ar = torch.arange(n * n, device=device)
            a_flat[(dst[:, None] + ar[None, :]).reshape(-1)] = A.reshape(-1)
    return dict(ns=ns, a_offsets=aoff, a_flat=a_flat, b_offsets=boff, b_flat=b_flat, nrhs=nrhs)


def ragged_ls(count: int, m_lo: int, m_hi: int, n: int = 64, seed: int = 0):
    """Tall-skinny least-squares problems: m ~ U{m_lo..m_hi} rows, n columns,
    A and b iid N(0,1), column-major.  Returns dict with ms, a_offsets, a_flat,
    b_offsets, b_flat, n."""
    rng = np.random.default_rng(seed)
    ms = rng.integers(m_lo, m_hi + 1, size=count).astype(np.int32)
    sizes = ms.astype(np.int64) * n
    aoff = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    boff = np.concatenate([[0], np.cumsum(ms.astype(np.int64))[:-1]]).astype(np.int64)
    a_flat = rng.standard_normal(int(sizes.sum()))
    b_flat = rng.standard_normal(int(ms.astype(np.int64).sum()))
    return dict(ms=ms, a_offsets=aoff, a_flat=a_flat, b_offsets=boff, b_flat=b_flat, n=n)


def spd_uniform(count: int, n: int, seed: int = 0, dtype=np.float64):
    """Equal-order SPD batch for the adjoint workload: A = B B^T + n I with
    B ~ N(0,1), right-hand sides b and loss weights w ~ N(0,1).  Returns
    (A (count, n*n) column-major rows, b (count, n), w (count, n))."""
    rng = np.random.default_rng(seed)
    bm = rng.standard_normal((count, n, n))
    a = bm @ np.transpose(bm, (0, 2, 1)) + n * np.eye(n)
    b = rng.standard_normal((count, n))
    w = rng.standard_normal((count, n))
    return (np.ascontiguousarray(a.reshape(count, n * n)).astype(dtype), b.astype(dtype), w.astype(dtype))


def _sigma(n: int, cond: float, rng) -> np.ndarray:
    u = rng.uniform(0.0, 1.0, n)
    u[0], u[-1] = 0.0, 1.0  # the extremes pin the condition number exactly
    return cond ** (-u)


def conditioned(n: int, cond: float, seed: int = 0):
    """(A column-major as an (n, n) Fortran array, b): A = U diag(s) V^T with
    U, V the Q factors of N(0,1) matrices and s log-uniform in [1/cond, 1]."""
    rng = np.random.default_rng(seed)
    u, _ = np.linalg.qr(rng.standard_normal((n, n)))
    v, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = _sigma(n, cond, rng)
    a = (u * s) @ v.T
    b = rng.standard_normal(n)
    return np.asfortranarray(a), b


def conditioned_torch(n: int, cond: float, seed: int = 0, device="cuda"):
    """The same distribution as `conditioned`, generated on the device (the
    QR factorizations of an 8192 x 8192 matrix are minutes on the host).
    Returns (A as a column-major flat FP64 device tensor, b device tensor)."""
    import torch

    g = torch.Generator(device=device).manual_seed(seed)
    gu = torch.randn(n, n, dtype=torch.float64, device=device, generator=g)
    gv = torch.randn(n, n, dtype=torch.float64, device=device, generator=g)
    try:
        u, _ = torch.linalg.qr(gu)
        v, _ = torch.linalg.qr(gv)
    except RuntimeError:  # torch's linalg library unavailable (e.g. under a profiler): QR on the host
        u = torch.from_numpy(np.linalg.qr(gu.cpu().numpy())[0]).to(device)
        v = torch.from_numpy(np.linalg.qr(gv.cpu().numpy())[0]).to(device)
    s = torch.from_numpy(_sigma(n, cond, np.random.default_rng(seed))).to(device)
    a = (u * s) @ v.T
    b = torch.randn(n, dtype=torch.float64, device=device, generator=g)
    return a.t().contiguous().reshape(-1), b  # a.t() row-major == a column-major
