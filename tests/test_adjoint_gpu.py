"""GPU checks of the adjoint of the batched Cholesky solve + log-determinant.

Loss l = w^T x + logdet A with x = A^-1 b.  The backward kernels' db and the
lower-triangle gradient dA are compared with (1) the FP64 analytic gradient
built from the CPU oracle (nalgebra's Cholesky, solve and inverse) and (2)
central finite differences with h = 1e-6 on the lower-triangle entries of A
(perturbing theta_ij perturbs A_ij and A_ji together, as nalgebra reads only
the lower triangle).  Store and recompute forms must agree."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import _lib
from nalgebra_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _gpu(cuda, a, b, w, n, dtype, recompute):
    torch = cuda
    count = a.shape[0]
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    pre = "d" if dtype == np.float64 else "s"
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x, dtype=dtype)).cuda()
    A, B, Wt = d(a), d(b), d(w)
    X = torch.zeros((count, n), dtype=tdt, device="cuda")
    L = torch.zeros_like(A)
    logdet = torch.zeros(count, dtype=tdt, device="cuda")
    info = torch.full((count,), -7, dtype=torch.int32, device="cuda")
    dA = torch.full_like(A, np.nan)
    db = torch.zeros_like(X)
    s = torch.cuda.current_stream().cuda_stream
    _lib.call(f"nacu_{pre}posv_logdet_forward", n, A.data_ptr(), n * n, B.data_ptr(), X.data_ptr(),
              0 if recompute else L.data_ptr(), logdet.data_ptr(), info.data_ptr(), count, s)
    src = A if recompute else L
    _lib.call(f"nacu_{pre}posv_logdet_backward", n, src.data_ptr(), n * n, 1 if recompute else 0, X.data_ptr(),
              Wt.data_ptr(), None, dA.data_ptr(), db.data_ptr(), info.data_ptr(), count, s)
    torch.cuda.synchronize()
    return (X.cpu().numpy().astype(np.float64), logdet.cpu().numpy().astype(np.float64),
            dA.cpu().numpy().astype(np.float64).reshape(count, n, n).transpose(0, 2, 1),
            db.cpu().numpy().astype(np.float64), info.cpu().numpy())


def _analytic(a_colmaj, b, w, n):
    """FP64 analytic gradient from the oracle (nalgebra's Cholesky::inverse =
    solve(I), src/linalg/cholesky.rs:147-153)."""
    A = a_colmaj.reshape(n, n).T
    l, info = O.cholesky(A)
    assert info == 0
    x = O.cholesky_solve(l, b)
    v = O.cholesky_solve(l, w)
    ainv = O.cholesky_solve(l, np.eye(n))
    G = -np.outer(v, x) - np.outer(x, v) + 2 * ainv
    G[np.diag_indices(n)] = -v * x + np.diag(ainv)
    return x, O.cholesky_ln_determinant(l), np.tril(G), v


def _loss(A, b, w):
    l, info = O.cholesky(A)
    return float(w @ O.cholesky_solve(l, b) + O.cholesky_ln_determinant(l))


@pytest.mark.parametrize("recompute", [0, 1])
def test_f64_gradient_matches_analytic_and_fd(cuda, recompute):
    n = 128
    a, b, w = W.spd_uniform(6, n, seed=1)
    X, logdet, dA, db, info = _gpu(cuda, a, b, w, n, np.float64, recompute)
    assert np.all(info == 0)
    for s in range(6):
        x, ld, G, v = _analytic(a[s], b[s], w[s], n)
        assert np.allclose(X[s], x, rtol=1e-12, atol=1e-14)
        assert abs(logdet[s] - ld) <= 1e-12 * abs(ld)
        assert np.allclose(db[s], v, rtol=1e-11, atol=1e-14)
        assert np.allclose(dA[s], G, rtol=1e-10, atol=1e-13)
        assert np.all(np.triu(dA[s], 1) == 0)
    # central differences, h = 1e-6, on a few lower-triangle entries
    rng = np.random.default_rng(0)
    A0 = a[0].reshape(n, n).T.copy()
    h = 1e-6
    for (i, j) in [(0, 0), (5, 5), (17, 3), (100, 40), (127, 0), (64, 63)]:
        Ap, Am = A0.copy(), A0.copy()
        Ap[i, j] += h
        Am[i, j] -= h
        if i != j:
            Ap[j, i] += h
            Am[j, i] -= h
        fd = (_loss(Ap, b[0], w[0]) - _loss(Am, b[0], w[0])) / (2 * h)
        assert abs(fd - dA[0][i, j]) <= 1e-5 * max(1.0, abs(fd)) + 1e-7, (i, j, fd, dA[0][i, j])
    # db by central differences on b
    for i in (0, 63, 127):
        bp, bm = b[0].copy(), b[0].copy()
        bp[i] += h
        bm[i] -= h
        fd = (_loss(A0, bp, w[0]) - _loss(A0, bm, w[0])) / (2 * h)
        assert abs(fd - db[0][i]) <= 1e-5 * max(1.0, abs(fd)) + 1e-7


def test_store_and_recompute_agree(cuda):
    n = 96
    a, b, w = W.spd_uniform(8, n, seed=2)
    r0 = _gpu(cuda, a, b, w, n, np.float64, 0)
    r1 = _gpu(cuda, a, b, w, n, np.float64, 1)
    assert np.allclose(r0[2], r1[2], rtol=1e-13, atol=1e-15)
    assert np.allclose(r0[3], r1[3], rtol=1e-13, atol=1e-15)


def test_f32_gradient_against_fp64_analytic(cuda):
    n = 128
    a, b, w = W.spd_uniform(4, n, seed=3)
    X, logdet, dA, db, info = _gpu(cuda, a.astype(np.float32), b.astype(np.float32), w.astype(np.float32), n,
                                   np.float32, 0)
    assert np.all(info == 0)
    for s in range(4):
        x, ld, G, v = _analytic(a[s], b[s], w[s], n)
        assert np.linalg.norm(dA[s] - G) <= 1e-4 * np.linalg.norm(G)
        assert np.linalg.norm(db[s] - v) <= 1e-4 * np.linalg.norm(v)
        assert abs(logdet[s] - ld) <= 1e-5 * abs(ld)


@pytest.mark.parametrize("n", [1, 2, 7, 33])
def test_small_orders_and_not_spd(cuda, n):
    a, b, w = W.spd_uniform(3, n, seed=n)
    a[1] = -a[1]  # not SPD: info = 1, no gradient written
    X, logdet, dA, db, info = _gpu(cuda, a, b, w, n, np.float64, 1)
    assert info[1] == 1 and info[0] == 0 and info[2] == 0
    for s in (0, 2):
        x, ld, G, v = _analytic(a[s], b[s], w[s], n)
        assert np.allclose(dA[s], G, rtol=1e-10, atol=1e-13)


@pytest.mark.parametrize("recompute", [False, True])
def test_mirror_reverse_mode_with_logdet_cotangent(cuda, recompute):
    """PosvLogdet.backward(x_bar, logdet_bar) for a general log-det cotangent g:
    A_bar = -sym(v x^T) + g A^-1 on the lower triangle, b_bar = A^-1 x_bar;
    checked against the oracle-built analytic gradient and against central
    differences of the loss sum_s w_s^T x_s + g_s logdet A_s."""
    torch = cuda
    from nalgebra_gb300 import PosvLogdet

    n, count = 24, 5
    a, b, w = W.spd_uniform(count, n, seed=31)
    g = np.array([0.5, -1.0, 2.0, 0.0, 3.0])
    op = PosvLogdet(n, count, "float64", recompute=recompute)
    x, logdet = op.forward(torch.from_numpy(a), torch.from_numpy(b))
    dA, db = op.backward(torch.from_numpy(w), torch.from_numpy(g))
    assert op.is_ok().all()
    dA = dA.to_numpy().reshape(count, n, n).transpose(0, 2, 1)
    db = db.to_numpy()
    for s in range(count):
        A = a[s].reshape(n, n).T
        l, _ = O.cholesky(A)
        xs = O.cholesky_solve(l, b[s])
        v = O.cholesky_solve(l, w[s])
        ainv = O.cholesky_solve(l, np.eye(n))
        G = -np.outer(v, xs) - np.outer(xs, v) + 2 * g[s] * ainv
        G[np.diag_indices(n)] = -v * xs + g[s] * np.diag(ainv)
        assert np.allclose(np.tril(dA[s]), np.tril(G), rtol=1e-9, atol=1e-12)
        assert np.all(np.triu(dA[s], 1) == 0.0)
        assert np.allclose(db[s], v, rtol=1e-10, atol=1e-13)
        # central differences on a few lower-triangle entries
        h = 1e-6

        def loss(M):
            lm, _ = O.cholesky(M)
            return float(w[s] @ O.cholesky_solve(lm, b[s]) + g[s] * O.cholesky_ln_determinant(lm))

        for (i, j) in [(0, 0), (5, 2), (n - 1, 0), (n - 1, n - 1)]:
            Ap, Am = A.copy(), A.copy()
            Ap[i, j] += h
            Am[i, j] -= h
            if i != j:
                Ap[j, i] += h
                Am[j, i] -= h
            fd = (loss(Ap) - loss(Am)) / (2 * h)
            assert abs(fd - dA[s][i, j]) <= 1e-5 * max(1.0, abs(fd))
