"""GPU parity of the ragged persistent Cholesky (factor + solve + log-det)
against the CPU oracle, through the C ABI.

Bar: info identical to nalgebra's Some/None; with NACU_FLAG_EXACT the factor
and the solutions are bit-identical to nalgebra's arithmetic and the
log-determinant agrees to 4 ulps per term (CUDA's log is not correctly
rounded); in the default FMA form ||LL^T - A|| / (||A|| n eps) <= 10,
backward error <= n eps64 and the log-determinant to 1e-12 relative."""
import os

import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import FLAG_EXACT, FLAG_SUBSTITUTE, DeviceBatch, DeviceMatrix, _lib
from nalgebra_gb300 import workloads as W
from tests.conftest import EPS64

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz")


def _posv_ragged(cuda, ns, a_flat, b_flat, nrhs, flags=0, order=None, substitute=0.0, mode="posv"):
    torch = cuda
    ns = np.asarray(ns, dtype=np.int32)
    count = ns.size
    aoff = np.concatenate([[0], np.cumsum(ns.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
    boff = np.concatenate([[0], np.cumsum(ns.astype(np.int64) * nrhs)[:-1]]).astype(np.int64)
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    A, B = d(a_flat), d(b_flat if nrhs else np.zeros(1))
    dns, daoff, dboff = d(ns), d(aoff), d(boff)
    info = torch.full((count,), -7, dtype=torch.int32, device="cuda")
    logdet = torch.zeros(count, dtype=torch.float64, device="cuda")
    ws = torch.zeros(_lib.load().nacu_ragged_workspace_bytes(count), dtype=torch.uint8, device="cuda")
    dorder = d(np.asarray(order, dtype=np.int32)) if order is not None else None
    s = torch.cuda.current_stream().cuda_stream
    n_max = int(ns.max())
    optr = dorder.data_ptr() if dorder is not None else 0
    if mode == "posv":
        _lib.call("nacu_dposv_ragged", count, n_max, dns.data_ptr(), daoff.data_ptr(), A.data_ptr(), nrhs,
                  dboff.data_ptr(), B.data_ptr(), info.data_ptr(), logdet.data_ptr(), optr, ws.data_ptr(),
                  ws.numel(), substitute, flags, s)
    else:
        _lib.call("nacu_dpotrf_ragged", count, n_max, dns.data_ptr(), daoff.data_ptr(), A.data_ptr(),
                  info.data_ptr(), logdet.data_ptr(), optr, ws.data_ptr(), ws.numel(), substitute, flags, s)
        _lib.call("nacu_dpotrs_ragged", count, n_max, dns.data_ptr(), daoff.data_ptr(), A.data_ptr(), nrhs,
                  dboff.data_ptr(), B.data_ptr(), optr, ws.data_ptr(), ws.numel(), flags, s)
    torch.cuda.synchronize()
    return A.cpu().numpy(), B.cpu().numpy(), info.cpu().numpy(), logdet.cpu().numpy(), aoff, boff


@pytest.mark.parametrize("mode", ["posv", "potrf+potrs"])
def test_exact_mode_bit_identical_to_oracle_golden(cuda, mode):
    sizes = [1, 3, 8, 17, 33, 64, 100]
    with np.load(GOLD) as z:
        a_flat = np.concatenate([z[f"chol_n{n}_a"].ravel(order="F") for n in sizes])
        b_flat = np.concatenate([z[f"chol_n{n}_b"].ravel(order="F") for n in sizes])
        A, B, info, logdet, aoff, boff = _posv_ragged(cuda, sizes, a_flat, b_flat, 4, FLAG_EXACT, mode=mode)
        assert np.all(info == 0)
        for s, n in enumerate(sizes):
            l = A[aoff[s]:aoff[s] + n * n].reshape(n, n).T
            assert np.array_equal(np.tril(l), np.tril(z[f"chol_n{n}_l"])), n
            assert np.array_equal(np.triu(l, 1), np.triu(z[f"chol_n{n}_a"], 1)), n  # untouched
            x = B[boff[s]:boff[s] + 4 * n].reshape(4, n).T
            assert np.array_equal(x, z[f"chol_n{n}_x"]), n
            ref = z[f"chol_n{n}_logdet"][0]
            assert abs(logdet[s] - ref) <= 4 * n * EPS64 * max(1.0, abs(ref)), n


def test_ragged_workload_slice_fma(cuda):
    """A 600-matrix slice of the ragged SPD workload (n in [8, 256], 4 RHS)."""
    w = W.ragged_spd(600, 8, 256, nrhs=4, seed=0)
    ns = w["ns"]
    order = np.argsort(-ns, kind="stable")
    A, B, info, logdet, aoff, boff = _posv_ragged(cuda, ns, w["a_flat"], w["b_flat"], 4, 0, order=order)
    Lo, Xo, info_o, logdet_o = O.posv_ragged(ns, w["a_offsets"], w["a_flat"], w["b_offsets"], w["b_flat"], 4)
    assert np.array_equal(info, info_o) and np.all(info == 0)
    assert np.allclose(logdet, logdet_o, rtol=1e-12, atol=0)
    worst_be = 0.0
    for s in range(0, 600, 11):
        n = int(ns[s])
        a = w["a_flat"][aoff[s]:aoff[s] + n * n].reshape(n, n).T
        x = B[boff[s]:boff[s] + 4 * n].reshape(4, n).T
        l = np.tril(A[aoff[s]:aoff[s] + n * n].reshape(n, n).T)
        rec = np.linalg.norm(l @ l.T - a) / (np.linalg.norm(a) * n * EPS64)
        assert rec <= 10.0, (s, n, rec)
        worst_be = max(worst_be, O.backward_error(a, x, w["b_flat"][boff[s]:boff[s] + 4 * n].reshape(4, n).T) / (n * EPS64))
    assert worst_be <= 1.0, worst_be
    assert np.allclose(B, Xo, rtol=1e-10, atol=1e-12)


def test_exact_mode_ragged_slice_bit_identical(cuda):
    w = W.ragged_spd(64, 8, 256, nrhs=4, seed=7)
    ns = w["ns"]
    A, B, info, logdet, aoff, boff = _posv_ragged(cuda, ns, w["a_flat"], w["b_flat"], 4, FLAG_EXACT)
    Lo, Xo, info_o, logdet_o = O.posv_ragged(ns, w["a_offsets"], w["a_flat"], w["b_offsets"], w["b_flat"], 4)
    assert np.array_equal(info, info_o)
    assert np.array_equal(A, Lo)
    assert np.array_equal(B, Xo)


def test_not_spd_nan_and_substitute(cuda):
    """cholesky.rs:237-268 and the known answer tests/linalg/cholesky.rs:5-12."""
    mats = [
        np.array([[1.0, np.nan], [1.0, 1e-32]]),           # None; Some with substitute
        np.array([[1.0, 2.0], [2.0, 1.0]]),                # indefinite: info 2
        np.array([[-1.0, 0.0], [0.0, 1.0]]),               # info 1
        np.array([[np.nan, 0.0], [0.0, 1.0]]),             # NaN pivot: info 1
        np.array([[4.0, 0.0], [2.0, 5.0]]),                # SPD (lower read only)
    ]
    ns = [2] * len(mats)
    a_flat = np.concatenate([m.ravel(order="F") for m in mats])
    b_flat = np.ones(2 * len(mats))
    for flags in (0, FLAG_EXACT):
        _, _, info, logdet, _, _ = _posv_ragged(cuda, ns, a_flat, b_flat, 1, flags)
        assert list(info) == [2, 2, 1, 1, 0]
        assert np.all(np.isnan(logdet[:4])) and np.isfinite(logdet[4])
    _, _, info, _, _, _ = _posv_ragged(cuda, ns, a_flat, b_flat, 1, FLAG_SUBSTITUTE, substitute=1e-8)
    assert info[0] == 0
    for s, m in enumerate(mats):
        _, io = O.cholesky(m, substitute=1e-8)
        assert (info[s] == 0) == (io == 0)


def test_single_matrix_plain_launch_and_api(cuda):
    rng = np.random.default_rng(4)
    n = 70
    bm = rng.standard_normal((n, n))
    a = bm @ bm.T + n * np.eye(n)
    rhs = rng.standard_normal((n, 3))
    ch = DeviceMatrix.from_numpy(a).cholesky(flags=FLAG_EXACT)
    assert ch is not None
    x = ch.solve(DeviceMatrix.from_numpy(rhs)).to_numpy()
    l_o, _ = O.cholesky(a)
    assert np.array_equal(ch.l(), np.tril(l_o))
    assert np.array_equal(x, O.cholesky_solve(l_o, rhs))
    assert abs(ch.ln_determinant() - O.cholesky_ln_determinant(l_o)) <= 4 * n * EPS64 * abs(O.cholesky_ln_determinant(l_o))
    assert DeviceMatrix.from_numpy(np.array([[1.0, 2.0], [2.0, 1.0]])).cholesky() is None


def test_device_batch_cholesky_api(cuda):
    rng = np.random.default_rng(8)
    mats, rhss = [], []
    for n in [5, 40, 9, 130]:
        bm = rng.standard_normal((n, n))
        mats.append(bm @ bm.T + n * np.eye(n))
        rhss.append(rng.standard_normal((n, 2)))
    batch = DeviceBatch.from_numpy(mats)
    chol = batch.cholesky()
    xs = chol.solve(DeviceBatch.from_numpy(rhss)).to_numpy()
    assert np.all(chol.is_ok())
    for m, r, x in zip(mats, rhss, xs):
        assert O.backward_error(m, x, r) <= m.shape[0] * EPS64
    ld = chol.ln_determinant()
    assert np.allclose(ld, [np.linalg.slogdet(m)[1] for m in mats], rtol=1e-12)


def test_cuda_graph_replay_matches_direct_launch(cuda):
    """The ragged persistent launch captured in a CUDA graph and replayed (the
    batching form): same results as the direct call, on every replay."""
    torch = cuda
    w = W.ragged_spd(200, 8, 256, nrhs=4, seed=12)
    mats = [w["a_flat"][o:o + k * k].reshape(k, k).T for o, k in zip(w["a_offsets"], w["ns"])]
    rhs = [w["b_flat"][o:o + 4 * k].reshape(4, k).T for o, k in zip(w["b_offsets"], w["ns"])]
    ref_batch = DeviceBatch.from_numpy(mats)
    ref = ref_batch.cholesky().solve(DeviceBatch.from_numpy(rhs)).to_numpy()
    batch = DeviceBatch.from_numpy(mats)
    b = DeviceBatch.from_numpy(rhs)
    a0, b0 = batch.data.clone(), b.data.clone()
    chol = batch.cholesky()
    g = chol.capture(b)
    for _ in range(2):
        batch.data.copy_(a0)
        b.data.copy_(b0)
        g.replay()
        torch.cuda.synchronize()
        got = b.to_numpy()
        for x, y in zip(got, ref):
            assert np.array_equal(x, y)
        assert np.all(chol.info.to_numpy() == 0)
