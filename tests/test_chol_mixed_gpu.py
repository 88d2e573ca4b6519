"""GPU checks of the mixed-precision ragged SPD solve (FP32 factor, FP64
refinement): every solution meets the FP64 backward-error target
||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= n eps64, measured by the
oracle's compensated residual; A and B are untouched; matrices that FP32
cannot factor fall back to FP64 and are still solved; non-SPD matrices report
nalgebra's None (info = failing column)."""
import numpy as np
import pytest

import oracle as O
from nalgebra_gb300 import _lib
from nalgebra_gb300 import workloads as W
from tests.conftest import EPS64

pytestmark = pytest.mark.gpu
FLAG_VERIFY = 8


def _mixed(cuda, ns, a_flat, b_flat, nrhs, flags=0, max_iter=0):
    torch = cuda
    ns = np.asarray(ns, dtype=np.int32)
    count = ns.size
    aoff = np.concatenate([[0], np.cumsum(ns.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
    boff = np.concatenate([[0], np.cumsum(ns.astype(np.int64) * nrhs)[:-1]]).astype(np.int64)
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    A, B = d(a_flat), d(b_flat)
    X = torch.full_like(B, np.nan)
    dns, daoff, dboff = d(ns), d(aoff), d(boff)
    order = d(np.argsort(-ns, kind="stable").astype(np.int32))
    info = torch.full((count,), -7, dtype=torch.int32, device="cuda")
    iters = torch.zeros(count, dtype=torch.int32, device="cuda")
    total = int(a_flat.size)
    ws = torch.zeros(_lib.load().nacu_mixed_workspace_bytes(count, total), dtype=torch.uint8, device="cuda")
    _lib.call("nacu_dposv_ragged_mixed", count, int(ns.max()), dns.data_ptr(), daoff.data_ptr(), A.data_ptr(), nrhs,
              dboff.data_ptr(), B.data_ptr(), X.data_ptr(), info.data_ptr(), iters.data_ptr(), order.data_ptr(),
              total, ws.data_ptr(), ws.numel(), 0.0, max_iter, 0.0, flags, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return (A.cpu().numpy(), B.cpu().numpy(), X.cpu().numpy(), info.cpu().numpy(), iters.cpu().numpy(), aoff, boff)


@pytest.mark.parametrize("flags", [0, FLAG_VERIFY])
def test_workload_slice_meets_fp64_backward_error(cuda, flags):
    w = W.ragged_spd(400, 8, 256, nrhs=4, seed=3)
    ns = w["ns"]
    A, B, X, info, iters, aoff, boff = _mixed(cuda, ns, w["a_flat"], w["b_flat"], 4, flags)
    assert np.array_equal(A, w["a_flat"]) and np.array_equal(B, w["b_flat"])
    assert np.all(info == 0)
    assert np.all(iters > 0), "no FP64 fallback expected on these well-conditioned SPD matrices"
    _, xo, _, _ = O.posv_ragged(ns, w["a_offsets"], w["a_flat"], w["b_offsets"], w["b_flat"], 4)
    worst = 0.0
    for s in range(ns.size):
        n = int(ns[s])
        a = w["a_flat"][aoff[s]:aoff[s] + n * n].reshape(n, n).T
        a = np.tril(a) + np.tril(a, -1).T
        x = X[boff[s]:boff[s] + 4 * n].reshape(4, n).T
        b = w["b_flat"][boff[s]:boff[s] + 4 * n].reshape(4, n).T
        worst = max(worst, O.backward_error(a, x, b) / (n * EPS64))
    assert worst <= 1.0, worst
    assert np.allclose(X, xo, rtol=1e-12, atol=1e-14)  # forward error ~ cond * eps, cond <= 5 here
    if flags == FLAG_VERIFY:
        assert np.all(iters >= 2)


def test_fp32_breakdown_falls_back_to_fp64(cuda):
    eps = 1e-9
    m_near = np.array([[1.0, 1.0 - eps], [1.0 - eps, 1.0]])     # SPD in FP64, singular in FP32
    m_big = 1e200 * np.array([[4.0, 1.0], [1.0, 3.0]])          # overflows FP32
    m_tiny = 1e-200 * np.array([[4.0, 1.0], [1.0, 3.0]])        # underflows FP32
    m_bad = np.array([[1.0, 2.0], [2.0, 1.0]])                   # not SPD at all
    rng = np.random.default_rng(0)
    bm = rng.standard_normal((30, 30))
    m_ok = bm @ bm.T + 30 * np.eye(30)
    mats = [m_near, m_big, m_tiny, m_bad, m_ok]
    ns = [m.shape[0] for m in mats]
    a_flat = np.concatenate([m.ravel(order="F") for m in mats])
    b_flat = rng.standard_normal(sum(ns))
    A, B, X, info, iters, aoff, boff = _mixed(cuda, ns, a_flat, b_flat, 1)
    assert list(info) == [0, 0, 0, 2, 0]
    assert iters[0] < 0 and iters[1] < 0 and iters[2] < 0 and iters[4] > 0
    for s in (0, 1, 2, 4):
        n = ns[s]
        a = mats[s]
        x = X[boff[s]:boff[s] + n]
        b = b_flat[boff[s]:boff[s] + n]
        assert O.backward_error(a, x, b) <= n * EPS64, s


def test_max_iter_one_forces_fallback_but_stays_correct(cuda):
    w = W.ragged_spd(20, 8, 64, nrhs=2, seed=5)
    A, B, X, info, iters, aoff, boff = _mixed(cuda, w["ns"], w["a_flat"], w["b_flat"], 2, 0, max_iter=1)
    assert np.all(info == 0)
    _, xo, _, _ = O.posv_ragged(w["ns"], w["a_offsets"], w["a_flat"], w["b_offsets"], w["b_flat"], 2)
    assert np.allclose(X, xo, rtol=1e-12, atol=1e-14)


def test_mirror_solve_refined_and_graph_capture(cuda):
    """CholeskyBatch.solve_refined (the precision form through the public
    mirror) and its CUDA-graph capture give FP64-accurate solutions."""
    from nalgebra_gb300 import DeviceBatch, Graph, synchronize
    w = W.ragged_spd(50, 8, 200, nrhs=4, seed=9)
    mats = [w["a_flat"][o:o + k * k].reshape(k, k).T for o, k in zip(w["a_offsets"], w["ns"])]
    rhs = [w["b_flat"][o:o + 4 * k].reshape(4, k).T for o, k in zip(w["b_offsets"], w["ns"])]
    chol = DeviceBatch.from_numpy(mats).cholesky()
    b = DeviceBatch.from_numpy(rhs)
    out = b.clone_owned()
    chol.solve_refined_into(b, out)
    g = Graph()
    with g.capture():
        chol.solve_refined_into(b, out)
    out.data.zero_()
    g.replay()
    synchronize()
    xs = out.to_numpy()
    for m, r, x in zip(mats, rhs, xs):
        assert O.backward_error(m, x, r) <= m.shape[0] * EPS64


def test_reads_only_the_lower_triangle(cuda):
    """nalgebra's Cholesky reads only the lower triangle (cholesky.rs:221-272):
    NaN in the strict upper triangle leaves every result bit-identical."""
    w = W.ragged_spd(60, 8, 200, nrhs=4, seed=11)
    ns, aoff = w["ns"], w["a_offsets"]
    poisoned = w["a_flat"].copy()
    for s in range(ns.size):
        n = int(ns[s])
        m = poisoned[aoff[s]:aoff[s] + n * n].reshape(n, n)  # row-major view of the column-major matrix
        m[np.tril_indices(n, -1)] = np.nan                   # (i > j) here is column i, row j < i: A's strict upper part
    _, _, X0, info0, it0, _, _ = _mixed(cuda, ns, w["a_flat"], w["b_flat"], 4)
    _, _, X1, info1, it1, _, _ = _mixed(cuda, ns, poisoned, w["b_flat"], 4)
    assert np.array_equal(info0, info1) and np.array_equal(it0, it1)
    assert np.array_equal(X0.view(np.uint64), X1.view(np.uint64))


@pytest.mark.parametrize("scale", [1e-36, 1e-20, 1e20, 1e36])
def test_extreme_scales_stay_correct(cuda, scale):
    """Entries near the ends of the FP32 range: the FP32 copy (integer
    conversion of the bit fields in the normal range, the hardware conversion
    outside it), the FP32 row sums of ||A|| (FP64 fallback when they overflow)
    and the refinement still meet the FP64 target, converged or fallen back."""
    rng = np.random.default_rng(int(abs(np.log10(scale))))
    mats = []
    for n in (12, 40, 96):
        bm = rng.standard_normal((n, n))
        mats.append(scale * (bm @ bm.T + n * np.eye(n)))
    ns = [m.shape[0] for m in mats]
    a_flat = np.concatenate([m.ravel(order="F") for m in mats])
    b_flat = scale * rng.standard_normal(sum(ns) * 2)
    A, B, X, info, iters, aoff, boff = _mixed(cuda, ns, a_flat, b_flat, 2)
    assert np.all(info == 0)
    for s, m in enumerate(mats):
        n = ns[s]
        x = X[boff[s]:boff[s] + 2 * n].reshape(2, n).T
        b = b_flat[boff[s]:boff[s] + 2 * n].reshape(2, n).T
        assert np.all(np.isfinite(x))
        assert O.backward_error(m, x, b) <= n * EPS64, (scale, s, iters[s])


@pytest.mark.parametrize("chunks,pinned", [(3, True), (7, False), (1, True)])
def test_host_pipeline_matches_device_call(cuda, chunks, pinned):
    """nacu_dposv_ragged_mixed_host (host arrays, chunked copy-in / solve /
    copy-out on internal streams) gives every system the device call's
    results bit for bit, pinned or pageable host memory."""
    torch = cuda
    w = W.ragged_spd(300, 8, 256, nrhs=4, seed=21)
    ns, aoff, boff = w["ns"], w["a_offsets"], w["b_offsets"]
    A0, B0, X0, info0, it0, _, _ = _mixed(cuda, ns, w["a_flat"], w["b_flat"], 4)

    def host(x):
        t = torch.from_numpy(np.ascontiguousarray(x))
        return t.pin_memory() if pinned else t

    hns, haoff, hboff = host(ns.astype(np.int32)), host(aoff.astype(np.int64)), host(boff.astype(np.int64))
    hA, hB = host(w["a_flat"]), host(w["b_flat"])
    hX = host(np.full(w["b_flat"].size, np.nan))
    hinfo = host(np.full(ns.size, -7, dtype=np.int32))
    hit = host(np.zeros(ns.size, dtype=np.int32))
    L = _lib.load()
    nbytes = L.nacu_mixed_host_workspace_bytes(ns.size, int(ns.max()), hns.data_ptr(), haoff.data_ptr(),
                                               hboff.data_ptr(), 4, chunks)
    assert nbytes > 0
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    _lib.call("nacu_dposv_ragged_mixed_host", ns.size, int(ns.max()), hns.data_ptr(), haoff.data_ptr(), hA.data_ptr(),
              4, hboff.data_ptr(), hB.data_ptr(), hX.data_ptr(), hinfo.data_ptr(), hit.data_ptr(), chunks,
              ws.data_ptr(), ws.numel(), 0.0, 0, 0.0, 0, stream.cuda_stream)
    stream.synchronize()
    assert np.array_equal(hinfo.numpy(), info0) and np.array_equal(hit.numpy(), it0)
    assert np.array_equal(hX.numpy().view(np.uint64), X0.view(np.uint64))
    assert np.array_equal(hA.numpy(), w["a_flat"]) and np.array_equal(hB.numpy(), w["b_flat"])


def test_host_pipeline_rejects_unordered_offsets(cuda):
    L = _lib.load()
    ns = np.array([4, 4], dtype=np.int32)
    aoff = np.array([16, 0], dtype=np.int64)  # decreasing
    boff = np.array([0, 4], dtype=np.int64)
    assert L.nacu_mixed_host_workspace_bytes(2, 4, ns.ctypes.data, aoff.ctypes.data, boff.ctypes.data, 1, 2) == 0


def test_mirror_host_solve(cuda):
    """cholesky_solve_refined_host (the mirror of the host-memory entry point)
    meets the FP64 backward-error target on a workload slice."""
    from nalgebra_gb300 import cholesky_solve_refined_host
    w = W.ragged_spd(120, 8, 200, nrhs=2, seed=31)
    ns = w["ns"]
    x, info, iters = cholesky_solve_refined_host(ns, w["a_offsets"], w["a_flat"], w["b_offsets"], w["b_flat"], 2,
                                                 chunks=4)
    assert np.all(info == 0) and np.all(iters != 0)
    for s in range(0, ns.size, 7):
        n = int(ns[s])
        a = w["a_flat"][w["a_offsets"][s]:w["a_offsets"][s] + n * n].reshape(n, n).T
        xs = x[w["b_offsets"][s]:w["b_offsets"][s] + 2 * n].reshape(2, n).T
        bs = w["b_flat"][w["b_offsets"][s]:w["b_offsets"][s] + 2 * n].reshape(2, n).T
        assert O.backward_error(a, xs, bs) <= n * EPS64


def test_2000_systems_without_verify_every_system_meets_n_eps(cuda):
    """2000 systems of the ragged SPD workload (n ~ U[8, 256], A = B B^T + n I,
    4 right-hand sides) through nacu_dposv_ragged_mixed WITHOUT
    NACU_FLAG_VERIFY, where the kernel may stop on its predicted convergence
    instead of a last residual: the backward error of EVERY system, with the
    residual by Dot2 on the host, is <= n eps64, and the solutions agree with
    the oracle's FP64 Cholesky::solve (cholesky.rs:122-143)."""
    w = W.ragged_spd(2000, 8, 256, nrhs=4, seed=0)
    ns = w["ns"]
    A, B, X, info, iters, aoff, boff = _mixed(cuda, ns, w["a_flat"], w["b_flat"], 4, 0)
    assert np.all(info == 0) and np.all(iters > 0)
    be = O.ragged_backward_errors(ns, aoff, w["a_flat"], boff, w["b_flat"], X, 4)
    units = be / (ns * EPS64)
    assert np.all(units <= 1.0), (float(units.max()), int(np.sum(units > 1.0)))
    _, xo, _, _ = O.posv_ragged(ns, w["a_offsets"], w["a_flat"], w["b_offsets"], w["b_flat"], 4)
    assert np.allclose(X, xo, rtol=1e-12, atol=1e-14)
