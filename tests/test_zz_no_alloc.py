"""The allocation-free ragged Cholesky entry point (nacu_dposv_ragged_noalloc).

It serves hosts that cannot allocate device memory when they solve: it keeps
its scratch in a fixed array inside the library instead of asking the caller
for a workspace.  This test calls it twice in a row through the C ABI and
checks both results against the regular entry point (nacu_dposv_ragged, with
a caller workspace) on the same inputs.  The file sorts last so that a run
stopping at the first failure has already run every other test.
"""
import numpy as np
import pytest

from nalgebra_gb300 import _lib
from nalgebra_gb300 import workloads as W
from tests.conftest import EPS64

pytestmark = pytest.mark.gpu


def _run(torch, w, noalloc):
    ns = w["ns"]
    count = ns.size
    d = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    A, B = d(w["a_flat"]), d(w["b_flat"])
    dns, daoff, dboff = d(ns), d(w["a_offsets"]), d(w["b_offsets"])
    info = torch.full((count,), -7, dtype=torch.int32, device="cuda")
    logdet = torch.zeros(count, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    n_max = int(ns.max())
    if noalloc:
        _lib.call("nacu_dposv_ragged_noalloc", count, n_max, dns.data_ptr(), daoff.data_ptr(), A.data_ptr(), 4,
                  dboff.data_ptr(), B.data_ptr(), info.data_ptr(), logdet.data_ptr(), 0.0, 0, s)
    else:
        order = d(np.argsort(-ns, kind="stable").astype(np.int32))
        ws = torch.zeros(_lib.load().nacu_ragged_workspace_bytes(count), dtype=torch.uint8, device="cuda")
        _lib.call("nacu_dposv_ragged", count, n_max, dns.data_ptr(), daoff.data_ptr(), A.data_ptr(), 4,
                  dboff.data_ptr(), B.data_ptr(), info.data_ptr(), logdet.data_ptr(), order.data_ptr(),
                  ws.data_ptr(), ws.numel(), 0.0, 0, s)
    torch.cuda.synchronize()
    return A.cpu().numpy(), B.cpu().numpy(), info.cpu().numpy(), logdet.cpu().numpy()


def test_noalloc_matches_regular_entry_point_twice(cuda):
    torch = cuda
    w = W.ragged_spd(300, 8, 256, nrhs=4, seed=21)
    ref_a, ref_x, ref_info, ref_ld = _run(torch, w, noalloc=False)
    assert np.all(ref_info == 0)
    for _ in range(2):  # the shared scratch must be reset by every call
        a, x, info, ld = _run(torch, w, noalloc=True)
        assert np.array_equal(info, ref_info)
        # each matrix is factored by one CTA with the same code, so results are
        # equal; the check uses the test suite's FMA-form tolerance
        assert np.allclose(x, ref_x, rtol=1e-12, atol=1e-14)
        assert np.allclose(a, ref_a, rtol=1e-12, atol=1e-14)
        assert np.allclose(ld, ref_ld, rtol=1e-12, atol=0)
    # backward error of one solution, as in the other Cholesky tests
    n = int(w["ns"][0])
    am = w["a_flat"][:n * n].reshape(n, n).T
    xm = x[: 4 * n].reshape(4, n).T
    bm = w["b_flat"][: 4 * n].reshape(4, n).T
    r = bm - am @ xm
    be = np.max(np.abs(r)) / (np.max(np.sum(np.abs(am), 1)) * np.max(np.abs(xm)) + np.max(np.abs(bm)))
    assert be <= 4 * n * EPS64


def test_noalloc_rejects_oversized_batches(cuda):
    L = _lib.load()
    too_many = 65536 + 1
    assert L.nacu_dposv_ragged_noalloc(too_many, 8, 16, 16, 16, 1, 16, 16, 16, 0, 0.0, 0, 0) == -1
    assert b"65536" in L.nacu_last_error()
