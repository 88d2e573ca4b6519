"""The mirror's host logic on the CPU: which C-ABI entry point each nalgebra
method reaches, with which sizes, strides, pointer offsets and stream.  The
library's plumbing entry points (nacu_malloc, nacu_memcpy, ...) are replaced
by a fake that keeps "device" buffers in host memory, and the compute entry
points are recorded instead of run; the workspace-size queries are the real
library's.  Nothing here needs a GPU."""
import ctypes as C

import numpy as np
import pytest

from nalgebra_gb300 import _lib, build


class _FakeLib:
    """Plumbing on host memory; compute entry points recorded, returning 0."""

    def __init__(self, real):
        self.real = real
        self.calls = []
        self.blocks = {}

    def _alloc(self, pp, nbytes):
        buf = np.zeros(max(int(nbytes), 1), np.uint8)
        self.blocks[buf.ctypes.data] = buf
        pp._obj.value = buf.ctypes.data
        return 0

    def nacu_malloc(self, pp, nbytes):
        return self._alloc(pp, nbytes)

    def nacu_host_alloc(self, pp, nbytes):
        return self._alloc(pp, nbytes)

    def nacu_free(self, p):
        self.blocks.pop(p, None)
        return 0

    nacu_host_free = nacu_free

    def nacu_memcpy(self, dst, src, nbytes, stream):
        C.memmove(dst, src, nbytes)
        self.calls.append(("nacu_memcpy", (nbytes, stream)))
        return 0

    def nacu_memset(self, p, value, nbytes, stream):
        C.memset(p, value, nbytes)
        return 0

    def nacu_device_count(self, pc):
        pc._obj.value = 1
        return 0

    def nacu_stream_create(self, ps):
        ps._obj.value = 0x5000 + len(self.calls)
        return 0

    def nacu_graph_end_capture(self, stream, pg):
        self.calls.append(("nacu_graph_end_capture", (stream,)))
        pg._obj.value = 0x7000
        return 0

    def __getattr__(self, name):
        if name.endswith("_workspace_bytes") or name in ("nacu_last_error", "nacu_version"):
            return getattr(self.real, name)

        def record(*args):
            self.calls.append((name, args))
            return 0

        return record

    def named(self, name):
        return [a for n, a in self.calls if n == name]


@pytest.fixture
def fake(monkeypatch):
    build.build()
    real = _lib.load()
    f = _FakeLib(real)
    from nalgebra_gb300 import _device

    monkeypatch.setattr(_lib, "load", lambda path=None: f)
    monkeypatch.setattr(_lib, "call", lambda name, *args: _lib.check(getattr(f, name)(*args), name))
    monkeypatch.setattr(_device, "require_gpu", lambda: None)
    yield f
    import gc

    gc.collect()  # buffers on the fake's host memory are released while it is still in place


def test_round_trip_keeps_nalgebra_column_major_layout(fake):
    import nalgebra_gb300 as ng

    a = np.arange(12, dtype=np.float64).reshape(3, 4)
    m = ng.DeviceMatrix.from_numpy(a)
    assert m.shape == (3, 4) and np.array_equal(m.data.to_numpy(), a.ravel(order="F"))
    assert np.array_equal(m.to_numpy(), a)
    b = ng.DeviceBatch.from_numpy([a, a[:2, :3]])
    assert list(b._d_rows.to_numpy()) == [3, 2] and list(b._d_off.to_numpy()) == [0, 12]
    assert all(np.array_equal(x, y) for x, y in zip(b.to_numpy(), [a, a[:2, :3]]))


def test_qr_routes_by_shape(fake):
    import nalgebra_gb300 as ng

    q = ng.DeviceMatrix.from_numpy(np.eye(4)).qr(flags=ng.FLAG_EXACT)
    (args,) = fake.named("nacu_dqr_batched")
    assert args[0] == 4 and args[3] == 16 and args[8] == 1 and args[9] == ng.FLAG_EXACT and not q.large
    for m, n in ((200, 200), (100, 500), (500, 100)):
        q = ng.DeviceMatrix.from_numpy(np.ones((m, n))).qr()
        args = fake.named("nacu_dqr")[-1]
        assert args[:2] == (m, n) and args[3] == m and args[2] == q.qr.data.data_ptr() and q.large
        assert q.diag.numel() == min(m, n)
    # a tall factor's least-squares solve: one call for all columns, ldb = m, the real workspace size
    b = ng.DeviceMatrix.from_numpy(np.ones((500, 3)))
    t = ng.DeviceMatrix.from_numpy(np.ones((500, 100))).qr()
    t.solve_least_squares(ng.DeviceMatrix.from_numpy(np.ones((500, 1))))
    args = fake.named("nacu_dqr_solve")[-1]
    assert args[:3] == (500, 100, 1) and args[7] == 500 and args[10] == fake.real.nacu_qr_solve_workspace_bytes(100)
    with pytest.raises(AssertionError):
        t.solve_mut(b)  # QR::solve_mut asserts a square factor


def test_batched_solves_go_sixteen_columns_per_call(fake):
    import nalgebra_gb300 as ng

    n = 10
    cq = ng.DeviceMatrix.from_numpy(np.eye(n)).col_piv_qr()
    b = ng.DeviceMatrix.from_numpy(np.ones((n, 40)))
    cq.solve_mut(b)
    calls = fake.named("nacu_dcolpivqr_solve_batched")
    assert [c[1] for c in calls] == [16, 16, 8]
    base = b.data.data_ptr()
    assert [c[6] - base for c in calls] == [0, 16 * n * 8, 32 * n * 8]
    assert [c[7] for c in calls] == [n * 16, n * 16, n * 8]


def test_lu_and_triangular_solves_route_by_order(fake):
    import nalgebra_gb300 as ng

    lu = ng.DeviceMatrix.from_numpy(np.eye(200)).lu()
    (args,) = fake.named("nacu_dgetrf")
    assert args[0] == 200 and args[2] == 200 and args[6] == fake.real.nacu_getrf_workspace_bytes(200) and lu.large
    b = ng.DeviceMatrix.from_numpy(np.ones((200, 3)))
    lu.solve_mut(b)
    calls = fake.named("nacu_dgetrs")
    assert len(calls) == 3 and [c[4] - b.data.data_ptr() for c in calls] == [0, 200 * 8, 400 * 8]
    small = ng.DeviceMatrix.from_numpy(np.eye(128))
    small.solve_lower_triangular_mut(ng.DeviceMatrix.from_numpy(np.ones((128, 1))))
    assert fake.named("nacu_dtrsv_batched")[-1][0] == 128
    big = ng.DeviceMatrix.from_numpy(np.eye(129))
    big.tr_solve_upper_triangular_mut(ng.DeviceMatrix.from_numpy(np.ones((129, 2))))
    args = fake.named("nacu_dtrsv")[-1]
    assert args[:4] == (129, 2, 1, 1) and args[12] == fake.real.nacu_trsv_workspace_bytes(129)


def test_calls_follow_the_current_stream(fake):
    import nalgebra_gb300 as ng

    m = ng.DeviceMatrix.from_numpy(np.eye(8))
    with ng.stream(0x1234):
        m.lu()
    assert fake.named("nacu_dgetrf_batched")[-1][-1] == 0x1234
    m.clone_owned().lu()
    assert fake.named("nacu_dgetrf_batched")[-1][-1] == 0


def test_graph_capture_records_on_its_own_stream(fake):
    import nalgebra_gb300 as ng

    a = ng.DeviceMatrix.from_numpy(np.eye(4))
    c = ng.DeviceMatrix.from_numpy(np.zeros((4, 4)))
    g = ng.Graph()
    with g.capture():
        ng.gemm(c, 1.0, a, a, 0.0)
    (begin,) = fake.named("nacu_graph_begin_capture")
    cap = begin[0]
    assert cap != 0 and fake.named("nacu_dgemm")[-1][-1] == cap
    assert fake.named("nacu_graph_end_capture")[-1] == (cap,)
    g.replay()
    assert fake.named("nacu_graph_launch")[-1] == (0x7000, 0)


def test_host_pipeline_passes_host_arrays(fake):
    import nalgebra_gb300 as ng

    ns = np.array([3, 2], np.int32)
    aoff = np.array([0, 9], np.int64)
    boff = np.array([0, 3], np.int64)
    a = np.arange(13, dtype=np.float64)
    b = np.ones(5)
    x, info, iters = ng.cholesky_solve_refined_host(ns, aoff, a, boff, b, 1, chunks=2)
    (args,) = fake.named("nacu_dposv_ragged_mixed_host")
    assert args[:2] == (2, 3) and args[5] == 1 and args[11] == 2
    assert x.shape == (5,) and info.shape == (2,) and iters.shape == (2,)
