"""The product's host mirror without PyTorch: importing it and loading the
library pulls in neither torch nor a CUDA Python binding, its device memory,
copies, streams and graphs go through the library's own plumbing entry points
(nacu_malloc, nacu_memcpy, nacu_graph_*), and without a GPU every device call
raises instead of falling back to the CPU."""
import subprocess
import sys

import pytest

from nalgebra_gb300 import _lib, build


@pytest.fixture(scope="module")
def L():
    build.build()
    return _lib.load()


def test_mirror_imports_and_loads_without_torch(L):
    code = ("import sys, nalgebra_gb300 as ng\n"
            "ng._lib.load()\n"
            "bad = [m for m in ('torch', 'cupy', 'numba', 'cuda', 'pycuda') if m in sys.modules]\n"
            "assert not bad, bad\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr


def _no_gpu(L) -> bool:
    import ctypes as C

    n = C.c_int(-1)
    return L.nacu_device_count(C.byref(n)) != 0 or n.value == 0


def test_device_calls_raise_without_a_gpu(L):
    if not _no_gpu(L):
        pytest.skip("a GPU is present")
    import numpy as np

    import nalgebra_gb300 as ng

    with pytest.raises(ng.NacuError):
        ng.DeviceMatrix.from_numpy(np.eye(3))
    with pytest.raises(ng.NacuError):
        ng.DeviceBuffer.zeros(4)


def test_plumbing_argument_errors(L):
    import ctypes as C

    assert L.nacu_malloc(None, 8) == -1
    p = C.c_void_p(1)
    assert L.nacu_malloc(C.byref(p), 0) == 0 and not p.value  # zero bytes: NULL, no device needed
    assert L.nacu_free(None) == 0 and L.nacu_host_free(None) == 0
    assert L.nacu_memcpy(None, None, 0, None) == 0
    assert L.nacu_memcpy(None, 1, 8, None) == -1 and L.nacu_memcpy(1, None, 8, None) == -2
    assert L.nacu_memset(None, 0, 8, None) == -1
    assert L.nacu_graph_begin_capture(None) == -1
    assert L.nacu_graph_launch(None, None) == -1
    assert L.nacu_graph_destroy(None) == 0 and L.nacu_stream_destroy(None) == 0


@pytest.mark.gpu
def test_buffers_streams_and_graphs_on_the_gpu(L):
    import numpy as np

    import nalgebra_gb300 as ng

    a = np.arange(12, dtype=np.float64).reshape(3, 4)
    buf = ng.DeviceBuffer.from_numpy(a)
    assert buf.shape == (3, 4) and np.array_equal(buf.to_numpy(), a)
    c = buf.clone()
    buf.zero_()
    assert np.array_equal(c.to_numpy(), a) and not buf.to_numpy().any()
    buf.copy_(c)
    assert np.array_equal(buf.to_numpy(), a)
    buf.fill_(2.5)
    assert np.all(buf.to_numpy() == 2.5) and buf.item() == 2.5
    v = buf.reshape(12)
    assert v.data_ptr() == buf.data_ptr() and v.numel() == 12
    # a side stream, ordered after the default one
    s = ng.Stream()
    s.wait(0)
    with ng.stream(s):
        d = ng.DeviceBuffer.from_numpy(a * 2)
        out = d.to_numpy()
    assert np.array_equal(out, a * 2)
    # page-locked host memory round trip
    h = ng.pinned_empty((3, 4))
    h[:] = a
    e = ng.DeviceBuffer.from_numpy(h)
    assert np.array_equal(e.to_numpy(), a)
    # a captured graph of mirror calls: a gemm, replayed after the inputs change
    ma, mb = np.eye(4) * 3.0, np.arange(16, dtype=np.float64).reshape(4, 4)
    A, B = ng.DeviceMatrix.from_numpy(ma), ng.DeviceMatrix.from_numpy(mb)
    C = ng.DeviceMatrix.from_numpy(np.zeros((4, 4)))
    ng.gemm(C, 1.0, A, B, 0.0)
    g = ng.Graph()
    with g.capture():
        ng.gemm(C, 1.0, A, B, 0.0)
    A.data.copy_(np.asfortranarray(np.eye(4) * 5.0).ravel(order="F"))
    g.replay()
    ng.synchronize()
    assert np.allclose(C.to_numpy(), 5.0 * mb, rtol=0, atol=1e-12)


@pytest.mark.gpu
def test_other_libraries_arrays_plug_in_without_a_copy(L, cuda):
    """A device array of another library (here a torch CUDA tensor) is used
    in place through __cuda_array_interface__, and a DeviceBuffer is viewed
    by that library the same way."""
    import numpy as np

    import nalgebra_gb300 as ng

    torch = cuda
    t = torch.arange(9, dtype=torch.float64, device="cuda")
    m = ng.DeviceMatrix(t, 3, 3)
    assert m.data.data_ptr() == t.data_ptr()
    m.data.zero_()
    ng.synchronize()
    assert float(t.abs().sum()) == 0.0
    buf = ng.DeviceBuffer.from_numpy(np.arange(5, dtype=np.float64))
    view = torch.as_tensor(buf, device="cuda")
    assert view.data_ptr() == buf.data_ptr() and view.cpu().tolist() == [0.0, 1.0, 2.0, 3.0, 4.0]
    with pytest.raises(TypeError):
        ng.DeviceMatrix(torch.zeros(9, dtype=torch.float32, device="cuda"), 3, 3)


class _FakeDeviceArray:
    """Exports the CUDA Array Interface only (no memory behind it: wrap reads
    the dict and touches no device)."""

    def __init__(self, shape, typestr, strides=None, ptr=0x7000):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False),
                                         "strides": strides, "version": 2}


def test_wrap_reads_the_cuda_array_interface():
    import numpy as np

    from nalgebra_gb300 import DeviceBuffer

    src = _FakeDeviceArray((3, 4), "<f8")
    w = DeviceBuffer.wrap(src)
    assert (w.data_ptr(), w.shape, w.dtype, w.numel(), w.nbytes) == (0x7000, (3, 4), np.float64, 12, 96)
    assert w.__cuda_array_interface__["data"] == (0x7000, False)
    assert DeviceBuffer.wrap(w) is w
    # explicit C-contiguous strides are accepted, others rejected
    assert DeviceBuffer.wrap(_FakeDeviceArray((3, 4), "<i4", strides=(16, 4))).dtype == np.int32
    with pytest.raises(ValueError):
        DeviceBuffer.wrap(_FakeDeviceArray((3, 4), "<f8", strides=(8, 24)))
    with pytest.raises(TypeError):
        DeviceBuffer.wrap(np.zeros(3))  # host memory is not a device array
    v = w.reshape(12)
    assert v.data_ptr() == w.data_ptr() and v.shape == (12,)
    with pytest.raises(ValueError):
        w.reshape(5)


def test_as_device_checks_the_dtype_of_device_arrays():
    import numpy as np

    from nalgebra_gb300 import _device

    with pytest.raises(TypeError):
        _device.as_device(_FakeDeviceArray((4,), "<f4"), np.float64)
    assert _device.as_device(_FakeDeviceArray((4,), "<f8"), np.float64).data_ptr() == 0x7000


def test_stream_context_is_per_thread():
    import threading

    from nalgebra_gb300 import _device

    assert _device.current_stream() == 0
    seen = []
    with _device.stream(0x1234):
        assert _device.current_stream() == 0x1234
        t = threading.Thread(target=lambda: seen.append(_device.current_stream()))
        t.start()
        t.join()
    assert _device.current_stream() == 0 and seen == [0]

    class _Other:
        cuda_stream = 0x99

    with _device.stream(_Other()):
        assert _device.current_stream() == 0x99
    with pytest.raises(TypeError):
        _device.set_stream("default")
