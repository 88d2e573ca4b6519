"""Device memory, streams and CUDA graphs for the mirror, through the
library's own plumbing entry points (nacu_malloc, nacu_memcpy, nacu_memset,
nacu_stream_*, nacu_graph_*).  The product path needs nothing but
libnalgebra_cuda.so: no PyTorch, no CUDA Python binding.

Buffers of other libraries plug in through the CUDA Array Interface
(``__cuda_array_interface__``: PyTorch, CuPy, Numba device arrays): they are
wrapped without a copy, and a ``DeviceBuffer`` exports the same interface, so
``torch.as_tensor(buf, device="cuda")`` views it in turn.

Every call of the mirror is queued on the thread's current stream: the legacy
default stream (0) unless ``stream(handle)`` or ``set_stream`` says
otherwise.
"""
from __future__ import annotations

import contextlib
import ctypes as C
import math
import threading

import numpy as np

from . import _lib
from ._lib import NacuError

_tls = threading.local()
_gpu_checked = False


def require_gpu() -> None:
    """Raise NacuError unless the library loads and sees a CUDA device: the
    mirror has no CPU fallback."""
    global _gpu_checked
    if _gpu_checked:
        return
    n = C.c_int(0)
    rc = _lib.load().nacu_device_count(C.byref(n))
    if rc != 0 or n.value == 0:
        raise NacuError("nalgebra_gb300 needs a CUDA GPU: there is no CPU fallback")
    _gpu_checked = True


# -- streams ---------------------------------------------------------------------------------------------

def _handle(s) -> int:
    if s is None:
        return 0
    if isinstance(s, int):
        return s
    if isinstance(s, Stream):
        return s.handle
    h = getattr(s, "cuda_stream", None)  # a stream object of another library
    if h is not None:
        return int(h)
    raise TypeError(f"not a CUDA stream: {s!r}")


def current_stream() -> int:
    """The cudaStream_t (as an int) the mirror queues its calls on."""
    return getattr(_tls, "stream", 0)


def set_stream(s) -> None:
    _tls.stream = _handle(s)


@contextlib.contextmanager
def stream(s):
    """Queue the mirror's calls on ``s`` inside the block: a ``Stream``, a raw
    cudaStream_t, or any object with a ``cuda_stream`` attribute."""
    prev = current_stream()
    set_stream(s)
    try:
        yield
    finally:
        _tls.stream = prev


def synchronize(s=None) -> None:
    """Wait for the work queued on ``s`` (default: the current stream)."""
    _lib.call("nacu_stream_synchronize", _handle(s) if s is not None else current_stream())


class Stream:
    """A non-blocking CUDA stream of the library's own (nacu_stream_create)."""

    def __init__(self):
        require_gpu()
        p = C.c_void_p()
        _lib.call("nacu_stream_create", C.byref(p))
        self.handle = int(p.value or 0)

    @property
    def cuda_stream(self) -> int:
        return self.handle

    def synchronize(self) -> None:
        _lib.call("nacu_stream_synchronize", self.handle)

    def wait(self, other) -> None:
        """Work queued on this stream from now on starts after the work queued
        on ``other`` so far."""
        _lib.call("nacu_stream_wait", self.handle, _handle(other))

    def __del__(self):
        try:
            if self.handle:
                _lib.load().nacu_stream_destroy(self.handle)
                self.handle = 0
        except Exception:  # interpreter shutdown
            pass


class Graph:
    """A CUDA graph of mirror calls.  ``with g.capture(): ...`` records the
    calls made in the block on a stream of its own instead of running them;
    ``g.replay()`` runs them on the current stream.  The library's compute
    calls neither allocate nor synchronize, so they capture; allocate every
    buffer (and run first-use set-up, e.g. a warm-up call) before capturing."""

    def __init__(self):
        self._exec = 0
        self._stream = None

    @contextlib.contextmanager
    def capture(self):
        if self._exec:
            raise RuntimeError("this graph was already captured")
        self._stream = Stream()
        _lib.call("nacu_device_synchronize")  # the captured work follows everything queued so far
        _lib.call("nacu_graph_begin_capture", self._stream.handle)
        ok = False
        try:
            with stream(self._stream):
                yield self
            ok = True
        finally:
            x = C.c_void_p()
            rc = _lib.load().nacu_graph_end_capture(self._stream.handle, C.byref(x))
            if ok:
                _lib.check(rc, "nacu_graph_end_capture")
                self._exec = int(x.value or 0)

    def replay(self, s=None) -> None:
        if not self._exec:
            raise RuntimeError("replay before capture")
        _lib.call("nacu_graph_launch", self._exec, _handle(s) if s is not None else current_stream())

    def __del__(self):
        try:
            if self._exec:
                _lib.load().nacu_graph_destroy(self._exec)
                self._exec = 0
        except Exception:
            pass


# -- device buffers --------------------------------------------------------------------------------------

def _shape(shape) -> tuple:
    if isinstance(shape, (int, np.integer)):
        return (int(shape),)
    return tuple(int(d) for d in shape)


class DeviceBuffer:
    """Contiguous device memory typed like a numpy array.  Owned buffers come
    from nacu_malloc and are freed with the object (nacu_free synchronizes the
    device: drop buffers outside a graph capture).  ``wrap`` views another
    library's device array without a copy and keeps it alive."""

    __slots__ = ("_ptr", "shape", "dtype", "_owned", "_base")

    def __init__(self, ptr: int, shape, dtype, owned: bool = False, base=None):
        self._ptr = int(ptr or 0)
        self.shape = _shape(shape)
        self.dtype = np.dtype(dtype)
        self._owned = owned
        self._base = base

    # construction
    @classmethod
    def empty(cls, shape, dtype=np.float64) -> "DeviceBuffer":
        require_gpu()
        shape, dtype = _shape(shape), np.dtype(dtype)
        nbytes = math.prod(shape) * dtype.itemsize
        p = C.c_void_p()
        _lib.call("nacu_malloc", C.byref(p), nbytes)
        return cls(p.value or 0, shape, dtype, owned=True)

    @classmethod
    def zeros(cls, shape, dtype=np.float64) -> "DeviceBuffer":
        return cls.empty(shape, dtype).zero_()

    @classmethod
    def full(cls, shape, value, dtype=np.float64) -> "DeviceBuffer":
        return cls.from_numpy(np.full(_shape(shape), value, dtype=dtype))

    @classmethod
    def from_numpy(cls, a, dtype=None) -> "DeviceBuffer":
        """A device copy of a host array (C order; queued on the current
        stream, the host array may be reused as soon as this returns)."""
        arr = np.ascontiguousarray(a, dtype=dtype)
        buf = cls.empty(arr.shape, arr.dtype)
        if arr.nbytes:
            _lib.call("nacu_memcpy", buf._ptr, arr.ctypes.data, arr.nbytes, current_stream())
        return buf

    @classmethod
    def wrap(cls, obj) -> "DeviceBuffer":
        """A view of ``obj``: a DeviceBuffer (returned as it is) or any
        C-contiguous device array exporting ``__cuda_array_interface__``."""
        if isinstance(obj, DeviceBuffer):
            return obj
        cai = getattr(obj, "__cuda_array_interface__", None)
        if cai is None:
            raise TypeError(f"not a device array (no __cuda_array_interface__): {type(obj).__name__}")
        shape = tuple(cai["shape"])
        dtype = np.dtype(cai["typestr"])
        strides = cai.get("strides")
        if strides is not None:
            expect, acc = [], dtype.itemsize
            for d in reversed(shape):
                expect.append(acc)
                acc *= d
            if tuple(strides) != tuple(reversed(expect)) and math.prod(shape) > 1:
                raise ValueError("device arrays must be C-contiguous")
        return cls(cai["data"][0], shape, dtype, owned=False, base=obj)

    # the interface other libraries read
    @property
    def __cuda_array_interface__(self):
        return {"shape": self.shape, "typestr": self.dtype.str, "data": (self._ptr, False), "strides": None,
                "version": 2}

    # introspection (the names PyTorch uses, so either kind of buffer reads the same)
    def data_ptr(self) -> int:
        return self._ptr

    def numel(self) -> int:
        return math.prod(self.shape)

    def element_size(self) -> int:
        return self.dtype.itemsize

    @property
    def nbytes(self) -> int:
        return self.numel() * self.dtype.itemsize

    def __len__(self) -> int:
        return self.shape[0] if self.shape else 1

    def reshape(self, *shape) -> "DeviceBuffer":
        shape = _shape(shape[0] if len(shape) == 1 else shape)
        if math.prod(shape) != self.numel():
            raise ValueError("reshape changes the element count")
        return DeviceBuffer(self._ptr, shape, self.dtype, owned=False, base=self)

    # data movement, on the current stream
    def to_numpy(self) -> np.ndarray:
        """A host copy (waits for the work queued on the current stream)."""
        out = np.empty(self.shape, dtype=self.dtype)
        if out.nbytes:
            s = current_stream()
            _lib.call("nacu_memcpy", out.ctypes.data, self._ptr, out.nbytes, s)
            _lib.call("nacu_stream_synchronize", s)
        return out

    def item(self):
        return self.to_numpy().reshape(-1)[0].item()

    def clone(self) -> "DeviceBuffer":
        out = DeviceBuffer.empty(self.shape, self.dtype)
        if self.nbytes:
            _lib.call("nacu_memcpy", out._ptr, self._ptr, self.nbytes, current_stream())
        return out

    def copy_(self, src) -> "DeviceBuffer":
        """Overwrite with ``src`` (a device array or a host array of the same
        byte size)."""
        if isinstance(src, np.ndarray):
            a = np.ascontiguousarray(src, dtype=self.dtype)
            nbytes, ptr, keep = a.nbytes, a.ctypes.data, a
        else:
            w = DeviceBuffer.wrap(src)
            nbytes, ptr, keep = w.nbytes, w._ptr, w
        if nbytes != self.nbytes:
            raise ValueError(f"copy_: {nbytes} bytes into a buffer of {self.nbytes}")
        if nbytes:
            _lib.call("nacu_memcpy", self._ptr, ptr, nbytes, current_stream())
        del keep
        return self

    def zero_(self) -> "DeviceBuffer":
        if self.nbytes:
            _lib.call("nacu_memset", self._ptr, 0, self.nbytes, current_stream())
        return self

    def fill_(self, value) -> "DeviceBuffer":
        return self.copy_(np.full(self.shape, value, dtype=self.dtype))

    def __repr__(self) -> str:
        return f"DeviceBuffer(shape={self.shape}, dtype={self.dtype}, ptr={self._ptr:#x})"

    def __del__(self):
        try:
            if self._owned and self._ptr:
                _lib.load().nacu_free(self._ptr)
                self._ptr = 0
        except Exception:
            pass


def empty(shape, dtype=np.float64) -> DeviceBuffer:
    return DeviceBuffer.empty(shape, dtype)


def zeros(shape, dtype=np.float64) -> DeviceBuffer:
    return DeviceBuffer.zeros(shape, dtype)


def from_numpy(a, dtype=None) -> DeviceBuffer:
    return DeviceBuffer.from_numpy(a, dtype)


def as_device(x, dtype=None) -> DeviceBuffer:
    """A device array as it is (wrapped, no copy) or a host array copied to
    the device; ``dtype`` is checked for device arrays and converted to for
    host ones."""
    if isinstance(x, DeviceBuffer) or hasattr(x, "__cuda_array_interface__"):
        buf = DeviceBuffer.wrap(x)
        if dtype is not None and buf.dtype != np.dtype(dtype):
            raise TypeError(f"device array of {buf.dtype}, expected {np.dtype(dtype)}")
        return buf
    return DeviceBuffer.from_numpy(x, dtype)


# -- page-locked host memory -------------------------------------------------------------------------------

def pinned_empty(shape, dtype=np.float64) -> np.ndarray:
    """A numpy array in page-locked host memory (nacu_host_alloc), released
    with the array.  Copies to and from it overlap with kernels."""
    require_gpu()
    shape, dtype = _shape(shape), np.dtype(dtype)
    nbytes = math.prod(shape) * dtype.itemsize
    if nbytes == 0:
        return np.empty(shape, dtype)
    p = C.c_void_p()
    _lib.call("nacu_host_alloc", C.byref(p), nbytes)

    def _release(self):
        try:
            _lib.load().nacu_host_free(C.addressof(self))
        except Exception:
            pass

    block_t = type("PinnedBlock", (C.c_char * nbytes,), {"__del__": _release})
    block = block_t.from_address(p.value)
    return np.frombuffer(block, dtype=dtype).reshape(shape)
