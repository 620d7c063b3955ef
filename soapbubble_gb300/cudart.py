"""Minimal ctypes access to the CUDA runtime that libsoapbubble_gb300 links
(libcudart.so.13): device buffers, pinned host buffers, stream-ordered
memset (L2 flushing between timed steps) and events."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

_rt = None


def rt() -> C.CDLL:
    global _rt
    if _rt is None:
        _lib.lib()  # loads libcudart.so.13 as a dependency
        _rt = C.CDLL("libcudart.so.13")
        vp, sz = C.c_void_p, C.c_size_t
        _rt.cudaMalloc.argtypes = [C.POINTER(vp), sz]
        _rt.cudaFree.argtypes = [vp]
        _rt.cudaHostAlloc.argtypes = [C.POINTER(vp), sz, C.c_uint]
        _rt.cudaFreeHost.argtypes = [vp]
        _rt.cudaMemsetAsync.argtypes = [vp, C.c_int, sz, vp]
        _rt.cudaStreamSynchronize.argtypes = [vp]
        _rt.cudaSetDevice.argtypes = [C.c_int]
        _rt.cudaDeviceSynchronize.argtypes = []
        _rt.cudaGetErrorString.restype = C.c_char_p
        _rt.cudaEventCreate.argtypes = [C.POINTER(vp)]
        _rt.cudaEventRecord.argtypes = [vp, vp]
        _rt.cudaEventSynchronize.argtypes = [vp]
        _rt.cudaEventElapsedTime.argtypes = [C.POINTER(C.c_float), vp, vp]
        _rt.cudaEventDestroy.argtypes = [vp]
        _rt.cudaMemcpy.argtypes = [vp, vp, sz, C.c_int]
        _rt.cudaMemGetInfo.argtypes = [C.POINTER(sz), C.POINTER(sz)]
    return _rt


def _ok(code: int, what: str) -> None:
    if code != 0:
        raise RuntimeError(f"{what}: {rt().cudaGetErrorString(code).decode()}")


def set_device(dev: int) -> None:
    _ok(rt().cudaSetDevice(dev), "cudaSetDevice")


def mem_get_info():
    """(free, total) bytes of the current device."""
    free, total = C.c_size_t(), C.c_size_t()
    _ok(rt().cudaMemGetInfo(C.byref(free), C.byref(total)), "cudaMemGetInfo")
    return free.value, total.value


class DeviceBuffer:
    def __init__(self, nbytes: int):
        self.ptr = C.c_void_p()
        self.nbytes = nbytes
        _ok(rt().cudaMalloc(C.byref(self.ptr), nbytes), "cudaMalloc")

    def memset_async(self, value: int, stream) -> None:
        _ok(rt().cudaMemsetAsync(self.ptr, value, self.nbytes, C.c_void_p(stream)), "cudaMemsetAsync")

    def free(self) -> None:
        if self.ptr:
            rt().cudaFree(self.ptr)
            self.ptr = C.c_void_p()


class PinnedArray:
    """A numpy array over page-locked host memory."""

    def __init__(self, shape, dtype=np.float32):
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.ptr = C.c_void_p()
        _ok(rt().cudaHostAlloc(C.byref(self.ptr), n, 0), "cudaHostAlloc")
        buf = (C.c_char * n).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self) -> None:
        if self.ptr:
            self.array = None
            rt().cudaFreeHost(self.ptr)
            self.ptr = C.c_void_p()


def stream_sync(stream) -> None:
    _ok(rt().cudaStreamSynchronize(C.c_void_p(stream)), "cudaStreamSynchronize")


class Event:
    def __init__(self):
        self.ev = C.c_void_p()
        _ok(rt().cudaEventCreate(C.byref(self.ev)), "cudaEventCreate")

    def record(self, stream) -> None:
        _ok(rt().cudaEventRecord(self.ev, C.c_void_p(stream)), "cudaEventRecord")

    def synchronize(self) -> None:
        _ok(rt().cudaEventSynchronize(self.ev), "cudaEventSynchronize")

    def elapsed_ms(self, end: "Event") -> float:
        ms = C.c_float(0)
        _ok(rt().cudaEventElapsedTime(C.byref(ms), self.ev, end.ev), "cudaEventElapsedTime")
        return ms.value


def memcpy_htod(dst: DeviceBuffer, src: np.ndarray) -> None:
    src = np.ascontiguousarray(src)
    assert src.nbytes <= dst.nbytes
    _ok(rt().cudaMemcpy(dst.ptr, src.ctypes.data_as(C.c_void_p), src.nbytes, 1), "cudaMemcpy")


def memcpy_dtoh(dst: np.ndarray, src: DeviceBuffer) -> None:
    assert dst.flags.c_contiguous and dst.nbytes <= src.nbytes
    _ok(rt().cudaMemcpy(dst.ctypes.data_as(C.c_void_p), src.ptr, dst.nbytes, 2), "cudaMemcpy")
