"""Python mirror of the reference SZx C interface, backed by libszx_gb300.so.

``fast_compress_args`` / ``fast_decompress`` take and return host arrays
exactly like ``SZx_fast_compress_args`` / ``SZx_fast_decompress``
(szx/include/szx.h:75-78): same fastMode, dataType, error-bound modes and
stream bytes.  ``DeviceCodec`` drives the device-pointer interface
(``SZxG_compress`` / ``SZxG_decompress``) on torch CUDA tensors, with the
workspace and output buffers owned by the caller.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import StreamInfo, lib, libc

SZx_FLOAT, SZx_DOUBLE = 0, 1
ABS, REL, FXR = 0, 1, 2
NO_BLOCK, WITH_BLOCK, RANDOM_ACCESS, OPENMP = 1, 2, 3, 4


class SZxError(RuntimeError):
    def __init__(self, code: int, what: str):
        self.code = code
        msg = lib().SZxG_error_string(code).decode()
        super().__init__(f"{what}: {msg} (code {code})")


def last_error() -> int:
    return lib().SZxG_get_last_error()


def _dtype_code(dtype) -> int:
    dt = np.dtype(dtype)
    if dt == np.float32:
        return SZx_FLOAT
    if dt == np.float64:
        return SZx_DOUBLE
    raise TypeError(f"SZx handles float32 and float64, not {dt}")


def _np_dtype(code: int):
    return np.float32 if code == SZx_FLOAT else np.float64


def _dims(n: int, dims=None):
    """r5..r1 of the reference call (r1 fastest); default 1-D."""
    if dims is None:
        return (0, 0, 0, 0, n)
    d = [0] * (5 - len(dims)) + list(dims)
    return tuple(d)


def _take(ptr: int, nbytes: int) -> bytes:
    b = C.string_at(ptr, nbytes)
    libc().free(ptr)
    return b


# ------------------------------------------------------------------ reference interface

def compute_data_length(r5=0, r4=0, r3=0, r2=0, r1=0) -> int:
    return lib().SZx_computeDataLength(r5, r4, r3, r2, r1)


def compute_dimension(r5=0, r4=0, r3=0, r2=0, r1=0) -> int:
    return lib().SZx_computeDimension(r5, r4, r3, r2, r1)


def filter_dimension(r5=0, r4=0, r3=0, r2=0, r1=0):
    c = (C.c_size_t * 5)()
    rc = lib().SZx_filterDimension(r5, r4, r3, r2, r1, c)
    return rc, list(c)


def compute_value_range(data: np.ndarray):
    """SZx_computeValueRange: (range, radius, median)."""
    x = np.ascontiguousarray(data)
    r, m = C.c_float(), C.c_float()
    v = lib().SZx_computeValueRange(x.ctypes.data, _dtype_code(x.dtype), x.size, C.byref(r), C.byref(m))
    if last_error():
        raise SZxError(last_error(), "SZx_computeValueRange")
    return v, r.value, m.value


def fast_compress_args(fastMode: int, data: np.ndarray, errBoundMode: int, absErrBound: float = 0.0,
                       relBoundRatio: float = 0.0, compressionRatio: float = 0.0, tolerance: float = 0.0,
                       dims=None) -> bytes:
    """SZx_fast_compress_args on a host array; returns the stream bytes."""
    x = np.ascontiguousarray(data)
    out = C.c_size_t()
    r5, r4, r3, r2, r1 = _dims(x.size, dims)
    p = lib().SZx_fast_compress_args(fastMode, _dtype_code(x.dtype), x.ctypes.data, C.byref(out), errBoundMode,
                                     absErrBound, relBoundRatio, compressionRatio, tolerance, r5, r4, r3, r2, r1)
    if not p:
        raise SZxError(last_error(), "SZx_fast_compress_args")
    return _take(p, out.value)


def fast_decompress(fastMode: int, dtype, stream: bytes, n: int | None = None, dims=None) -> np.ndarray:
    """SZx_fast_decompress of a host stream; returns a host array."""
    code = _dtype_code(dtype)
    r5, r4, r3, r2, r1 = _dims(n, dims)
    n = compute_data_length(r5, r4, r3, r2, r1)
    s = np.frombuffer(stream, np.uint8)
    p = lib().SZx_fast_decompress(fastMode, code, s.ctypes.data, s.size, r5, r4, r3, r2, r1)
    if not p:
        raise SZxError(last_error(), "SZx_fast_decompress")
    nd = np.dtype(_np_dtype(code))
    return np.frombuffer(_take(p, n * nd.itemsize), nd).copy()


def estimate_error_bound(data: np.ndarray, compressionRatio: float, tolerance: float, initErrorBound: float,
                         blockSize: int = 128) -> float:
    """SZx_estimateErrorBoundbasedonCR: the bound the sampled-ratio search settles on."""
    x = np.ascontiguousarray(data)
    eb = lib().SZx_estimateErrorBoundbasedonCR(_dtype_code(x.dtype), compressionRatio, tolerance, x.ctypes.data,
                                               initErrorBound, blockSize, x.size)
    if last_error():
        raise SZxError(last_error(), "SZx_estimateErrorBoundbasedonCR")
    return eb


def compute_radius_buffer(data: np.ndarray, samplingRate: int = 10, blockSize: int = 128):
    """computeRadiusBuffer: (sampled range, radius[], median[], copies of the sampled blocks)."""
    x = np.ascontiguousarray(data)
    rp, mp, bp = C.POINTER(C.c_float)(), C.POINTER(C.c_float)(), C.c_void_p()
    rng = lib().computeRadiusBuffer(x.ctypes.data, _dtype_code(x.dtype), x.size, samplingRate, blockSize,
                                    C.byref(rp), C.byref(mp), C.byref(bp))
    if last_error():
        raise SZxError(last_error(), "computeRadiusBuffer")
    ns = x.size // (samplingRate * blockSize)
    free = libc().free
    try:
        rads = np.ctypeslib.as_array(rp, shape=(ns,)).copy() if ns else np.zeros(0, np.float32)
        meds = np.ctypeslib.as_array(mp, shape=(ns,)).copy() if ns else np.zeros(0, np.float32)
        buf = (np.frombuffer(C.string_at(bp.value, ns * blockSize * x.itemsize), x.dtype).copy()
               if ns else np.zeros(0, x.dtype))
    finally:
        free(C.cast(rp, C.c_void_p)); free(C.cast(mp, C.c_void_p)); free(bp)
    return rng, rads, meds, buf


def estimate_cr_buffered(buffer: np.ndarray, medians: np.ndarray, radii: np.ndarray, errorBound: float, nbEle: int,
                         samplingRate: int = 10, blockSize: int = 128):
    """estimateCRbasedonErrorBound_buffered: (ratio estimate, sum of required bytes, sum of leads)."""
    b = np.ascontiguousarray(buffer)
    m = np.ascontiguousarray(medians, np.float32)
    r = np.ascontiguousarray(radii, np.float32)
    a, c = C.c_size_t(), C.c_size_t()
    fp = C.POINTER(C.c_float)
    cr = lib().estimateCRbasedonErrorBound_buffered(_dtype_code(b.dtype), errorBound, b.ctypes.data,
                                                    m.ctypes.data_as(fp), r.ctypes.data_as(fp), samplingRate,
                                                    blockSize, nbEle, C.byref(a), C.byref(c))
    if last_error():
        raise SZxError(last_error(), "estimateCRbasedonErrorBound_buffered")
    return cr, a.value, c.value


def compress_blocked(data: np.ndarray, absErrBound: float, blockSize: int, native_medians: bool = False) -> bytes:
    """SZx_fast_compress_args_unpredictable_blocked(_randomaccess_openmp)."""
    x = np.ascontiguousarray(data)
    out = C.c_size_t()
    fn = (lib().SZx_fast_compress_args_unpredictable_blocked_randomaccess_openmp if native_medians
          else lib().SZx_fast_compress_args_unpredictable_blocked)
    p = fn(x.ctypes.data, _dtype_code(x.dtype), C.byref(out), absErrBound, x.size, blockSize)
    if not p:
        raise SZxError(last_error(), fn.__name__)
    return _take(p, out.value)


def compress_host(fastMode: int, data: np.ndarray, blockSize: int = 128, errBoundMode: int = ABS,
                  absErrBound: float = 0.0, relBoundRatio: float = 0.0) -> bytes:
    """SZxG_compress_host: the reference stream with an explicit block size."""
    x = np.ascontiguousarray(data)
    out = C.c_size_t()
    p = lib().SZxG_compress_host(fastMode, _dtype_code(x.dtype), x.ctypes.data, x.size, blockSize, errBoundMode,
                                 absErrBound, relBoundRatio, C.byref(out))
    if not p:
        raise SZxError(last_error(), "SZxG_compress_host")
    return _take(p, out.value)


def decompress_host(fastMode: int, dtype, stream: bytes, n: int) -> np.ndarray:
    code = _dtype_code(dtype)
    s = np.frombuffer(stream, np.uint8)
    p = lib().SZxG_decompress_host(fastMode, code, s.ctypes.data, s.size, n)
    if not p:
        raise SZxError(last_error(), "SZxG_decompress_host")
    nd = np.dtype(_np_dtype(code))
    return np.frombuffer(_take(p, n * nd.itemsize), nd).copy()


# ------------------------------------------------------------------ device interface

class DeviceCodec:
    """Device-pointer codec on torch CUDA tensors (SZxG_compress / SZxG_decompress).

    Buffers are sized for `max_elems` values of `dtype` and reused; calls are
    enqueued on the current torch stream and do not synchronise.
    """

    def __init__(self, fastMode: int, dtype, max_elems: int, blockSize: int = 128, device=None):
        import torch
        self.torch = torch
        self.mode, self.bs = fastMode, blockSize
        self.code = _dtype_code(dtype)
        self.max_elems = max_elems
        dev = torch.device(device or "cuda")
        L = lib()
        self.cap = L.SZxG_compress_bound(fastMode, self.code, max_elems, blockSize)
        self.wsb = L.SZxG_workspace_size(fastMode, self.code, max_elems, blockSize)
        self.out = torch.empty(self.cap, dtype=torch.uint8, device=dev)
        self.ws = torch.zeros(self.wsb, dtype=torch.uint8, device=dev)
        self.info = torch.zeros(C.sizeof(StreamInfo), dtype=torch.uint8, device=dev)

    def _stream(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def compress(self, x, errBoundMode: int = ABS, absErrBound: float = 0.0, relBoundRatio: float = 0.0):
        """Enqueue; the stream is at out[info.offset : info.offset + info.size]."""
        assert x.is_cuda and x.is_contiguous() and x.numel() <= self.max_elems
        rc = lib().SZxG_compress(self.mode, self.code, C.c_void_p(x.data_ptr()), x.numel(), self.bs, errBoundMode,
                                 absErrBound, relBoundRatio, C.c_void_p(self.out.data_ptr()), self.cap,
                                 C.c_void_p(self.ws.data_ptr()), self.wsb, C.c_void_p(self.info.data_ptr()),
                                 self._stream())
        if rc:
            raise SZxError(rc, "SZxG_compress")
        return self.out

    def stream_info(self) -> StreamInfo:
        raw = self.info.cpu().numpy().tobytes()
        return StreamInfo.from_buffer_copy(raw)

    def stream_bytes(self):
        """Device tensor view of the last compressed stream (synchronises)."""
        inf = self.stream_info()
        if inf.status:
            raise SZxError(inf.status, "SZxG_compress")
        return self.out[inf.offset: inf.offset + inf.size]

    def decompress(self, stream, n: int, out=None):
        torch = self.torch
        assert stream.is_cuda and stream.dtype == torch.uint8
        if out is None:
            out = torch.empty(n, dtype=torch.float32 if self.code == SZx_FLOAT else torch.float64,
                              device=stream.device)
        bs = 0 if self.mode == NO_BLOCK else self.bs
        rc = lib().SZxG_decompress(self.mode, self.code, C.c_void_p(stream.data_ptr()), stream.numel(), n, bs,
                                   C.c_void_p(out.data_ptr()), C.c_void_p(self.ws.data_ptr()), self.wsb,
                                   self._stream())
        if rc:
            raise SZxError(rc, "SZxG_decompress")
        return out

    def status(self) -> int:
        return lib().SZxG_workspace_status(C.c_void_p(self.ws.data_ptr()), self._stream())
