"""ctypes binding of libszx_gb300.so (the C ABI declared in include/szx_gb300.h).

The library is the product: loading fails loudly when it has not been built,
and nothing here computes anything itself.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_lib: C.CDLL | None = None

c_size_p = C.POINTER(C.c_size_t)
c_float_p = C.POINTER(C.c_float)


class StreamInfo(C.Structure):
    """SZxG_StreamInfo."""
    _fields_ = [("offset", C.c_ulonglong), ("size", C.c_ulonglong), ("nb_const", C.c_ulonglong),
                ("eb", C.c_float), ("status", C.c_int)]


def _declare(L: C.CDLL) -> None:
    sz = C.c_size_t
    L.SZx_computeDimension.restype = C.c_int
    L.SZx_computeDimension.argtypes = [sz] * 5
    L.SZx_computeDataLength.restype = sz
    L.SZx_computeDataLength.argtypes = [sz] * 5
    L.SZx_filterDimension.restype = C.c_int
    L.SZx_filterDimension.argtypes = [sz] * 5 + [c_size_p]
    L.SZx_fast_compress_args.restype = C.c_void_p
    L.SZx_fast_compress_args.argtypes = [C.c_int, C.c_int, C.c_void_p, c_size_p, C.c_int, C.c_float, C.c_float,
                                         C.c_float, C.c_float] + [sz] * 5
    L.SZx_fast_decompress.restype = C.c_void_p
    L.SZx_fast_decompress.argtypes = [C.c_int, C.c_int, C.c_void_p, sz] + [sz] * 5
    L.SZx_computeValueRange.restype = C.c_double
    L.SZx_computeValueRange.argtypes = [C.c_void_p, C.c_int, sz, c_float_p, c_float_p]
    L.SZx_fast_compress_args_unpredictable_blocked_randomaccess_openmp.restype = C.c_void_p
    L.SZx_fast_compress_args_unpredictable_blocked_randomaccess_openmp.argtypes = [C.c_void_p, C.c_int, c_size_p,
                                                                                  C.c_float, sz, C.c_int]
    L.SZx_fast_decompress_args_unpredictable_blocked_randomaccess_openmp.restype = C.c_void_p
    L.SZx_fast_decompress_args_unpredictable_blocked_randomaccess_openmp.argtypes = [C.c_int, sz, C.c_void_p]
    L.SZx_estimateErrorBoundbasedonCR.restype = C.c_float
    L.SZx_estimateErrorBoundbasedonCR.argtypes = [C.c_int, C.c_float, C.c_float, C.c_void_p, C.c_float, C.c_int, sz]
    L.SZx_fast_compress_args_unpredictable_blocked.restype = C.c_void_p
    L.SZx_fast_compress_args_unpredictable_blocked.argtypes = [C.c_void_p, C.c_int, c_size_p, C.c_float, sz, C.c_int]
    L.SZx_fast_compress_args_unpredictable_blocked_args.restype = sz
    L.SZx_fast_compress_args_unpredictable_blocked_args.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_float, sz,
                                                                    C.c_int]
    L.SZx_fast_decompress_args_unpredictable_blocked.restype = None
    L.SZx_fast_decompress_args_unpredictable_blocked.argtypes = [C.c_void_p, C.c_int, sz, C.c_void_p]
    L.computeRadiusBuffer.restype = C.c_float
    L.computeRadiusBuffer.argtypes = [C.c_void_p, C.c_int, sz, C.c_int, C.c_int, C.POINTER(c_float_p),
                                      C.POINTER(c_float_p), C.c_void_p]
    L.estimateCRbasedonErrorBound_buffered.restype = C.c_float
    L.estimateCRbasedonErrorBound_buffered.argtypes = [C.c_int, C.c_float, C.c_void_p, c_float_p, c_float_p, C.c_int,
                                                       C.c_int, sz, c_size_p, c_size_p]
    L.SZxG_get_last_error.restype = C.c_int
    L.SZxG_get_last_error.argtypes = []
    L.SZxG_error_string.restype = C.c_char_p
    L.SZxG_error_string.argtypes = [C.c_int]
    L.SZxG_compress_bound.restype = sz
    L.SZxG_compress_bound.argtypes = [C.c_int, C.c_int, sz, C.c_int]
    L.SZxG_workspace_size.restype = sz
    L.SZxG_workspace_size.argtypes = [C.c_int, C.c_int, sz, C.c_int]
    L.SZxG_compress.restype = C.c_int
    L.SZxG_compress.argtypes = [C.c_int, C.c_int, C.c_void_p, sz, C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p,
                                sz, C.c_void_p, sz, C.c_void_p, C.c_void_p]
    L.SZxG_decompress.restype = C.c_int
    L.SZxG_decompress.argtypes = [C.c_int, C.c_int, C.c_void_p, sz, sz, C.c_int, C.c_void_p, C.c_void_p, sz,
                                  C.c_void_p]
    L.SZxG_workspace_status.restype = C.c_int
    L.SZxG_workspace_status.argtypes = [C.c_void_p, C.c_void_p]
    L.SZxG_compress_host.restype = C.c_void_p
    L.SZxG_compress_host.argtypes = [C.c_int, C.c_int, C.c_void_p, sz, C.c_int, C.c_int, C.c_float, C.c_float,
                                     c_size_p]
    L.SZxG_decompress_host.restype = C.c_void_p
    L.SZxG_decompress_host.argtypes = [C.c_int, C.c_int, C.c_void_p, sz, sz]
    L.SZxG_compress_host_into.restype = sz
    L.SZxG_compress_host_into.argtypes = [C.c_int, C.c_int, C.c_void_p, sz, C.c_int, C.c_int, C.c_float, C.c_float,
                                          C.c_void_p, sz]
    L.SZxG_trace_enable.restype = None
    L.SZxG_trace_enable.argtypes = [C.c_int]
    L.SZxG_trace_collect.restype = C.c_int
    L.SZxG_trace_collect.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_double), C.POINTER(C.c_ulonglong),
                                     C.c_int]
    vp, ip, fp = C.c_void_p, C.POINTER(C.c_int), c_float_p
    L.SZxG_batch_create.restype = vp
    L.SZxG_batch_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp]
    L.SZxG_batch_run.restype = C.c_int
    L.SZxG_batch_run.argtypes = [vp, vp, vp]
    L.SZxG_batch_status.restype = C.c_int
    L.SZxG_batch_status.argtypes = [vp, vp]
    L.SZxG_batch_destroy.restype = None
    L.SZxG_batch_destroy.argtypes = [vp]
    L.SZxG_batch_set_bounds.restype = C.c_int
    L.SZxG_batch_set_bounds.argtypes = [vp, C.c_int, ip, fp, vp]
    L.SZxG_mlp_param_count.restype = sz
    L.SZxG_mlp_param_count.argtypes = []
    L.SZxG_mlp_create.restype = vp
    L.SZxG_mlp_create.argtypes = [C.c_ulonglong]
    L.SZxG_mlp_destroy.restype = None
    L.SZxG_mlp_destroy.argtypes = [vp]
    L.SZxG_mlp_get_params.restype = C.c_int
    L.SZxG_mlp_get_params.argtypes = [vp, fp, sz]
    L.SZxG_mlp_set_params.restype = C.c_int
    L.SZxG_mlp_set_params.argtypes = [vp, fp, sz]
    L.SZxG_mlp_forward.restype = C.c_int
    L.SZxG_mlp_forward.argtypes = [vp, vp, sz, vp, vp]
    L.SZxG_mlp_gradient.restype = C.c_int
    L.SZxG_mlp_gradient.argtypes = [vp, vp, vp, sz, vp, fp, vp]
    L.SZxG_mlp_train.restype = C.c_int
    L.SZxG_mlp_train.argtypes = [vp, vp, vp, sz, C.c_int, C.c_int, C.c_float, C.c_ulonglong, fp, vp]
    L.SZxG_batch_features.restype = C.c_int
    L.SZxG_batch_features.argtypes = [vp, C.c_int, ip, fp, vp, fp, vp]
    L.SZxG_batch_fixed_rate.restype = C.c_int
    L.SZxG_batch_fixed_rate.argtypes = [vp, vp, fp, C.c_float, C.c_int, fp, fp, ip, vp, vp]
    L.SZxG_decompress_host_into.restype = C.c_int
    L.SZxG_decompress_host_into.argtypes = [C.c_int, C.c_int, C.c_void_p, sz, sz, C.c_void_p]


def lib() -> C.CDLL:
    """The loaded native library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB):
            raise RuntimeError(f"{_build.LIB} is missing: build it with `python -m szx_gb300.build` "
                               "(szx_gb300 has no CPU fallback)")
        L = C.CDLL(_build.LIB)
        _declare(L)
        _lib = L
    return _lib


def libc() -> C.CDLL:
    c = C.CDLL(None)
    c.free.argtypes = [C.c_void_p]
    c.free.restype = None
    return c
