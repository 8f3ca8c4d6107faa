"""CPU oracle for the SZx codec -- test infrastructure only.

ctypes bindings to ``liboracle.so`` (this project's plain-C restatement of the
reference codec, ``szx_oracle.c``) and, when it has been built, to
``_ref/libszxref.so`` (the reference library compiled from its own sources by
``oracle/Makefile``).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this package; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libszxref.so")
# Where the reference's sources are read from, when they are on this machine:
# the SZX_REFERENCE_SRC environment variable, else the path the build recipe
# (__graft_entry__.build) passes in.  No default: without it only the
# restatement is built.
REF_SRC = os.environ.get("SZX_REFERENCE_SRC", "")

FLOAT, DOUBLE = 0, 1
_u8p = C.POINTER(C.c_uint8)
_lib = None
_ref = None


def build(reference: bool = True, reference_src: str | None = None) -> None:
    """Compile liboracle.so, and the reference library when its sources exist
    (at `reference_src`, else SZX_REFERENCE_SRC)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    src = reference_src or REF_SRC
    if reference and src and os.path.isdir(os.path.join(src, "szx", "src")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={src}"], check=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(reference=False)
        L = C.CDLL(ORACLE_SO)
        L.orc_value_range_f32.restype = C.c_float
        L.orc_value_range_f32.argtypes = [C.c_void_p, C.c_size_t, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_value_range_f64.restype = C.c_double
        L.orc_value_range_f64.argtypes = [C.c_void_p, C.c_size_t, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_capacity.restype = C.c_size_t
        L.orc_capacity.argtypes = [C.c_int, C.c_int, C.c_size_t, C.c_int]
        L.orc_compress.restype = C.c_size_t
        L.orc_compress.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_float, C.c_int, C.c_void_p, C.c_size_t]
        L.orc_fast_compress_args.restype = C.c_size_t
        L.orc_fast_compress_args.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_int, C.c_float,
                                             C.c_float, C.c_int, C.c_void_p, C.c_size_t]
        L.orc_decompress.restype = C.c_int
        L.orc_decompress.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p, C.c_int]
        L.orc_block_stats.restype = C.c_size_t
        L.orc_block_stats.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_float, C.c_int, C.c_void_p,
                                      C.c_void_p, C.c_void_p]
        L.orc_cusz_bound.restype = C.c_size_t
        L.orc_cusz_bound.argtypes = [C.c_size_t, C.c_int]
        L.orc_cusz_compress.restype = C.c_size_t
        L.orc_cusz_compress.argtypes = [C.c_void_p, C.c_size_t, C.c_float, C.c_int, C.c_void_p]
        L.orc_cusz_decompress.restype = C.c_int
        L.orc_cusz_decompress.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p]
        L.orc_compress_m3_omp.restype = C.c_size_t
        L.orc_compress_m3_omp.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_float, C.c_int, C.c_void_p,
                                          C.c_size_t, C.c_int]
        L.orc_decompress_m3_omp.restype = C.c_int
        L.orc_decompress_m3_omp.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p, C.c_int]
        L.orc_fxr_estimate_cr_f32.restype = C.c_float
        L.orc_fxr_estimate_cr_f32.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_float,
                                              C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
        L.orc_fxr_bound_f32.restype = C.c_float
        L.orc_fxr_bound_f32.argtypes = [C.c_void_p, C.c_size_t, C.c_float, C.c_float, C.c_int]
        L.orc_fxr_range.restype = C.c_float
        L.orc_fxr_range.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_int]
        L.orc_fxr_estimate_cr.restype = C.c_float
        L.orc_fxr_estimate_cr.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_int, C.c_float,
                                          C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
        L.orc_fxr_bound.restype = C.c_float
        L.orc_fxr_bound.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_float, C.c_float, C.c_int]
        _lib = L
    return _lib


def _dt(arr: np.ndarray) -> int:
    if arr.dtype == np.float32:
        return FLOAT
    if arr.dtype == np.float64:
        return DOUBLE
    raise TypeError(f"unsupported dtype {arr.dtype}")


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def capacity(mode: int, dtype: int, n: int, bs: int = 128) -> int:
    return lib().orc_capacity(mode, dtype, n, bs)


def value_range(x: np.ndarray):
    x = np.ascontiguousarray(x)
    r, m = C.c_float(), C.c_float()
    fn = lib().orc_value_range_f32 if _dt(x) == FLOAT else lib().orc_value_range_f64
    v = fn(_ptr(x), x.size, C.byref(r), C.byref(m))
    return v, r.value, m.value


def compress(mode: int, x: np.ndarray, eb: float, bs: int = 128) -> bytes:
    x = np.ascontiguousarray(x)
    cap = capacity(mode, _dt(x), x.size, bs)
    out = np.empty(max(cap, 1), np.uint8)
    n = lib().orc_compress(mode, _dt(x), _ptr(x), x.size, eb, bs, _ptr(out), cap)
    if n == 0:
        raise ValueError("oracle compress failed")
    return out[:n].tobytes()


def fast_compress_args(mode: int, x: np.ndarray, err_mode: int, abs_eb: float, rel: float, bs: int = 128) -> bytes:
    x = np.ascontiguousarray(x)
    cap = capacity(mode, _dt(x), x.size, bs)
    out = np.empty(max(cap, 1), np.uint8)
    n = lib().orc_fast_compress_args(mode, _dt(x), _ptr(x), x.size, err_mode, abs_eb, rel, bs, _ptr(out), cap)
    if n == 0:
        raise ValueError("oracle compress failed")
    return out[:n].tobytes()


def decompress(mode: int, dtype, stream: bytes, n: int, ref_compat: bool = False) -> np.ndarray:
    dt = np.dtype(dtype)
    out = np.empty(n, dt)
    s = np.frombuffer(stream, np.uint8)
    rc = lib().orc_decompress(mode, FLOAT if dt == np.float32 else DOUBLE, _ptr(s), s.size, n, _ptr(out),
                              int(ref_compat))
    if rc != 0:
        raise ValueError(f"oracle decompress failed ({rc})")
    return out


def block_stats(x: np.ndarray, eb: float, bs: int = 128):
    x = np.ascontiguousarray(x)
    nb = -(-x.size // bs)
    st = np.empty(nb, np.uint8)
    med = np.empty(nb, np.float32)
    rad = np.empty(nb, np.float32)
    nc = lib().orc_block_stats(_dt(x), _ptr(x), x.size, eb, bs, _ptr(st), _ptr(med), _ptr(rad))
    return nc, st, med, rad


def compress_m3_omp(x: np.ndarray, eb: float, bs: int = 128, threads: int = 0, out: np.ndarray | None = None):
    x = np.ascontiguousarray(x)
    cap = capacity(3, _dt(x), x.size, bs)
    if out is None or out.size < cap:
        out = np.empty(cap, np.uint8)
    n = lib().orc_compress_m3_omp(_dt(x), _ptr(x), x.size, eb, bs, _ptr(out), cap, threads)
    return out, n


def decompress_m3_omp(dtype, stream: np.ndarray, length: int, n: int, threads: int = 0,
                      out: np.ndarray | None = None) -> np.ndarray:
    dt = np.dtype(dtype)
    if out is None:
        out = np.empty(n, dt)
    rc = lib().orc_decompress_m3_omp(FLOAT if dt == np.float32 else DOUBLE, _ptr(stream), length, n, _ptr(out),
                                     threads)
    if rc != 0:
        raise ValueError(f"oracle decompress failed ({rc})")
    return out


def fxr_bound(x: np.ndarray, ratio: float, tolerance: float, bs: int = 128) -> float:
    """Error bound the reference fixed-rate search settles on (float or double data)."""
    x = np.ascontiguousarray(x)
    return lib().orc_fxr_bound(_dt(x), _ptr(x), x.size, ratio, tolerance, bs)


def fxr_range(x: np.ndarray, bs: int = 128) -> float:
    """Value range over the sampled blocks (every 10th block of bs values)."""
    x = np.ascontiguousarray(x)
    return lib().orc_fxr_range(_dt(x), _ptr(x), x.size, bs)


def fxr_estimate(x: np.ndarray, eb: float, bs: int = 128):
    """(ratio estimate, sum of required bytes, sum of leads, constant sampled blocks)."""
    x = np.ascontiguousarray(x)
    a, b, c = C.c_size_t(), C.c_size_t(), C.c_size_t()
    cr = lib().orc_fxr_estimate_cr(_dt(x), _ptr(x), x.size, bs, eb, C.byref(a), C.byref(b), C.byref(c))
    return cr, a.value, b.value, c.value


# ---------------------------------------------------------------- reference library

def reference() -> C.CDLL | None:
    """The reference library built from its sources, or None where it is absent."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            return None
        R = C.CDLL(REF_SO)
        R.SZx_fast_compress_args.restype = C.c_void_p
        R.SZx_fast_compress_args.argtypes = [C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_size_t), C.c_int,
                                             C.c_float, C.c_float, C.c_float, C.c_float] + [C.c_size_t] * 5
        R.SZx_fast_decompress.restype = C.c_void_p
        R.SZx_fast_decompress.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_size_t] + [C.c_size_t] * 5
        R.ref_compress_blocked.restype = C.c_void_p
        R.ref_compress_blocked.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_float, C.c_int,
                                           C.POINTER(C.c_size_t)]
        R.ref_fxr_bound_float.restype = C.c_float
        R.ref_fxr_bound_float.argtypes = [C.c_void_p, C.c_size_t, C.c_float, C.c_float, C.c_int]
        R.ref_fxr_bound_double.restype = C.c_float
        R.ref_fxr_bound_double.argtypes = [C.c_void_p, C.c_size_t, C.c_float, C.c_float, C.c_int]
        R.ref_fxr_estimate.restype = C.c_float
        R.ref_fxr_estimate.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_int, C.c_float, C.POINTER(C.c_size_t),
                                       C.POINTER(C.c_size_t), C.POINTER(C.c_float)]
        R.ref_free.restype = None
        R.ref_free.argtypes = [C.c_void_p]
        _ref = R
    return _ref


def _take(R, p: int, nbytes: int) -> bytes:
    b = C.string_at(p, nbytes)
    R.ref_free(p)
    return b


def ref_compress_args(mode: int, x: np.ndarray, err_mode: int, abs_eb: float, rel: float, ratio: float = 0.0,
                      tolerance: float = 0.0) -> bytes:
    """SZx_fast_compress_args of the reference (block size 128)."""
    R = reference()
    x = np.ascontiguousarray(x)
    sz = C.c_size_t()
    p = R.SZx_fast_compress_args(mode, _dt(x), _ptr(x), C.byref(sz), err_mode, abs_eb, rel, ratio, tolerance,
                                 0, 0, 0, 0, x.size)
    return _take(R, p, sz.value)


def ref_compress_blocked(mode: int, x: np.ndarray, eb: float, bs: int) -> bytes:
    R = reference()
    x = np.ascontiguousarray(x)
    sz = C.c_size_t()
    p = R.ref_compress_blocked(mode, _dt(x), _ptr(x), x.size, eb, bs, C.byref(sz))
    return _take(R, p, sz.value)


def ref_decompress(mode: int, dtype, stream: bytes, n: int) -> np.ndarray:
    R = reference()
    dt = np.dtype(dtype)
    s = np.frombuffer(stream, np.uint8).copy()
    p = R.SZx_fast_decompress(mode, FLOAT if dt == np.float32 else DOUBLE, _ptr(s), s.size, 0, 0, 0, 0, n)
    out = np.frombuffer(_take(R, p, n * dt.itemsize), dt).copy()
    return out


def ref_fxr_bound(x: np.ndarray, ratio: float, tolerance: float, bs: int = 128) -> float:
    x = np.ascontiguousarray(x)
    R = reference()
    f = R.ref_fxr_bound_float if x.dtype == np.float32 else R.ref_fxr_bound_double
    return f(_ptr(x), x.size, ratio, tolerance, bs)


def ref_fxr_estimate(x: np.ndarray, eb: float, bs: int = 128):
    """(ratio estimate, sum of required bytes, sum of leads, sampled range) from the reference."""
    x = np.ascontiguousarray(x)
    a, b, r = C.c_size_t(), C.c_size_t(), C.c_float()
    cr = reference().ref_fxr_estimate(_dt(x), _ptr(x), x.size, bs, eb, C.byref(a), C.byref(b), C.byref(r))
    return cr, a.value, b.value, r.value


def cusz_compress(x: np.ndarray, eb: float, bs: int) -> bytes:
    """The cuSZx float stream of x (cuszx_oracle.c)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty(lib().orc_cusz_bound(x.size, bs), np.uint8)
    n = lib().orc_cusz_compress(_ptr(x), x.size, eb, bs, _ptr(out))
    return out[:n].tobytes()


def cusz_decompress(stream: bytes, n: int) -> np.ndarray:
    s = np.frombuffer(stream, np.uint8).copy()
    y = np.zeros(n, np.float32)
    if lib().orc_cusz_decompress(_ptr(s), s.size, n, _ptr(y)) != 0:
        raise ValueError("oracle: malformed cuSZx stream")
    return y
