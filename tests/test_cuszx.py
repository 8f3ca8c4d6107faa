"""cuSZx ABI (include/cuszx_entry.h): the reference's GPU codec format.

The oracle (oracle/cuszx_oracle.c) restates the reference's cuSZx kernels and
host code from their source, and is pinned to golden vectors the reference's
own cuSZx codec made on a GB300 (tests/golden/cuszx_golden.json, from
tests/golden/make_cuszx_golden.py: 80 cases, 5 fields x 2 sizes x blockSize
32/64/128/224 x 2 bounds): every stream and every decode equals the
reference's, byte for byte.  The CPU tests pin the oracle to those vectors
and its own corner cases; the GPU tests require the library's streams and
decodes to equal the golden vectors and the oracle's bit for bit.

The reference's block range covers the first 32 * 2^floor(log2(bs/32))
values only (its cross-warp reduction, szx/src/cuszx_float.cu:248-256), so
at blockSize 224 (7 warps: the first 128 values) a block can be declared
constant or given too few bits and break the bound; the bound holds when
bs/32 is a power of two.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O


def _fields(seed):
    rng = np.random.default_rng(seed)
    walk = (np.cumsum(rng.normal(size=100_003)) * 1e-2).astype(np.float32)
    steps = np.repeat(rng.uniform(-2, 2, size=2000), 64)[:100_000].astype(np.float32)   # constant blocks
    noise = rng.normal(size=50_000).astype(np.float32)
    runs = np.repeat(rng.uniform(-1, 1, size=10_000), 4).astype(np.float32)             # repeated values
    return {"walk": walk, "steps": steps, "noise": noise, "runs": runs}


# (field, bound) pairs inside the range the reference's codec handles: no
# repeated values at 4 required bytes, no block longer than blockSize * 4 bytes
SOUND = [("walk", 1e-1), ("walk", 1e-3), ("walk", 1e-5), ("steps", 1e-1), ("steps", 1e-3), ("noise", 1e-1),
         ("noise", 1e-3), ("runs", 1e-1), ("runs", 1e-3)]


def test_oracle_round_trips_within_the_bound():
    f = _fields(1)
    for name, eb in SOUND:
        x = f[name]
        for bs in (32, 64, 128):
            s = O.cusz_compress(x, eb, bs)
            y = O.cusz_decompress(s, x.size)
            assert np.abs(y.astype(np.float64) - x).max() <= eb, (name, bs, eb)
            assert s[:5] == bytes([1, 1, 1, 0, bs])


def _golden():
    import hashlib
    import json
    import os
    import sys
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, here)
    import make_cuszx_golden as M
    with open(os.path.join(here, "cuszx_golden.json")) as f:
        g = json.load(f)
    for c in g["cases"]:
        x = M.make_field(c["field"], c["n"], c["seed"])
        assert hashlib.sha256(x.view(np.uint8)).hexdigest() == c["x_sha256"], c["name"]
        yield c, x


def _sha(b):
    import hashlib
    return hashlib.sha256(bytes(b)).hexdigest()


def test_oracle_matches_the_reference_cuszx_golden_vectors():
    n = 0
    for c, x in _golden():
        s = O.cusz_compress(x, c["eb"], c["bs"])
        assert len(s) == c["stream_len"] and _sha(s) == c["stream_sha256"], c["name"]
        y = O.cusz_decompress(s, x.size)
        assert _sha(y.view(np.uint8)) == c["decode_sha256"], c["name"]
        n += 1
    assert n == 80


def test_the_reference_block_range_stops_at_a_power_of_two_of_warps():
    """blockSize 224: a block whose last 96 values move while its first 128
    are flat is constant for the reference (and decodes to the median)."""
    x = np.zeros(224, np.float32)
    x[128:] = 0.5
    s = O.cusz_compress(x, 0.01, 224)
    assert s[5:13] == (1).to_bytes(8, "big")          # one constant block
    assert np.array_equal(O.cusz_decompress(s, 224), np.zeros(224, np.float32))
    s = O.cusz_compress(x, 0.01, 32)
    assert O.cusz_decompress(s, 224)[200] == np.float32(0.5)


def test_oracle_reproduces_the_reference_corner_cases():
    f = _fields(2)
    x = f["runs"]
    # reqLength 25..32 and a value equal to its predecessor: its lead of 4 cannot be coded
    s = O.cusz_compress(x, 2.0 ** -18, 128)
    y = O.cusz_decompress(s, x.size)
    assert not (np.abs(y.astype(np.float64) - x) <= 2.0 ** -18).all()
    # reqLength above 32: the block is longer than the reference decoder accepts
    with pytest.raises(ValueError):
        O.cusz_decompress(O.cusz_compress(x, 2.0 ** -30, 128), x.size)
    # incompressible blocks at 4 required bytes: also longer than a block
    with pytest.raises(ValueError):
        O.cusz_decompress(O.cusz_compress(f["noise"], 1e-5, 32), f["noise"].size)


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a CUDA device is required")
    from szx_gb300 import build
    build.build()
    from szx_gb300._lib import libc
    L = C.CDLL(build.LIB)
    L.cuSZx_fast_compress_args_unpredictable_blocked_float.restype = C.c_void_p
    L.cuSZx_fast_compress_args_unpredictable_blocked_float.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), C.c_float,
                                                                       C.c_size_t, C.c_int]
    L.cuSZx_fast_decompress_args_unpredictable_blocked_float.restype = None
    L.cuSZx_fast_decompress_args_unpredictable_blocked_float.argtypes = [C.POINTER(C.c_void_p), C.c_size_t,
                                                                         C.c_void_p]
    return L, libc()


def _compress(L, libc, x, eb, bs):
    out = C.c_size_t()
    p = L.cuSZx_fast_compress_args_unpredictable_blocked_float(x.ctypes.data, C.byref(out), eb, x.size, bs)
    if not p:
        return None
    s = C.string_at(p, out.value)
    libc.free(p)
    return s


def _decompress(L, libc, s, n):
    buf = np.frombuffer(s, np.uint8).copy()
    p = C.c_void_p()
    L.cuSZx_fast_decompress_args_unpredictable_blocked_float(C.byref(p), n, buf.ctypes.data)
    if not p.value:
        return None
    y = np.frombuffer(C.string_at(p.value, 4 * n), np.float32).copy()
    libc.free(p)
    return y


def _same(a, b):
    """Bitwise equal, any NaN matching any NaN (the oracle does not model the GPU's NaN rules)."""
    na, nb = np.isnan(a), np.isnan(b)
    return bool((na == nb).all() and np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32)))


@pytest.mark.gpu
@pytest.mark.parametrize("bs", [32, 64, 128, 224])
def test_streams_and_values_equal_the_oracle(lib, bs):
    L, libc = lib
    for name, x in _fields(3).items():
        for eb in (1e-1, 1e-3, 1e-5, 2.0 ** -18):
            s = _compress(L, libc, x, eb, bs)
            want = O.cusz_compress(x, eb, bs)
            assert s == want, (name, bs, eb)
            y = _decompress(L, libc, s, x.size)
            try:
                z = O.cusz_decompress(want, x.size)
            except ValueError:
                assert y is None, (name, bs, eb)
                continue
            assert y is not None and _same(y, z), (name, bs, eb)


@pytest.mark.gpu
def test_short_inputs_and_refused_block_sizes(lib):
    L, libc = lib
    x = np.arange(100, dtype=np.float32) * 0.5
    for n in (0, 1, 31, 32, 33, 100):
        s = _compress(L, libc, x[:n].copy(), 1e-2, 32)
        assert s == O.cusz_compress(x[:n], 1e-2, 32), n
        if n:
            assert _same(_decompress(L, libc, s, n), O.cusz_decompress(s, n)), n
    for bs in (16, 48 + 1, 256, 0):
        assert _compress(L, libc, x, 1e-2, bs) is None, bs
    # a stream whose block claims more bytes than a block holds is refused
    s = bytearray(O.cusz_compress(_fields(4)["noise"], 1e-3, 64))
    nb = 50_000 // 64
    o0 = 13 + (nb + 7) // 8 + 4 * (50_000 % 64) + 4 * int.from_bytes(bytes(s[5:13]), "big")
    s[o0:o0 + 2] = (4 * 64).to_bytes(2, "little")
    assert _decompress(L, libc, bytes(s), 50_000) is None


@pytest.mark.gpu
def test_library_matches_the_reference_cuszx_golden_vectors(lib):
    """The library's cuSZx entry points against what the reference's own cuSZx
    codec produced for the same inputs: streams and decodes byte for byte."""
    L, libc = lib
    n = 0
    for c, x in _golden():
        s = _compress(L, libc, x, c["eb"], c["bs"])
        assert s is not None and len(s) == c["stream_len"] and _sha(s) == c["stream_sha256"], c["name"]
        y = _decompress(L, libc, s, x.size)
        assert y is not None and _sha(y.view(np.uint8)) == c["decode_sha256"], c["name"]
        n += 1
    assert n == 80
