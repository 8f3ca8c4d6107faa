"""Parity of the CUDA codec (through the C ABI) with the oracle and the
reference's golden vectors.  Integer/byte work: everything is bit-exact.

Decoded double values are compared with the oracle's faithful decode, not
with the reference decoder's reqBytes==5 byte slip (szx/src/szxd_double.cc:244);
tests/test_oracle_golden.py shows the two differ only there.
"""
import hashlib
import zlib

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def szx():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a CUDA device is required for the gpu tests")
    import szx_gb300
    from szx_gb300 import build
    build.build()
    return szx_gb300


def sha(b):
    return hashlib.sha256(b).hexdigest()


def same_bits(a, b):
    return a.dtype == b.dtype and a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def gpu_compress(szx, c):
    if c["bs"] == 128 and c["mode"] in (1, 3):
        return szx.fast_compress_args(c["mode"], c["x"], c["err_mode"], c["eb"], c["rel"])
    return szx.compress_host(c["mode"], c["x"], c["bs"], c["err_mode"], c["eb"], c["rel"])


def test_golden_streams_bit_exact(szx, golden):
    for c in golden:
        s = gpu_compress(szx, c)
        assert len(s) == c["stream_len"], c["name"]
        assert sha(s) == c["stream_sha256"], c["name"]


def test_golden_decode_bit_exact(szx, golden):
    for c in golden:
        y = szx.decompress_host(c["mode"], c["x"].dtype, c["stream"], c["n"])
        z = O.decompress(c["mode"], c["x"].dtype, c["stream"], c["n"])
        assert same_bits(y, z), c["name"]
        if c["x"].dtype == np.float32 and c["bs"] == 128:
            # and through the reference's own decode entry point
            w = szx.fast_decompress(c["mode"], np.float32, c["stream"], c["n"])
            assert same_bits(w, z), c["name"]


def _field(rng, kind, n, dt):
    i = np.arange(n)
    if kind == "smooth":
        x = sum(rng.uniform(0.1, 1) * np.sin(2 * np.pi * rng.integers(1, 65) * i / n) for _ in range(8))
        x = x + rng.normal(0, 1e-3, n)
        x = x.astype(dt)
        nb = n // 128
        for b in np.nonzero(rng.random(nb) < 0.1)[0]:
            x[b * 128:(b + 1) * 128] = x[b * 128]
        return x
    if kind == "noise":
        return rng.normal(0, 1, n).astype(dt)
    if kind == "walk":
        return (np.cumsum(rng.normal(0, 1, n)) * 0.01).astype(dt)
    if kind == "offset":
        return (rng.normal(0, 1, n) * 1e3 + 1e7).astype(dt)
    if kind == "slabs":
        x = rng.normal(0, 1, n).astype(dt)
        x[n // 3: n // 2] = 0
        return x
    raise ValueError(kind)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("kind", ["smooth", "noise", "walk", "offset", "slabs"])
def test_seeded_fields_match_oracle(szx, dt, kind):
    rng = np.random.default_rng(zlib.crc32(f"{kind}{np.dtype(dt).itemsize}".encode()))
    n = 1_000_003
    x = _field(rng, kind, n, dt)
    for mode, bs in ((1, 128), (3, 128), (3, 64), (3, 256), (2, 128), (4, 128)):
        for err_mode, eb, rel in ((0, 1e-3, 0.0), (1, 0.0, 1e-4), (1, 0.0, 1e-2)):
            want = O.fast_compress_args(mode, x, err_mode, eb, rel, bs)
            got = szx.compress_host(mode, x, bs, err_mode, eb, rel)
            assert got == want, (kind, mode, bs, err_mode, rel)
            y = szx.decompress_host(mode, dt, got, n)
            z = O.decompress(mode, dt, want, n)
            assert same_bits(y, z), (kind, mode, bs, err_mode, rel)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_every_block_size_and_ragged_length(szx, dt):
    rng = np.random.default_rng(17)
    for bs in (1, 2, 3, 5, 8, 31, 32, 33, 63, 64, 65, 100, 127, 128, 129, 200, 255, 256):
        for n in (1, 2, bs, bs + 1, 3 * bs - 1, 4097):
            x = (np.sin(np.arange(n) / 17.0) + rng.normal(0, 1e-2, n)).astype(dt)
            for mode in ((3, 2) if bs <= 255 else (3,)):
                want = O.compress(mode, x, 1e-3, bs)
                got = szx.compress_host(mode, x, bs, 0, 1e-3, 0.0)
                assert got == want, (mode, bs, n)
                assert same_bits(szx.decompress_host(mode, dt, got, n), O.decompress(mode, dt, want, n)), (mode, bs, n)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_tiny_arrays_all_modes(szx, dt):
    rng = np.random.default_rng(23)
    for n in (1, 2, 3, 4, 5, 15, 16, 17, 127, 128, 129, 4095, 4096, 4097, 8193):
        x = rng.normal(size=n).astype(dt)
        for mode in (1, 2, 3, 4):
            want = O.compress(mode, x, 1e-2, 128)
            got = szx.compress_host(mode, x, 128, 0, 1e-2, 0.0)
            assert got == want, (n, mode)
            assert same_bits(szx.decompress_host(mode, dt, got, n), O.decompress(mode, dt, want, n)), (n, mode)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_special_values(szx, dt):
    """NaN first / later, infinities, signed zeros, all-constant, huge dynamic
    range, reqLength clamps: the GPU follows the reference's sequential
    min/max and arithmetic exactly."""
    n = 4096
    rng = np.random.default_rng(29)
    cases = []
    x = rng.normal(size=n).astype(dt); x[0] = np.nan; cases.append(x)
    x = rng.normal(size=n).astype(dt); x[5::97] = np.nan; cases.append(x)
    x = rng.normal(size=n).astype(dt); x[130] = np.inf; x[700] = -np.inf; cases.append(x)
    x = np.where(rng.random(n) < 0.5, -0.0, 0.0).astype(dt); cases.append(x)
    x = np.where(rng.random(n) < 0.5, -0.0, 0.0).astype(dt); x[::3] = rng.normal(size=x[::3].size); cases.append(x)
    x = np.abs(rng.normal(size=n)).astype(dt); x[::5] = 0.0; x[7::11] = -0.0; cases.append(x)
    cases.append(np.full(n, 3.5, dt))
    cases.append((rng.normal(size=n) * 1e30).astype(dt))
    cases.append((1e6 + np.sin(np.arange(n) / 30.0)).astype(dt))
    for k, x in enumerate(cases):
        for mode in (1, 3):
            for eb in (1e-6, 1e-2):
                want = O.compress(mode, x, eb, 128)
                got = szx.compress_host(mode, x, 128, 0, eb, 0.0)
                assert got == want, (k, mode, eb)
                assert same_bits(szx.decompress_host(mode, dt, got, n), O.decompress(mode, dt, want, n)), (k, mode)
        # REL takes the range from the same sequential min/max semantics
        if not np.isnan(x).any() and not np.isinf(x).any():
            want = O.fast_compress_args(3, x, 1, 0.0, 1e-3, 128)
            assert szx.compress_host(3, x, 128, 1, 0.0, 1e-3) == want, k


def test_value_range_entry_point(szx):
    rng = np.random.default_rng(31)
    for dt in (np.float32, np.float64):
        x = rng.normal(size=100_001).astype(dt)
        x[0] = -0.0
        v, r, m = szx.compute_value_range(x)
        w, rr, mm = O.value_range(x)
        assert (v, r, m) == (w, rr, mm)


def test_device_api_matches_host_api(szx):
    import torch
    rng = np.random.default_rng(37)
    for dt, tdt in ((np.float32, torch.float32), (np.float64, torch.float64)):
        n = 300_001
        x = (np.sin(np.arange(n) / 50.0) + rng.normal(0, 1e-3, n)).astype(dt)
        for mode, bs in ((3, 128), (1, 128), (4, 64)):
            codec = szx.DeviceCodec(mode, dt, n, bs)
            xt = torch.from_numpy(x).cuda()
            codec.compress(xt, 1, 0.0, 1e-3)
            s = codec.stream_bytes()
            want = O.fast_compress_args(mode, x, 1, 0.0, 1e-3, bs)
            assert s.cpu().numpy().tobytes() == want, (dt, mode)
            y = codec.decompress(s.clone(), n)
            torch.cuda.synchronize()
            assert codec.status() == 0
            assert same_bits(y.cpu().numpy(), O.decompress(mode, dt, want, n)), (dt, mode)
            # two calls in a row on the same buffers give the same stream
            codec.compress(xt, 1, 0.0, 1e-3)
            assert codec.stream_bytes().cpu().numpy().tobytes() == want


def test_corrupt_and_truncated_streams_fail_cleanly(szx):
    rng = np.random.default_rng(41)
    x = rng.normal(size=50_000).astype(np.float32)
    s = szx.fast_compress_args(3, x, 0, 1e-3)
    with pytest.raises(szx.SZxError):
        szx.fast_decompress(3, np.float32, s[:100], x.size)
    with pytest.raises(szx.SZxError):
        szx.fast_decompress(3, np.float32, s[: len(s) // 2], x.size)
    bad = bytearray(s)
    bad[12:20] = (10 ** 9).to_bytes(8, "big")   # more constant blocks than blocks
    with pytest.raises(szx.SZxError):
        szx.fast_decompress(3, np.float32, bytes(bad), x.size)
    s1 = szx.fast_compress_args(1, x, 0, 1e-3)
    with pytest.raises(szx.SZxError):
        szx.fast_decompress(1, np.float32, s1[: len(s1) - 1000], x.size)
    with pytest.raises(szx.SZxError):   # shorter than the fastMode-1 header
        szx.fast_decompress(1, np.float32, s1[:10], x.size)
    for req in (0, 65):                  # reqLength outside 1..64
        bad1 = bytearray(s1)
        bad1[4] = req
        with pytest.raises(szx.SZxError):
            szx.fast_decompress(1, np.float32, bytes(bad1), x.size)
    # a lead-code count that does not match the value count
    bad1 = bytearray(s1)
    bad1[9:17] = ((x.size + 3) // 4 + 1).to_bytes(8, "big")
    with pytest.raises(szx.SZxError):
        szx.fast_decompress(1, np.float32, bytes(bad1), x.size)
    # lead codes scrambled: whatever the counts say, every read stays inside
    # the stream (an error or some values, never a fault)
    bad1 = bytearray(s1)
    bad1[17:17 + 4096] = np.random.default_rng(5).integers(0, 256, 4096, dtype=np.uint8).tobytes()
    try:
        szx.fast_decompress(1, np.float32, bytes(bad1), x.size)
    except szx.SZxError:
        pass
    # the library still works afterwards
    assert szx.fast_compress_args(3, x, 0, 1e-3) == s
    assert szx.fast_decompress(1, np.float32, s1, x.size).tobytes() == \
        O.decompress(1, np.float32, s1, x.size).tobytes()


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_mode2_decode_large_and_periodic(szx, dt):
    """fastMode 2 has no size index: block boundaries come from a parallel
    speculative search.  A large field exercises many segments; a periodic
    field (identical blocks) makes false walks survive in step with the true
    one, which the search must detect and repair."""
    rng = np.random.default_rng(31)
    n = 3_000_017
    x = (np.cumsum(rng.normal(size=n)) * 1e-2).astype(dt)
    for eb in (1e-4, 1e-2):
        s = szx.compress_host(2, x, 128, 0, eb, 0.0)
        assert s == O.compress(2, x, eb, 128)
        assert same_bits(szx.decompress_host(2, dt, s, n), O.decompress(2, dt, s, n)), eb
    tile = rng.normal(size=128 * 7).astype(dt)
    xp = np.tile(tile, 4000)
    s = szx.compress_host(2, xp, 128, 0, 1e-3, 0.0)
    assert s == O.compress(2, xp, 1e-3, 128)
    assert same_bits(szx.decompress_host(2, dt, s, xp.size), O.decompress(2, dt, s, xp.size))


def test_mode2_entry_point_without_length(szx):
    """SZx_fast_decompress_args_unpredictable_blocked takes no stream length."""
    import ctypes as C
    from szx_gb300._lib import lib, libc
    rng = np.random.default_rng(37)
    for dt, code in ((np.float32, 0), (np.float64, 1)):
        x = rng.normal(size=100_003).astype(dt)
        s = np.frombuffer(O.compress(2, x, 1e-2, 128), np.uint8).copy()
        out = C.c_void_p()
        lib().SZx_fast_decompress_args_unpredictable_blocked(C.byref(out), code, x.size, s.ctypes.data)
        assert out.value
        y = np.frombuffer(C.string_at(out.value, x.nbytes), dt).copy()
        libc().free(out)
        assert same_bits(y, O.decompress(2, dt, s.tobytes(), x.size))


def test_fixed_rate_round_trip_within_the_bound(szx):
    """A fixed-rate stream (fastMode-2 layout) decodes through the drop-in
    entry point within the bound the search chose."""
    rng = np.random.default_rng(41)
    x = (np.cumsum(rng.normal(size=1 << 20)) * 1e-2).astype(np.float32)
    for ratio in (4.0, 8.0, 16.0):
        s = szx.fast_compress_args(3, x, 2, compressionRatio=ratio, tolerance=0.1)
        eb = O.fxr_bound(x, ratio, 0.1)
        y = szx.fast_decompress(2, np.float32, s, x.size)
        assert np.max(np.abs(y.astype(np.float64) - x)) <= eb * (1 + 1e-6), ratio
