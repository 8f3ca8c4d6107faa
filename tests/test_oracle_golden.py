"""The CPU oracle against the reference's own outputs (golden vectors).

The golden vectors were produced by the reference library compiled from its
sources (tests/golden/make_golden.py).  These tests pin the oracle before any
GPU result is compared with it.
"""
import hashlib

import numpy as np
import pytest

import oracle as O


def sha(b) -> str:
    return hashlib.sha256(b).hexdigest()


def bound_of(c) -> float:
    """The absolute bound the reference used for a case (szx/src/szx.cc:249-253, :304-308)."""
    if c["err_mode"] == 0:
        return c["eb"]
    rng = O.value_range(c["x"])[0]
    if c["x"].dtype == np.float32:
        return float(np.float32(rng) * np.float32(c["rel"]))
    return float(np.float32(rng * np.float64(np.float32(c["rel"]))))


def test_golden_set_covers_the_path(golden):
    modes = {(c["dtype"], c["mode"]) for c in golden}
    for dt in ("float32", "float64"):
        for m in (1, 2, 3, 4):
            assert (dt, m) in modes
    assert {c["bs"] for c in golden} >= {64, 128, 256}
    assert any(c["err_mode"] == 1 for c in golden)


def test_oracle_streams_bit_exact(golden):
    for c in golden:
        s = O.fast_compress_args(c["mode"], c["x"], c["err_mode"], c["eb"], c["rel"], c["bs"])
        assert len(s) == c["stream_len"], c["name"]
        assert sha(s) == c["stream_sha256"], c["name"]


def test_oracle_matches_reference_decoder(golden):
    """With the reference-compat switch the oracle reproduces the reference
    decoder bit for bit, including its double reqBytes==5 byte slip."""
    for c in golden:
        d = O.decompress(c["mode"], c["x"].dtype, c["stream"], c["n"], ref_compat=True)
        assert sha(d.tobytes()) == c["ref_decoded_sha256"], c["name"]


def _violations(x, y, eb):
    x = x.astype(np.float64)
    y = y.astype(np.float64)
    ok = np.isfinite(x)
    err = np.abs(x - y)
    # slack of two units in the last place of the value: the reference
    # subtracts and re-adds the median in the data's own precision
    ulp = np.spacing(np.abs(x).astype(np.float32 if x.dtype == np.float32 else np.float64))
    return np.nonzero(ok & (err > eb + 2 * np.abs(ulp)))[0]


def _finite_scope(c):
    """Values whose block (or, for the non-blocked layout, whole array) holds
    no NaN or infinity: elsewhere the reference's median arithmetic itself
    degenerates to NaN and no bound applies."""
    x = c["x"]
    fin = np.isfinite(x)
    if c["mode"] == 1:
        return np.full(x.size, fin.all())
    bs = c["bs"]
    nb = -(-x.size // bs)
    pad = np.ones(nb * bs, bool)
    pad[:x.size] = fin
    blk = pad.reshape(nb, bs).all(axis=1)
    return np.repeat(blk, bs)[:x.size]


def test_oracle_decode_within_bound(golden):
    for c in golden:
        eb = bound_of(c)
        if not np.isfinite(eb):
            continue
        y = O.decompress(c["mode"], c["x"].dtype, c["stream"], c["n"])
        x = c["x"]
        scope = _finite_scope(c)
        bad = _violations(x.astype(np.float64), y, eb)
        bad = bad[scope[bad]]
        if x.dtype == np.float64 and bad.size:
            # fp64 constant blocks store a float median (szx/src/szx_double.cc:1002);
            # the reference itself exceeds the bound there.  Only those may fail.
            nb = -(-x.size // c["bs"])
            _, st, _, _ = O.block_stats(x, eb, c["bs"])
            assert c["mode"] != 1, c["name"]
            assert np.all(st[bad // c["bs"]] == 0), c["name"]
            assert nb > 0
        else:
            assert bad.size == 0, (c["name"], bad[:5])


def test_double_decoder_slip_is_exercised_and_isolated(golden):
    """Where the reference decoder's byte slip bites, the correct decode stays
    within the bound and the reference one does not."""
    hit = 0
    for c in golden:
        if c["x"].dtype != np.float64:
            continue
        a = O.decompress(c["mode"], np.float64, c["stream"], c["n"], ref_compat=True)
        b = O.decompress(c["mode"], np.float64, c["stream"], c["n"], ref_compat=False)
        diff = np.nonzero(a.view(np.uint64) != b.view(np.uint64))[0]
        if diff.size == 0:
            continue
        hit += 1
        eb = bound_of(c)
        x = c["x"]
        diff = diff[_finite_scope(c)[diff]]
        assert _violations(x[diff], b[diff], eb).size == 0, c["name"]
        assert np.any(np.abs(a[diff] - x[diff]) > eb), c["name"]
    assert hit >= 1


def test_omp_codec_matches_serial(golden):
    """The block-parallel CPU baseline emits the serial mode-3 stream."""
    for c in golden:
        if c["mode"] != 3:
            continue
        eb = bound_of(c)
        ser = O.compress(3, c["x"], eb, c["bs"])
        buf, n = O.compress_m3_omp(c["x"], eb, c["bs"], threads=4)
        assert buf[:n].tobytes() == ser, c["name"]
        y = O.decompress_m3_omp(c["x"].dtype, np.frombuffer(ser, np.uint8), len(ser), c["n"], threads=4)
        z = O.decompress(3, c["x"].dtype, ser, c["n"])
        assert np.array_equal(y.view(np.uint8), z.view(np.uint8)), c["name"]


def test_oracle_tiny_and_ragged_sizes():
    """Sizes the reference cannot run (its output buffer is sizeof(T)*n) still
    round-trip within the bound in the oracle."""
    rng = np.random.default_rng(3)
    for dt in (np.float32, np.float64):
        for n in (1, 2, 3, 4, 5, 127, 128, 129, 255, 257):
            x = rng.normal(size=n).astype(dt)
            for mode, bs in ((1, 128), (3, 128), (3, 64), (3, 256), (3, 7), (2, 128), (4, 128)):
                s = O.compress(mode, x, 1e-3, bs)
                y = O.decompress(mode, dt, s, n)
                assert _violations(x.astype(np.float64), y, 1e-3).size == 0, (dt, n, mode, bs)


def _fxr_fields():
    rng = np.random.default_rng(11)
    i = np.arange(1 << 18)
    smooth = np.sin(i / 300.0) + 0.01 * rng.normal(size=i.size)
    steps = np.repeat(rng.normal(size=i.size // 512), 512) + 1e-4 * rng.normal(size=i.size)
    walk = np.cumsum(rng.normal(size=i.size)) * 1e-3
    return {"smooth": smooth, "steps": steps, "walk": walk}


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_fxr_search_matches_reference_when_built(dt):
    """Sampled range, one ratio estimate and the settled bound of the
    fixed-rate search equal the reference's, number for number."""
    if O.reference() is None:
        pytest.skip("reference library not built here (needs the reference sources)")
    for name, f in _fxr_fields().items():
        x = (f * (1e3 if dt == np.float64 else 1.0)).astype(dt)
        bits = lambda v: np.float32(v).view(np.uint32)   # NaN-safe: an all-constant sample gives 0/0
        for scale in (1e-5, 1e-3, 3e-2):
            eb = np.float32(scale * np.ptp(x))
            cr, req, lead, rng_ = O.ref_fxr_estimate(x, eb)
            ocr, oreq, olead, _ = O.fxr_estimate(x, eb)
            assert (bits(ocr), oreq, olead) == (bits(cr), req, lead), (name, scale)
            assert bits(O.fxr_range(x)) == bits(rng_), name
        for ratio in (4.0, 8.0, 16.0, 32.0):
            for tol in (0.05, 0.1):
                assert bits(O.fxr_bound(x, ratio, tol)) == bits(O.ref_fxr_bound(x, ratio, tol)), (name, ratio, tol)
