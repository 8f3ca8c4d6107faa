"""Fixed-rate mode (errBoundMode FXR): the reference's sampled-ratio search.

Expected values come from tests/golden/fxr.json, written by
tests/golden/make_fxr_golden.py from the reference library itself on the
deterministic fields of tests/golden/fields.py.  The CPU test checks that the
oracle restatement reproduces them; the GPU tests check the library: sampled
range and ratio estimates (computeRadiusBuffer /
estimateCRbasedonErrorBound_buffered), the settled bound, and the fixed-rate
stream of SZx_fast_compress_args (bit-exact where the reference could write it,
otherwise equal to the oracle's fastMode-2 stream at the reference's bound).
"""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import fields as F  # noqa: E402
import oracle as O  # noqa: E402

FXR = 2
GOLD = json.load(open(os.path.join(HERE, "golden", "fxr.json")))["fields"]


def _f32(b: int) -> np.float32:
    return np.uint32(b).view(np.float32)


def _bits(v) -> int:
    return int(np.float32(v).view(np.uint32))


def _cases():
    for g in GOLD:
        yield g, F.make(g["field"], g["n"], np.dtype(g["dtype"]))


def test_oracle_reproduces_fixed_rate_fixtures():
    for g, x in _cases():
        assert _bits(O.fxr_range(x)) == g["range_bits"], g["field"]
        for e in g["estimates"]:
            cr, req, lead, _ = O.fxr_estimate(x, e["eb"])
            assert (_bits(cr), req, lead) == (e["cr_bits"], e["sum_req"], e["sum_lead"]), (g["field"], e["eb"])
        for s in g["searches"]:
            assert _bits(O.fxr_bound(x, s["ratio"], s["tolerance"])) == s["eb_bits"], (g["field"], s)


@pytest.fixture(scope="module")
def szx():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a CUDA device is required")
    from szx_gb300 import build
    build.build()
    import szx_gb300
    return szx_gb300


@pytest.mark.gpu
def test_sampled_range_and_estimates_match_reference(szx):
    from szx_gb300 import api
    for g, x in _cases():
        rng, rads, meds, buf = api.compute_radius_buffer(x, 10, 128)
        assert _bits(rng) == g["range_bits"], g["field"]
        ns = x.size // 1280
        assert rads.size == ns and buf.size == ns * 128
        assert np.array_equal(buf.reshape(ns, 128), x[: ns * 1280].reshape(ns, 1280)[:, :128])
        for e in g["estimates"]:
            cr, req, lead = api.estimate_cr_buffered(buf, meds, rads, e["eb"], x.size, 10, 128)
            assert (_bits(cr), req, lead) == (e["cr_bits"], e["sum_req"], e["sum_lead"]), (g["field"], e["eb"])


@pytest.mark.gpu
def test_fixed_rate_streams_match_reference(szx):
    from szx_gb300 import api
    for g, x in _cases():
        for s in g["searches"]:
            got = api.fast_compress_args(3, x, FXR, compressionRatio=s["ratio"], tolerance=s["tolerance"])
            assert got[:4] == bytes([1, 1, 1, 0]) and got[4] == 128   # fastMode-2 layout, whatever fastMode says
            if "stream_sha256" in s:
                assert len(got) == s["stream_len"], (g["field"], s)
                assert hashlib.sha256(got).hexdigest() == s["stream_sha256"], (g["field"], s)
            else:
                assert got == O.compress(2, x, _f32(s["eb_bits"]), 128), (g["field"], s)


@pytest.mark.gpu
def test_unbuffered_bound_search_runs_and_is_deterministic(szx):
    from szx_gb300 import api
    x = F.make("smooth", 1 << 18, np.float32)
    init = float(np.float32(np.ptp(x)) * np.float32(1e-2))
    a = api.estimate_error_bound(x, 8.0, 0.05, init, 128)
    b = api.estimate_error_bound(x, 8.0, 0.05, init, 128)
    assert a == b and np.isfinite(a) and a > 0
