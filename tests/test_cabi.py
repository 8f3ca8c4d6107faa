"""The C-ABI library: it loads without a GPU, exports every symbol the public
headers (include/*.h) declare, and its host-only helpers behave like the
reference's."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
HEADERS = sorted(os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h"))


@pytest.fixture(scope="module")
def L():
    from szx_gb300 import build
    build.build()
    from szx_gb300._lib import lib
    return lib()


def _text():
    return re.sub(r"/\*.*?\*/", "", "\n".join(open(h).read() for h in HEADERS), flags=re.S)


def declared_functions():
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", _text())
    return sorted({n for n in names if n not in ("if", "sizeof")})


def declared_variables():
    return sorted(set(re.findall(r"^\s*extern\s+[A-Za-z_][A-Za-z0-9_ ]*?\b([A-Za-z_][A-Za-z0-9_]*)\s*;", _text(),
                                 flags=re.M)))


def test_header_declares_the_reference_entry_points():
    names = declared_functions()
    for ref in ("SZx_fast_compress_args", "SZx_fast_decompress", "SZx_computeDataLength", "SZx_computeDimension",
                "SZx_filterDimension", "SZx_computeValueRange",
                "SZx_fast_compress_args_unpredictable_blocked_randomaccess_openmp",
                "SZx_fast_decompress_args_unpredictable_blocked_randomaccess_openmp",
                "SZx_estimateErrorBoundbasedonCR", "SZx_fast_compress_args_unpredictable_blocked",
                "computeRadiusBuffer", "estimateCRbasedonErrorBound_buffered",
                "SZx_fast_compress_args_unpredictable_blocked_args",
                "SZx_fast_decompress_args_unpredictable_blocked"):
        assert ref in names, ref


def test_library_exports_every_declared_symbol(L):
    names = declared_functions() + declared_variables()
    assert len(names) > 20 and "SZx_readFloatData" in names and "dataEndianType" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_dimension_helpers_match_reference_rules(L):
    # szx/src/szx.cc:41-101
    assert L.SZx_computeDimension(0, 0, 0, 0, 0) == 0
    assert L.SZx_computeDimension(0, 0, 0, 0, 7) == 1
    assert L.SZx_computeDimension(0, 0, 512, 512, 512) == 3
    assert L.SZx_computeDimension(2, 3, 4, 5, 6) == 5
    assert L.SZx_computeDataLength(0, 0, 0, 0, 0) == 0
    assert L.SZx_computeDataLength(0, 0, 512, 512, 512) == 512 ** 3
    assert L.SZx_computeDataLength(2, 3, 4, 5, 6) == 720
    # szx/src/szx.cc:109-229
    c = (C.c_size_t * 5)()
    assert L.SZx_filterDimension(0, 0, 4, 1, 6, c) == 1 and list(c)[:3] == [6, 4, 0]
    assert L.SZx_filterDimension(0, 0, 0, 0, 5, c) == 0 and c[0] == 5
    assert L.SZx_filterDimension(0, 0, 0, 3, 1, c) == 1 and list(c)[:2] == [3, 0]


def test_bounds_and_workspace_sizes(L):
    import numpy as np

    import oracle as O
    rng = np.random.default_rng(5)
    for dt, npdt in ((0, np.float32), (1, np.float64)):
        es = 4 if dt == 0 else 8
        for n in (1, 3, 1000, 4099, 1 << 20):
            worst = rng.normal(size=min(n, 5000)).astype(npdt) if n <= 5000 else None
            for mode, bs in ((1, 128), (3, 128), (3, 64), (3, 256), (2, 128), (4, 128)):
                b = L.SZxG_compress_bound(mode, dt, n, bs)
                assert b <= 2 * es * n + 4096
                if worst is not None:
                    # incompressible data at a negligible bound is the largest stream
                    assert b >= len(O.compress(mode, worst, 1e-30, bs)) + 16, (dt, n, mode, bs)
                assert L.SZxG_workspace_size(mode, dt, n, bs) > 0
    assert L.SZxG_compress_bound(9, 0, 10, 128) == 0


def test_error_strings(L):
    for code in range(7):
        assert L.SZxG_error_string(code)
    assert L.SZxG_error_string(0) == b"ok"


def test_unsupported_paths_fail_cleanly_without_touching_the_gpu(L):
    import numpy as np
    x = np.zeros(16, np.float32)
    sz = C.c_size_t(123)
    # bad arguments are rejected before any device work
    assert not L.SZx_fast_compress_args(7, 0, x.ctypes.data, C.byref(sz), 0, 1e-3, 0.0, 0.0, 0.0, 0, 0, 0, 0, 16)
    assert L.SZxG_get_last_error() == 4
    assert not L.SZx_fast_compress_args(3, 5, x.ctypes.data, C.byref(sz), 0, 1e-3, 0.0, 0.0, 0.0, 0, 0, 0, 0, 16)
    # a fastMode-2 stream whose block size byte is 0 is malformed
    assert not L.SZx_fast_decompress(2, 0, x.ctypes.data, 64, 0, 0, 0, 0, 16)
    assert L.SZxG_get_last_error() == 3
