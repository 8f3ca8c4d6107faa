"""Bounded device waits give up instead of hanging.

The codecs place variable-length payloads with decoupled look-back scans: a
tile waits for its predecessors' status words.  The self-test entry point runs
those same look-back functions with one tile withheld (it never publishes) and
a small poll limit: the waiting tile must give up, the call must report
SZXG_ERR_LOOKBACK within a fraction of a second, and the CUDA context must stay
usable (a normal compress right after still matches the oracle).  With nothing
withheld the scan returns the exact exclusive prefixes.  Nothing faults or
waits without a limit.
"""
import ctypes as C
import time

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

ERR_LOOKBACK = 1


@pytest.fixture(scope="module")
def L():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a CUDA device is required")
    from szx_gb300 import build
    build.build()
    from szx_gb300._lib import lib
    L = lib()
    L.SZxG_selftest_lookback.restype = C.c_int
    L.SZxG_selftest_lookback.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint, C.c_void_p, C.c_void_p]
    return L


def _run(L, scan, ntiles, withheld, limit):
    import torch
    pre = np.zeros(ntiles, np.uint64)
    t0 = time.perf_counter()
    rc = L.SZxG_selftest_lookback(scan, ntiles, withheld, limit, pre.ctypes.data,
                                  C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc, pre, time.perf_counter() - t0


@pytest.mark.parametrize("scan", [0, 1])
def test_lookback_returns_exact_prefixes(L, scan):
    rc, pre, _ = _run(L, scan, 1000, -1, 1 << 22)
    assert rc == 0
    t = np.arange(1000, dtype=np.uint64)
    assert np.array_equal(pre, t * (t + 1) // 2)


@pytest.mark.parametrize("scan", [0, 1])
@pytest.mark.parametrize("withheld", [0, 37, 999])
def test_lookback_gives_up_on_a_tile_that_never_publishes(L, scan, withheld):
    import szx_gb300 as S
    rc, pre, dt = _run(L, scan, 1000, withheld, 4000)
    if withheld == 999:
        # nobody waits on the last tile: no error, and the tiles before it are exact
        assert rc == 0
        t = np.arange(999, dtype=np.uint64)
        assert np.array_equal(pre[:999], t * (t + 1) // 2)
    else:
        assert rc == ERR_LOOKBACK
        assert L.SZxG_get_last_error() == ERR_LOOKBACK
        t = np.arange(withheld, dtype=np.uint64)
        assert np.array_equal(pre[:withheld], t * (t + 1) // 2)   # tiles before the gap are exact
    assert dt < 5.0
    # the context is still usable
    x = np.sin(np.arange(100_000, dtype=np.float32) / 50)
    assert S.fast_compress_args(3, x, S.ABS, 1e-3) == O.fast_compress_args(3, x, 0, 1e-3, 0.0)
