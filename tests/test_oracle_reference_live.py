"""Live cross-check of the oracle against the reference library, compiled from
the reference sources by oracle/Makefile.  Skipped where the reference is not
available (it is never shipped with this repository)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.skipif(O.reference() is None, reason="reference library not built here")


def _fields(rng, n, dt):
    i = np.arange(n)
    yield (sum(rng.uniform(0.1, 1) * np.sin(2 * np.pi * rng.integers(1, 64) * i / n) for _ in range(8))
           + rng.normal(0, 1e-3, n)).astype(dt)
    yield rng.normal(0, 1, n).astype(dt)
    yield (np.cumsum(rng.normal(0, 1, n)) * 0.01).astype(dt)
    yield (rng.normal(0, 1, n) * 1e6 + 3e7).astype(dt)


def _fits_reference(mode, x, eb, bs):
    s = O.compress(mode, x, eb, bs)
    if len(s) >= x.nbytes - 64:
        return False
    if mode == 4:
        s3 = np.frombuffer(O.compress(3, x, eb, bs), np.uint8)
        nb = -(-x.size // bs)
        nnc = nb - int.from_bytes(s3[12:20].tobytes(), "big")
        if nnc and s3[20:20 + 2 * nnc].view("<u2").max() > 4 * bs:
            return False
    return True


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_streams_and_decodes_match_reference(dt):
    rng = np.random.default_rng(7)
    checked = 0
    for n in (1000, 4096, 9999):
        for x in _fields(rng, n, dt):
            r = float(x.max()) - float(x.min())
            for rel in (1e-1, 1e-3, 1e-5):
                eb = float(np.float32(rel * r))
                for mode, bs in ((1, 128), (2, 128), (3, 128), (3, 64), (3, 256), (4, 128)):
                    if not _fits_reference(mode, x, eb, bs):
                        continue
                    so = O.compress(mode, x, eb, bs)
                    sr = O.ref_compress_args(1, x, 0, eb, 0.0) if mode == 1 else O.ref_compress_blocked(mode, x, eb, bs)
                    assert so == sr, (dt, n, rel, mode, bs)
                    if mode == 2 and bs != 128:
                        continue
                    a = O.ref_decompress(mode, dt, sr, n)
                    b = O.decompress(mode, dt, so, n, ref_compat=True)
                    assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), (dt, n, rel, mode, bs)
                    checked += 1
    assert checked > 50
