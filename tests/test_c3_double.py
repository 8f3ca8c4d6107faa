"""Full-size double path: a 1024 x 1024 x 256 float64 field (2 GiB).

The field: a seeded k^-5/3 Gaussian random field scaled by 1e6, plus a
seeded linear trend, plus 1% outliers drawn from N(0, 1e8).  For blockSize
64 and 256 and absolute bounds 1e-1 and 1e-3, the GPU stream (fastMode 3) must
equal the oracle's block-parallel port of the reference double codec
(szx/src/szx_double.cc:1509-1590, one block: :34-433) byte for byte, and the
GPU decode must equal the oracle's faithful decode (szx/src/szxd_double.cc:
25-449 without its reqBytes==5 byte slip) bit for bit.  Points off the bound
are the reference's own float-median constant blocks (the double block's
median is stored as a float, szx/src/szx_double.cc:973-1030): both decoders
agree on them, they miss by at most half an ulp of that float, and every
non-constant block's values lie within the bound.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

SHAPE = (1024, 1024, 256)


@pytest.fixture(scope="module")
def field():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a CUDA device is required")
    from szx_gb300 import build
    build.build()
    g = torch.Generator(device="cuda").manual_seed(3003)
    nx, ny, nz = SHAPE
    kx = torch.fft.fftfreq(nx, device="cuda", dtype=torch.float64).view(nx, 1, 1)
    ky = torch.fft.fftfreq(ny, device="cuda", dtype=torch.float64).view(1, ny, 1)
    kz = torch.fft.rfftfreq(nz, device="cuda", dtype=torch.float64).view(1, 1, nz // 2 + 1)
    k = torch.sqrt(kx * kx + ky * ky + kz * kz)
    k[0, 0, 0] = 1.0
    amp = k.pow_(-5.0 / 6.0)
    amp[0, 0, 0] = 0.0
    spec = torch.complex(torch.randn(amp.shape, generator=g, device="cuda", dtype=torch.float64),
                         torch.randn(amp.shape, generator=g, device="cuda", dtype=torch.float64))
    spec.mul_(amp)
    del amp, k
    x = torch.fft.irfftn(spec, s=SHAPE)
    del spec
    x.sub_(x.mean()).div_(x.std()).mul_(1e6)
    a, b, c = (torch.rand(3, generator=g, device="cuda", dtype=torch.float64) * 2 - 1).tolist()
    x.add_(a * 100.0 * torch.arange(nx, device="cuda", dtype=torch.float64).view(nx, 1, 1))
    x.add_(b * 100.0 * torch.arange(ny, device="cuda", dtype=torch.float64).view(1, ny, 1))
    x.add_(c * 100.0 * torch.arange(nz, device="cuda", dtype=torch.float64).view(1, 1, nz))
    flat = x.view(-1)
    m = flat.numel() // 100
    idx = torch.randint(0, flat.numel(), (m,), generator=g, device="cuda")
    flat[idx] = torch.randn(m, generator=g, device="cuda", dtype=torch.float64) * 1e8
    torch.cuda.synchronize()
    return flat, flat.cpu().numpy()


@pytest.mark.parametrize("bs,eb", [(64, 1e-1), (64, 1e-3), (256, 1e-1), (256, 1e-3)])
def test_full_size_double_streams_and_values(field, bs, eb):
    import torch
    from szx_gb300.api import DeviceCodec
    xd, xh = field
    n = xh.size
    codec = DeviceCodec(3, np.float64, n, blockSize=bs)
    codec.compress(xd, 0, eb, 0.0)
    s = codec.stream_bytes()
    got = s.cpu().numpy()
    want, wlen = O.compress_m3_omp(xh, eb, bs)
    assert got.size == wlen
    assert np.array_equal(got, want[:wlen]), (bs, eb)
    y = codec.decompress(s, n)
    torch.cuda.synchronize()
    assert codec.status() == 0
    yh = y.cpu().numpy()
    ref = O.decompress_m3_omp(np.float64, want, wlen, n)
    assert np.array_equal(yh.view(np.uint64), ref.view(np.uint64)), (bs, eb)
    # off-bound points only in constant blocks, by at most the rounding of their float median
    off = np.nonzero(np.abs(yh - xh) > eb)[0]
    if off.size:
        blk = off // bs
        _, state, med, _ = O.block_stats(xh, eb, bs)
        assert not state[blk].any(), "a non-constant block is off the bound"
        slack = 0.5 * np.spacing(np.abs(med[blk])).astype(np.float64)
        assert (np.abs(yh[off] - xh[off]) <= eb * (1 + 1e-12) + slack).all()
    del codec


@pytest.mark.parametrize("eb", [1e-1, 1e-3])
def test_full_size_double_fastmode1(field, eb):
    """The same 2 GiB field through fastMode 1 (the non-blocked layout,
    szx/src/szx_double.cc:1593-2011, decoded by szx/src/szxd_double.cc:
    683-1114): 65,536 tiles of 4096 values, so every persistent CTA of the
    encoder and of the decoder works through many tiles (claim-ahead,
    window placement, both staging buffers, the two-ahead prefetch).  Stream
    and values must equal the serial oracle's."""
    import torch
    from szx_gb300.api import DeviceCodec
    xd, xh = field
    n = xh.size
    codec = DeviceCodec(1, np.float64, n, blockSize=128)
    codec.compress(xd, 0, eb, 0.0)
    s = codec.stream_bytes()
    got = s.cpu().numpy().tobytes()
    want = O.fast_compress_args(1, xh, 0, eb, 0.0, 128)
    assert len(got) == len(want) and got == want, eb
    y = codec.decompress(s, n)
    torch.cuda.synchronize()
    assert codec.status() == 0
    ref = O.decompress(1, np.float64, want, n)
    assert np.array_equal(y.cpu().numpy().view(np.uint64), ref.view(np.uint64)), eb
    del codec
