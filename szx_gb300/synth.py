"""Seeded synthetic fields shaped like the SZx workloads, generated on the GPU.

No dataset ships with the reference; these stand in for it:

* ``sinusoid_field``  -- 1-D sum of 8 sinusoids (seeded frequencies 1..64
  cycles, amplitudes U(0.1,1)) + N(0,1e-3) noise, 10% of 128-value blocks
  overwritten by the block's first value.
* ``spectral_field``  -- 3-D Gaussian random field with an isotropic
  k^-5/3 power spectrum (white noise shaped in Fourier space), normalised to
  zero mean / unit variance, a fraction of z-slabs set to zero.
* ``trend_field``     -- the spectral field scaled by 1e6, plus a seeded linear
  trend, with 1% of values replaced by N(0,1e8) outliers (float64).
* ``mixed_field``     -- one of spectral / piecewise-constant / white noise.
* ``batch_fields``    -- many fields of log-uniform sizes, each spectral (1-D
  k^-5/3), piecewise-constant or white noise, with an ABS bound log-uniform
  in 1e-5..1e-2 of its range (the mixed-size batch workload).
"""
from __future__ import annotations

import math

import torch


def _gen(seed: int, device) -> torch.Generator:
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    return g


def sinusoid_field(n: int, seed: int, device="cuda", dtype=torch.float32) -> torch.Tensor:
    g = _gen(seed, device)
    i = torch.arange(n, device=device, dtype=torch.float64)
    x = torch.zeros(n, device=device, dtype=torch.float64)
    freqs = torch.randint(1, 65, (8,), generator=g, device=device)
    amps = torch.rand(8, generator=g, device=device, dtype=torch.float64) * 0.9 + 0.1
    for k in range(8):
        x += amps[k] * torch.sin(2 * math.pi * freqs[k].double() * i / n)
    x += torch.randn(n, generator=g, device=device, dtype=torch.float64) * 1e-3
    x = x.to(dtype)
    nb = n // 128
    pick = torch.rand(nb, generator=g, device=device) < 0.1
    blocks = x[: nb * 128].view(nb, 128)
    blocks[pick] = blocks[pick][:, :1].expand(-1, 128)
    return x


def spectral_field(shape, seed: int, device="cuda", dtype=torch.float32, zero_slabs: float = 0.05,
                   work_dtype=torch.float32) -> torch.Tensor:
    """Flattened 3-D field (C order, last axis fastest) with P(k) ~ k^-5/3."""
    nz, ny, nx = shape
    g = _gen(seed, device)
    noise = torch.randn((nz, ny, nx), generator=g, device=device, dtype=work_dtype)
    F = torch.fft.rfftn(noise)
    del noise
    kz = torch.fft.fftfreq(nz, device=device, dtype=work_dtype)
    ky = torch.fft.fftfreq(ny, device=device, dtype=work_dtype)
    kx = torch.fft.rfftfreq(nx, device=device, dtype=work_dtype)
    for z in range(0, nz, 64):   # in slabs: the amplitude never materialises whole
        k2 = kz[z:z + 64, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2
        if z == 0:
            k2[0, 0, 0] = 1.0
        amp = k2 ** (-5.0 / 12.0)          # sqrt(P), P ~ k^-5/3
        if z == 0:
            amp[0, 0, 0] = 0.0
        F[z:z + 64] *= amp
        del k2, amp
    f = torch.fft.irfftn(F, s=(nz, ny, nx))
    del F
    f = (f - f.mean()) / f.std()
    if zero_slabs > 0:
        ns = max(1, int(round(nz * zero_slabs)))
        slabs = torch.randperm(nz, generator=_gen(seed + 1, "cpu"))[:ns].to(device)
        f[slabs] = 0
    return f.to(dtype).reshape(-1).contiguous()


def trend_field(shape, seed: int, device="cuda") -> torch.Tensor:
    """float64: spectral field x1e6 + linear trend + 1% N(0,1e8) outliers."""
    nz, ny, nx = shape
    f = spectral_field(shape, seed, device, torch.float64, zero_slabs=0.0, work_dtype=torch.float64) * 1e6
    g = _gen(seed + 2, device)
    a, b, c = (torch.randn(3, generator=g, device=device, dtype=torch.float64) * 1e5).tolist()
    v = f.view(nz, ny, nx)
    v += a * torch.arange(nx, device=device, dtype=torch.float64)[None, None, :]
    v += b * torch.arange(ny, device=device, dtype=torch.float64)[None, :, None]
    v += c * torch.arange(nz, device=device, dtype=torch.float64)[:, None, None]
    m = f.numel() // 100
    idx = torch.randint(0, f.numel(), (m,), generator=g, device=device)
    f[idx] = torch.randn(m, generator=g, device=device, dtype=torch.float64) * 1e8
    return f


def mixed_field(n: int, seed: int, device="cuda") -> torch.Tensor:
    """float32 field of one of three kinds (spectral / piecewise-constant / noise)."""
    g = _gen(seed, device)
    kind = int(torch.randint(0, 3, (1,), generator=g, device=device).item())
    if kind == 0:
        side = max(8, int(round(n ** (1 / 3))))
        f = spectral_field((side, side, side), seed, device, zero_slabs=0.0)
        reps = (n + f.numel() - 1) // f.numel()
        return f.repeat(reps)[:n].contiguous()
    if kind == 1:
        seg = torch.randint(1, 4096, (1,), generator=g, device=device).item()
        levels = torch.randn((n + seg - 1) // seg, generator=g, device=device)
        return levels.repeat_interleave(seg)[:n].contiguous()
    return torch.randn(n, generator=g, device=device)


def batch_fields(nf: int, seed: int, lo_exp: float = 14, hi_exp: float = 26, device="cuda",
                 dtype=torch.float32):
    """nf fields with sizes log-uniform in [2^lo_exp, 2^hi_exp], each a seeded
    1-D k^-5/3 spectral field (unit variance), piecewise-constant levels (runs
    of 64..4095) or white noise, and per-field ABS bounds log-uniform in
    1e-5..1e-2 of the field's range (computed in float32).  Returns
    (fields, bounds)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(2.0 ** lo_exp), np.log(2.0 ** hi_exp), nf)).astype(np.int64)
    kinds = rng.integers(0, 3, nf)
    scales = 10.0 ** rng.uniform(-5, -2, nf)
    g = torch.Generator(device=device).manual_seed(seed)
    xs, ebs = [], []
    for n, kind, sc in zip(sizes, kinds, scales):
        n = int(n)
        if kind == 0:   # synthesised at the next power of two, then truncated
            n2 = 1 << (n - 1).bit_length()
            nh = n2 // 2 + 1
            k = torch.arange(nh, device=device, dtype=torch.float32)
            k[0] = 1.0
            amp = k ** (-5.0 / 6.0)
            amp[0] = 0.0
            z = torch.complex(torch.randn(nh, generator=g, device=device),
                              torch.randn(nh, generator=g, device=device)) * amp
            x = torch.fft.irfft(z, n=n2)[:n]
            x = (x - x.mean()) / (x.std() + 1e-30)
        elif kind == 1:
            run = int(rng.integers(64, 4096))
            x = torch.repeat_interleave(torch.randn(n // run + 1, generator=g, device=device), run)[:n].contiguous()
        else:
            x = torch.randn(n, generator=g, device=device)
        x = x.to(dtype).contiguous()
        r = float((x.max() - x.min()).item()) or 1.0
        xs.append(x)
        ebs.append(float(np.float32(r * sc)))
    return xs, ebs
