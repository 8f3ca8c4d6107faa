"""Generate the golden vectors in this folder from the reference library itself.

Runs the reference SZx codec -- compiled from its own sources by
``oracle/Makefile`` (``make -C oracle ref``) -- on small seeded synthetic
inputs and stores, per case:

* the input array            (golden.npz, key ``<case>/x``)
* the reference stream       (golden.npz, key ``<case>/stream``)
* sha256 of the reference decoder's output (golden.json)

Cases whose stream would not fit the reference's own output buffer
(``sizeof(T)*n``, szx/src/szx_float.cc:1413-1416) are not run through the
reference: it would overflow its heap.  Mode-4 cases are kept only where every
block payload fits the reference OpenMP scratch slot (``4*blockSize`` bytes,
szx/src/szx_float.cc:1290), which it would otherwise overrun.

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle as O  # noqa: E402

ABS, REL = 0, 1


def smooth_1d(rng, n, dtype):
    """Sum of 8 sinusoids + N(0, 1e-3) noise + 10% constant 128-blocks."""
    i = np.arange(n)
    x = np.zeros(n)
    for _ in range(8):
        x += rng.uniform(0.1, 1.0) * np.sin(2 * np.pi * rng.integers(1, 65) * i / n)
    x += rng.normal(0, 1e-3, n)
    x = x.astype(dtype)
    nb = n // 128
    for b in np.nonzero(rng.random(nb) < 0.1)[0]:
        x[b * 128:(b + 1) * 128] = x[b * 128]
    return x


def spectral_3d(rng, side, dtype, scale=1.0, trend=False, outliers=0.0, zero_slabs=0.05):
    """Gaussian random field with a k^-5/3 spectrum on a side^3 grid."""
    k = np.fft.fftfreq(side)
    kk = np.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2)
    kk[0, 0, 0] = 1.0
    amp = kk ** (-5.0 / 6.0)
    amp[0, 0, 0] = 0.0
    noise = rng.normal(size=(side, side, side)) + 1j * rng.normal(size=(side, side, side))
    f = np.fft.ifftn(noise * amp).real
    f = (f - f.mean()) / f.std() * scale
    if trend:
        a, b, c = rng.normal(size=3) * scale * 0.1
        z, y, xg = np.meshgrid(np.arange(side), np.arange(side), np.arange(side), indexing="ij")
        f = f + a * xg + b * y + c * z
    f = f.astype(dtype)
    if zero_slabs:
        for s in rng.choice(side, size=max(1, int(side * zero_slabs)), replace=False):
            f[s] = 0
    flat = f.reshape(-1)
    if outliers:
        idx = rng.choice(flat.size, size=int(flat.size * outliers), replace=False)
        flat[idx] = rng.normal(0, 1e8, idx.size).astype(dtype)
    return flat


def noise(rng, n, dtype):
    return rng.normal(0, 1, n).astype(dtype)


def ar1(rng, n, dtype):
    return (np.cumsum(rng.normal(0, 1, n)) * 0.01).astype(dtype)


def signed_zeros(rng, n, dtype):
    """Blocks of mixed +0/-0 next to ordinary values: pins which zero the
    reference's min/max keep (the first one seen)."""
    x = rng.normal(0, 1, n).astype(dtype)
    for b in range(0, n // 128, 3):
        blk = np.where(rng.random(128) < 0.5, -0.0, 0.0).astype(dtype)
        x[b * 128:(b + 1) * 128] = blk
    return x


def offset_smooth(rng, n, dtype, offset):
    i = np.arange(n)
    return (offset + np.sin(i / 37.0) * 3 + rng.normal(0, 1e-2, n)).astype(dtype)


def cases():
    rng = np.random.default_rng(20260101)
    out = []

    def add(name, x, mode, err_mode, eb=0.0, rel=0.0, bs=128):
        out.append(dict(name=name, x=x, mode=mode, err_mode=err_mode, eb=float(np.float32(eb)),
                        rel=float(np.float32(rel)), bs=bs))

    for dt, tag in ((np.float32, "f32"), (np.float64, "f64")):
        for n in (4096, 12345):
            x = smooth_1d(rng, n, dt)
            r = float(x.max()) - float(x.min())
            add(f"{tag}_smooth_n{n}_m1_abs", x, 1, ABS, eb=1e-3 * r)
            add(f"{tag}_smooth_n{n}_m3_abs", x, 3, ABS, eb=1e-3 * r)
        x = spectral_3d(rng, 24, dt)  # 13824 elements, 5% zero slabs
        for rel in (1e-2, 1e-3, 1e-4):
            add(f"{tag}_spectral_m1_rel{rel:g}", x, 1, REL, rel=rel)
            add(f"{tag}_spectral_m3_rel{rel:g}", x, 3, REL, rel=rel)
        add(f"{tag}_spectral_m2_rel1e-3", x, 2, REL, rel=1e-3)
        add(f"{tag}_spectral_m4_rel1e-3", x, 4, REL, rel=1e-3)
        for n, ebv in ((5000, 1e-1), (5000, 1e-4)):
            add(f"{tag}_noise_n{n}_m3_eb{ebv:g}", noise(rng, n, dt), 3, ABS, eb=ebv)
            add(f"{tag}_ar1_n{n}_m1_eb{ebv:g}", ar1(rng, n, dt), 1, ABS, eb=ebv)
        add(f"{tag}_zeros_m3", signed_zeros(rng, 3000, dt), 3, ABS, eb=1e-2)
        add(f"{tag}_zeros_m1", signed_zeros(rng, 3000, dt), 1, ABS, eb=1e-2)
        add(f"{tag}_allconst_m3", np.full(2000, 1.25, dt), 3, ABS, eb=1e-3)
        add(f"{tag}_ragged_n1025_m3", smooth_1d(rng, 1025, dt), 3, ABS, eb=1e-3)
    # NaN / infinity inputs: pins the x86 NaN propagation of the reference
    for dt, tag in ((np.float32, "f32"), (np.float64, "f64")):
        base = np.sin(np.arange(3000) / 40.0).astype(dt)
        x = base.copy(); x[0] = np.nan
        add(f"{tag}_nan_first_m3", x, 3, ABS, eb=1e-2)
        add(f"{tag}_nan_first_m1", x, 1, ABS, eb=1e-2)
        x = base.copy(); x[300::257] = np.nan
        add(f"{tag}_nan_inside_m3", x, 3, ABS, eb=1e-2)
        add(f"{tag}_nan_inside_m1", x, 1, ABS, eb=1e-2)
        x = base.copy(); x[130] = np.inf; x[140] = -np.inf; x[1000] = np.inf
        add(f"{tag}_inf_m3", x, 3, ABS, eb=1e-2)
        add(f"{tag}_inf_m1", x, 1, ABS, eb=1e-2)
    # reqLength clamp at 32 (float, median forced to 0) and at 64 (double)
    add("f32_clamp32_m3", offset_smooth(rng, 4000, np.float32, 1e6), 3, ABS, eb=1e-6)
    add("f32_clamp32_m1", offset_smooth(rng, 4000, np.float32, 1e6), 1, ABS, eb=1e-6)
    add("f64_clamp64_m3", offset_smooth(rng, 4000, np.float64, 1e10), 3, ABS, eb=1e-8)
    # block sizes of the double configuration (64 and 256) through the mode-3 layout
    xd = spectral_3d(rng, 20, np.float64, scale=1e6, trend=True, outliers=0.01, zero_slabs=0.0)
    for bs in (64, 256):
        for ebv in (1e-1, 1e-3):
            add(f"f64_trend_bs{bs}_m3_eb{ebv:g}", xd, 3, ABS, eb=ebv, bs=bs)
    xf = spectral_3d(rng, 20, np.float32)
    for bs in (64, 256):
        add(f"f32_spectral_bs{bs}_m3", xf, 3, ABS, eb=1e-3, bs=bs)
    return out


def run_reference(c):
    x = c["x"]
    mode, bs = c["mode"], c["bs"]
    eb = c["eb"]
    if c["err_mode"] == REL:
        rng_ = O.value_range(x)[0]
        eb = float(np.float32(rng_ * c["rel"])) if x.dtype == np.float64 else float(
            np.float32(np.float32(rng_) * np.float32(c["rel"])))
    # size check with the oracle before touching the reference
    so = O.fast_compress_args(mode, x, c["err_mode"], c["eb"], c["rel"], bs)
    if len(so) >= x.nbytes:
        return None, "ratio below 1: reference buffer would overflow"
    if mode == 4:
        s3 = np.frombuffer(O.compress(3, x, eb, bs), np.uint8)
        nb = -(-x.size // bs)
        nnc = nb - int.from_bytes(s3[12:20].tobytes(), "big")
        if nnc and s3[20:20 + 2 * nnc].view("<u2").max() > 4 * bs:
            return None, "block payload above the reference OpenMP scratch slot"
    if bs == 128 and mode in (1, 3, 4):
        stream = O.ref_compress_args(mode, x, c["err_mode"], c["eb"], c["rel"])
    else:
        stream = O.ref_compress_blocked(mode, x, eb, bs)
    dec = O.ref_decompress(mode, x.dtype, stream, x.size)
    return (stream, dec), None


def main():
    if O.reference() is None:
        O.build(reference=True, reference_src=os.environ.get("SZX_REFERENCE_SRC"))
    assert O.reference() is not None, "reference library not built: set SZX_REFERENCE_SRC to the reference source tree"
    manifest, arrays = [], {}
    for c in cases():
        res, why = run_reference(c)
        if res is None:
            print("skip", c["name"], why)
            continue
        stream, dec = res
        x = c["x"]
        arrays[c["name"] + "/x"] = x
        arrays[c["name"] + "/stream"] = np.frombuffer(stream, np.uint8)
        manifest.append(dict(
            name=c["name"], dtype=str(x.dtype), n=int(x.size), mode=c["mode"], err_mode=c["err_mode"],
            eb=c["eb"], rel=c["rel"], bs=c["bs"], stream_len=len(stream),
            stream_sha256=hashlib.sha256(stream).hexdigest(),
            ref_decoded_sha256=hashlib.sha256(dec.tobytes()).hexdigest(),
        ))
        print("case", c["name"], x.dtype, x.size, "mode", c["mode"], "bytes", len(stream))
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(dict(generator="tests/golden/make_golden.py",
                       reference="szcompressor/SZx compiled from source by oracle/Makefile",
                       cases=manifest), f, indent=1)
    print(len(manifest), "cases written")


if __name__ == "__main__":
    main()
