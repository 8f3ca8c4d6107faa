"""Generate golden vectors for the cuSZx format from the reference's own cuSZx codec.

Runs ``cuSZx_fast_compress_args_unpredictable_blocked_float`` and
``cuSZx_fast_decompress_args_unpredictable_blocked_float``
(szx/src/cuszx_entry.cu:72-209) -- compiled with their CPU helpers from the
reference sources by ``make -C oracle cuszx_ref REF=<tree>`` -- on small
seeded inputs, and stores per case the input's, the stream's and the decoded
values' sha256 (cuszx_golden.json); the inputs are regenerated from their
seeds by ``cases()``.

Needs a CUDA GPU and the reference source tree (SZX_REFERENCE_SRC).  Only
cases the reference codec handles within its own buffers are run: every
non-constant block needs at most 3 stored bytes per value (reqLength <= 24),
which keeps its decoder's shared-memory reads inside the block and its host
check (a block longer than blockSize * 4 bytes ends the process) quiet; the
cases are checked against that on the CPU, with the oracle, before the
reference sees them.

Usage:  SZX_REFERENCE_SRC=<tree> python tests/golden/make_cuszx_golden.py [out.json]
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import oracle as O  # noqa: E402

FIELDS = ("walk", "steps", "noise", "runs", "smooth")
SIZES = (16384, 16384 + 37)
BLOCKS = (32, 64, 128, 224)
BOUNDS = (1e-1, 1e-3)


def make_field(name: str, n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    if name == "walk":
        return (np.cumsum(rng.normal(size=n)) * 1e-2).astype(np.float32)
    if name == "steps":      # piecewise constant: constant blocks
        return np.repeat(rng.uniform(-0.9, 0.9, size=n // 64 + 1), 64)[:n].astype(np.float32)
    if name == "noise":
        return (rng.normal(size=n) * 0.3).astype(np.float32)
    if name == "runs":       # repeated values
        return np.repeat(rng.uniform(-0.9, 0.9, size=n // 4 + 1), 4)[:n].astype(np.float32)
    if name == "smooth":
        i = np.arange(n)
        return (0.5 * np.sin(2 * np.pi * 7 * i / n) + rng.normal(size=n) * 1e-3).astype(np.float32)
    raise ValueError(name)


def cases():
    """(name, field, n, seed, bs, eb) of every golden case."""
    out = []
    for fi, f in enumerate(FIELDS):
        for n in SIZES:
            for bs in BLOCKS:
                for eb in BOUNDS:
                    seed = 1000 + 17 * fi + n % 97
                    out.append((f"{f}_n{n}_bs{bs}_eb{eb:g}", f, n, seed, bs, eb))
    return out


def sha(b) -> str:
    return hashlib.sha256(bytes(b)).hexdigest()


def _exp(v):
    return ((np.asarray(v, np.float32).view(np.uint32) >> 23) & 0xFF).astype(np.int64) - 127


def fits_reference(x: np.ndarray, bs: int, eb: float) -> bool:
    """Every non-constant full block at <= 3 stored bytes per value, and the
    oracle's decoder accepts the stream (no block longer than bs * 4 bytes)."""
    nb = x.size // bs
    blk = x[: nb * bs].reshape(nb, bs)
    r = ((blk.max(axis=1) - blk.min(axis=1)) / np.float32(2)).astype(np.float32)
    nc = r > np.float32(eb)
    if nc.any():
        req = 10 + _exp(r[nc]) - _exp(np.float32(eb))
        if req.max() > 24:
            return False
    try:
        O.cusz_decompress(O.cusz_compress(x, eb, bs), x.size)
    except ValueError:
        return False
    return True


def main(out_path=os.path.join(HERE, "cuszx_golden.json")):
    src = os.environ.get("SZX_REFERENCE_SRC")
    if not src:
        raise SystemExit("set SZX_REFERENCE_SRC to the reference source tree")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "cuszx_ref", f"REF={src}"], check=True)
    R = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libcuszxref.so"))
    R.refcusz_compress.restype = C.c_size_t
    R.refcusz_compress.argtypes = [C.c_void_p, C.c_size_t, C.c_float, C.c_int, C.c_void_p, C.c_size_t]
    R.refcusz_decompress.restype = C.c_int
    R.refcusz_decompress.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p]
    manifest = []
    for name, f, n, seed, bs, eb in cases():
        x = make_field(f, n, seed)
        if not fits_reference(x, bs, eb):
            print("skip", name)
            continue
        cap = x.nbytes + 64
        out = np.zeros(cap, np.uint8)
        sz = R.refcusz_compress(x.ctypes.data, n, eb, bs, out.ctypes.data, cap)
        if sz == 0:
            print("skip (no stream)", name)
            continue
        s = out[:sz].copy()
        y = np.zeros(n, np.float32)
        if R.refcusz_decompress(s.ctypes.data, s.size, n, y.ctypes.data) != 0:
            print("skip (no decode)", name)
            continue
        manifest.append(dict(name=name, field=f, n=n, seed=seed, bs=bs, eb=eb, x_sha256=sha(x.view(np.uint8)),
                             stream_len=int(sz), stream_sha256=sha(s), decode_sha256=sha(y.view(np.uint8))))
        print("ok", name, sz)
    with open(out_path, "w") as fh:
        json.dump({"generator": "tests/golden/make_cuszx_golden.py", "reference":
                   "szx/src/cuszx_entry.cu cuSZx_fast_(de)compress_args_unpredictable_blocked_float",
                   "cases": manifest}, fh, indent=1)
    print(len(manifest), "cases ->", out_path)


if __name__ == "__main__":
    main(*sys.argv[1:])
