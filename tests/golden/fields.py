"""Deterministic synthetic fields for the fixed-rate fixtures.

Every value comes from integer hashing and exact dyadic arithmetic (no libm
calls, no library random streams), so the same arrays come out bit for bit on
any machine and numpy version: the fixtures store only the expected results,
not the inputs.
"""
from __future__ import annotations

import numpy as np

_M = np.uint64(0xFFFFFFFF)


def _uniform(n: int, seed: int) -> np.ndarray:
    """n values in [0, 1), multiples of 2^-32, from a 64-bit integer hash."""
    i = np.arange(n, dtype=np.uint64) + np.uint64((seed * 0x9E3779B97F4A7C15) % (1 << 64))
    z = i * np.uint64(0xBF58476D1CE4E5B9)
    z ^= z >> np.uint64(31)
    z *= np.uint64(0x94D049BB133111EB)
    z ^= z >> np.uint64(29)
    return (z & _M).astype(np.float64) / 4294967296.0


def _triangle(n: int, period: int) -> np.ndarray:
    """Exact triangle wave in [-1, 1] with the given period (a power of two)."""
    p = np.arange(n, dtype=np.int64) % period
    half = period // 2
    return (np.where(p < half, p, period - p).astype(np.float64) / half) * 2.0 - 1.0


def smooth(n: int, seed: int = 1) -> np.ndarray:
    """Sum of triangle waves + small noise + runs of constant 128-blocks."""
    x = _triangle(n, 4096) + 0.5 * _triangle(n, 1024) + 0.25 * _triangle(n, 256)
    x += (_uniform(n, seed) - 0.5) * 2.0 ** -6
    flags = _uniform(n // 128, seed + 7) < 0.1
    for b in np.nonzero(flags)[0]:
        x[b * 128:(b + 1) * 128] = x[b * 128]
    return x


def steps(n: int, seed: int = 2) -> np.ndarray:
    """Piecewise-constant levels (runs of 512) + tiny noise."""
    lv = np.repeat(_uniform(-(-n // 512), seed), 512)[:n] * 8.0 - 4.0
    return lv + (_uniform(n, seed + 3) - 0.5) * 2.0 ** -14


def walk(n: int, seed: int = 3) -> np.ndarray:
    """Random walk of uniform steps (exact cumulative sum of dyadic values)."""
    return np.cumsum(_uniform(n, seed) - 0.5) * 2.0 ** -5


FIELDS = {"smooth": smooth, "steps": steps, "walk": walk}


def make(name: str, n: int, dtype) -> np.ndarray:
    x = FIELDS[name](n)
    if np.dtype(dtype) == np.float64:
        return (x * 1024.0).astype(np.float64)
    return x.astype(np.float32)
