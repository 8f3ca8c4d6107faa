"""CPU oracle for the learned fixed-rate path -- test infrastructure only.

Restates, in numpy, what szx_gb300/csrc/learned.cu computes on the GPU:

* ``sums`` / ``center`` / ``probe_sums`` / ``center2`` / ``features``: the
  sampled-block sums, the two per-target probe windows and the 32-float
  feature row of a float32 field (every 10th full block of 128 values).  The byte count at a
  probe bound follows the codec's block format (szx/src/szx_float.cc:49-252:
  constant block -> 4-byte median; otherwise reqLength
  (szx/src/szx_float.cc:1708-1717), a 5-byte block header, 2-bit lead codes
  and the stored bytes left after the XOR lead of consecutive shifted words).
* ``mlp_forward`` / ``mlp_loss_grad``: the 32-64-64-64-1 GELU network in
  float64, its mean squared error and the gradient of that error by
  backpropagation, in the library's parameter layout.

Only tests import this module.
"""
from __future__ import annotations

import math

import numpy as np

F, H = 32, 64
PROBES = 16
RATE, BS = 10, 128
P_MU, P_SD, P_W1 = 0, 32, 64
P_B1 = P_W1 + H * F
P_W2 = P_B1 + H
P_B2 = P_W2 + H * H
P_W3 = P_B2 + H
P_B3 = P_W3 + H * H
P_W4 = P_B3 + H
P_B4 = P_W4 + H
P_TOTAL = P_B4 + 1
P_NTRAIN = P_TOTAL - P_W1

PROBE = np.exp2(-1.5 * np.arange(1, PROBES + 1)).astype(np.float32)
FRAC64 = np.exp2(np.arange(64) / 64.0).astype(np.float32)
QMIN, QMAX = -100, 4


def _exp_f32(v: np.ndarray) -> np.ndarray:
    """Biased exponent field minus 127 (getExponent_float)."""
    return ((v.astype(np.float32).view(np.uint32) & np.uint32(0x7F800000)) >> np.uint32(23)).astype(np.int64) - 127


def _exp_f64(v: np.ndarray) -> np.ndarray:
    """Exponent field of the double minus 1023 (getPrecisionReqLength_double)."""
    b = v.astype(np.float64).view(np.uint64)
    return ((b & np.uint64(0x7FF0000000000000)) >> np.uint64(52)).astype(np.int64) - 1023


def _lead(x: np.ndarray) -> np.ndarray:
    return np.where(x < (1 << 8), 3, np.where(x < (1 << 16), 2, np.where(x < (1 << 24), 1, 0)))


OFF2 = 5   # the second sample: full blocks 5, 15, 25, ...


def _blocks(x: np.ndarray, off: int = 0):
    """(sampled blocks [ns, 128], radius, median, sampled range) as the codec
    computes them; off 0: every 10th full block from block 0 (the range is
    always this sample's), off OFF2: the second, disjoint sample."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    full = x.size // BS
    ns = -(-full // RATE)
    blk0 = x[: full * BS].reshape(full, BS)[np.arange(ns) * RATE]
    fin = blk0[np.isfinite(blk0)]
    blk = blk0 if off == 0 else x[: full * BS].reshape(full, BS)[np.arange(off, full, RATE)]
    rng = np.float32(fin.max() - fin.min()) if fin.size else np.float32(0.0)
    mn = blk.min(axis=1)
    mx = blk.max(axis=1)
    r = ((mx - mn) * np.float32(0.5)).astype(np.float32)
    med = (mn + r).astype(np.float32)
    return blk, r, med, rng


def block_bytes(blk, r, med, eb) -> np.ndarray:
    """Stream bytes of every block at bound eb (without its state bit)."""
    eb = np.float32(eb)
    ns = blk.shape[0]
    const = r <= eb
    req = 10 + _exp_f32(r) - _exp_f64(np.full(r.shape, eb, np.float32))
    zm = req > 32
    req = np.clip(req, 9, 32)
    R = (req >> 3) + ((req & 7) != 0)
    s = np.where((req & 7) != 0, 8 - (req & 7), 0).astype(np.uint32)
    m = np.where(zm, np.float32(0), med).astype(np.float32)
    cur = (blk - m[:, None]).astype(np.float32).view(np.uint32) >> s[:, None]
    prev = np.concatenate([np.zeros((ns, 1), np.uint32), cur[:, :-1]], axis=1)
    stored = np.maximum(R[:, None] - _lead(cur ^ prev), 0).sum(axis=1)
    return np.where(const, 4, 5 + BS // 4 + stored).astype(np.int64)


def probe_bound(rng, m: int) -> np.float32:
    """range * 2^(m/64) rounded as the GPU does: range * 2^(frac/64), then exact scaling."""
    fr = m & 63
    return np.float32(np.float32(rng * FRAC64[fr]) * np.float32(2.0 ** ((m - fr) // 64)))


COARSE_STEP = 4   # the coarse curve uses every 4th sampled block


def sums(x: np.ndarray):
    """(sampled range, per-field sums[18]) as k_lfx_range / k_lfx_accumulate:
    over every 4th sampled block, their count, bytes at the 16 coarse probes,
    blocks of radius 0."""
    blk, r, med, rng = _blocks(x)
    acc = np.zeros(18, dtype=np.int64)
    if blk.shape[0] == 0:
        return np.float32(0.0), acc
    blk, r, med = blk[::COARSE_STEP], r[::COARSE_STEP], med[::COARSE_STEP]
    acc[0] = blk.shape[0]
    for j in range(PROBES):
        acc[1 + j] = int(block_bytes(blk, r, med, np.float32(rng * PROBE[j])).sum())
    acc[17] = int((r == 0).sum())
    return rng, acc


def _l2r(b, ns):
    return math.log2(4.0 * 128.0 * ns / (b + ns / 8.0))


def center(acc, target) -> int:
    """Start of the quarter-step window, 1/64 units (k_lfx_center)."""
    ns = float(acc[0])
    lt = math.log2(float(np.float32(target)))
    yc = -12.0
    if ns > 0:
        cprev = _l2r(acc[1], ns) - lt
        if cprev < 0:
            yc = -1.0
        else:
            yc = -24.0
            for j in range(1, PROBES):
                c = _l2r(acc[1 + j], ns) - lt
                if c < 0:
                    yc = -1.5 * j - 1.5 * cprev / (cprev - c)
                    break
                cprev = c
    q = min(max(int(math.floor(yc * 4.0 + 0.5)), QMIN), QMAX)
    return 16 * q - 128


def probe_sums(x: np.ndarray, mstart: int, stride: int, off: int = 0) -> np.ndarray:
    """Bytes of the sampled blocks (sample `off`) at the 16 bounds
    range * 2^((mstart + stride k)/64) (k_lfx_probe)."""
    blk, r, med, rng = _blocks(x, off)
    out = np.zeros(16, dtype=np.int64)
    if blk.shape[0] == 0:
        return out
    for k in range(16):
        out[k] = int(block_bytes(blk, r, med, probe_bound(rng, mstart + stride * k)).sum())
    return out


def sampled_blocks(x: np.ndarray, off: int = 0) -> int:
    """Every 10th full block of 128 values, from block `off`."""
    full = x.size // BS
    return -(-(full - off) // RATE) if full > off else 0


def center2(ns, fine, target, mq: int) -> int:
    """Start of the 1/64-step window (k_lfx_center2)."""
    lt = math.log2(float(np.float32(target)))
    kx = 0
    if ns > 0:
        d = [_l2r(b, ns) - lt for b in fine]
        if d[15] < 0:
            kx = 15
        else:
            for k in range(15):
                if d[k] < 0 <= d[k + 1]:
                    kx = k
                    break
    return mq + 16 * kx


def features(x: np.ndarray, target: float, mq: int | None = None, mu: int | None = None) -> np.ndarray:
    """The feature row of field x for a target ratio (k_lfx_rows); mq / mu: the
    probe windows (computed when None)."""
    rng, a = sums(x)
    ns, nc = float(sampled_blocks(x)), float(a[0])
    if mq is None:
        mq = center(a, target)
    fine = probe_sums(x, mq, 16)
    if mu is None:
        mu = center2(ns, fine, target, mq)
    ultra = probe_sums(x, mu, 1)
    out = np.zeros(F, dtype=np.float64)
    lt = math.log2(float(np.float32(target)))
    yu = mu / 64.0
    kx = (mu - mq) // 16
    u = [(_l2r(b, ns) - lt) if ns > 0 else 0.0 for b in ultra]
    u.append((_l2r(fine[kx + 1], ns) - lt) if (ns > 0 and kx + 1 < 16) else u[15])
    ys, slope = yu, 0.0
    if ns > 0:
        if u[0] >= 0:
            ys = yu
        elif u[16] < 0:
            ys = yu + 16 / 64.0
        else:
            for j in range(16):
                if u[j] < 0 <= u[j + 1]:
                    ys = yu + (j + (-u[j]) / (u[j + 1] - u[j])) / 64.0
                    slope = (u[j + 1] - u[j]) * 64.0
                    break
    # the second sample's curve at ys, linear between its 1/64 probes
    ns2 = float(sampled_blocks(x, OFF2))
    ub = 0.0
    if ns2 > 0:
        second = probe_sums(x, mu, 1, OFF2)
        pos = (ys - yu) * 64.0
        j0 = 0 if pos <= 0 else (14 if pos >= 15 else int(math.floor(pos)))
        w = 0.0 if pos <= 0 else (1.0 if pos >= 15 else pos - j0)
        b0 = _l2r(second[j0], ns2) - lt
        b1 = _l2r(second[j0 + 1], ns2) - lt
        ub = b0 + (b1 - b0) * w
    out[0] = lt
    out[1] = ys
    out[2] = min(slope, 256.0)
    out[3] = ub
    out[4] = yu
    if ns > 0:
        out[5:13] = [_l2r(fine[4 + k], ns) - lt for k in range(8)]
        out[29] = a[17] / nc
    out[13:29] = u[:16]
    out[30] = math.log2(x.size) / 26.0
    out[31] = math.log2(ns + 1.0) / 20.0
    return out


# ------------------------------------------------------------------ network

def _erf(z):
    return np.vectorize(math.erf)(z)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_d(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def unpack(p: np.ndarray):
    p = np.asarray(p, dtype=np.float64)
    return dict(mu=p[P_MU:P_MU + F], sd=p[P_SD:P_SD + F],
                W1=p[P_W1:P_B1].reshape(H, F), b1=p[P_B1:P_W2], W2=p[P_W2:P_B2].reshape(H, H), b2=p[P_B2:P_W3],
                W3=p[P_W3:P_B3].reshape(H, H), b3=p[P_B3:P_W4], W4=p[P_W4:P_B4], b4=p[P_B4])


def mlp_forward(p: np.ndarray, X: np.ndarray):
    q = unpack(p)
    a0 = (np.asarray(X, np.float64) - q["mu"]) / q["sd"]
    z1 = a0 @ q["W1"].T + q["b1"]
    a1 = gelu(z1)
    z2 = a1 @ q["W2"].T + q["b2"]
    a2 = gelu(z2)
    z3 = a2 @ q["W3"].T + q["b3"]
    a3 = gelu(z3)
    out = a3 @ q["W4"] + q["b4"]
    return out, (a0, z1, a1, z2, a2, z3, a3)


def mlp_loss_grad(p: np.ndarray, X: np.ndarray, y: np.ndarray):
    """(mean squared error, gradient over the trainable parameters W1..b4)."""
    q = unpack(p)
    out, (a0, z1, a1, z2, a2, z3, a3) = mlp_forward(p, X)
    n = len(y)
    err = out - np.asarray(y, np.float64)
    loss = float((err ** 2).mean())
    g4 = 2.0 * err / n
    gW4 = g4 @ a3
    gb4 = g4.sum()
    dz3 = np.outer(g4, q["W4"]) * gelu_d(z3)
    gW3 = dz3.T @ a2
    gb3 = dz3.sum(0)
    dz2 = (dz3 @ q["W3"]) * gelu_d(z2)
    gW2 = dz2.T @ a1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ q["W2"]) * gelu_d(z1)
    gW1 = dz1.T @ a0
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3, gW4, [gb4]])
    assert g.size == P_NTRAIN
    return loss, g
