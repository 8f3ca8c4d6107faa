"""Autotuner for the launch shapes of batched fields, per field-size class.

For every size class it draws synthetic float32 fields of that class (the
mixed-field generator: spectral / piecewise-constant / white noise, per-field
ABS bound log-uniform in 1e-5..1e-2 of the range, fastMode 3, blockSize 128),
times a batched compress and a batched decompress (one persistent launch per
kernel, replayed from a CUDA graph) under every candidate shape, and keeps
the fastest encoder shape (tile size and threads per CTA -- the two go
together --, CTAs per SM) and the fastest decoder shape (CTAs per SM).  The
table goes to ``tuning/batch_shapes.txt`` beside the library, where
``SZxG_batch_create`` reads it.  Shapes never change a stream (the tests
check every candidate), only how the work is cut and spread.

    python -m szx_gb300.tune [--out PATH] [--quick]
"""
from __future__ import annotations

import argparse
import ctypes as C
import datetime
import os
import statistics

import numpy as np

from ._lib import StreamInfo, lib

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_OUT = os.path.join(HERE, "tuning", "batch_shapes.txt")

# (upper bound of the class in values, field sizes drawn log-uniform in [lo, hi], fields)
CLASSES = [
    (1 << 18, (1 << 14, 1 << 18), 1500),
    (1 << 22, (1 << 18, 1 << 22), 200),
    ((1 << 64) - 1, (1 << 22, 1 << 26), 24),
]
# encoder (tile variant, CTAs per SM; 0 = as many as fit), decoder CTAs per SM
ENC_CANDIDATES = [(0, 0), (0, 2), (1, 0), (1, 4), (1, 3)]
DEC_CANDIDATES = [0, 3, 2]


class LaunchShape(C.Structure):
    """SZxG_LaunchShape."""
    _fields_ = [("maxValues", C.c_ulonglong), ("encTileVariant", C.c_int), ("encCtasPerSm", C.c_int),
                ("decCtasPerSm", C.c_int), ("reserved", C.c_int)]


class Field(C.Structure):
    """SZxG_Field."""
    _fields_ = [("in_", C.c_void_p), ("nbEle", C.c_size_t), ("inBytes", C.c_size_t), ("absErrBound", C.c_float),
                ("reserved", C.c_int), ("out", C.c_void_p), ("outCapacity", C.c_size_t)]


def _declare(L):
    L.SZxG_set_launch_shapes.restype = C.c_int
    L.SZxG_set_launch_shapes.argtypes = [C.c_void_p, C.c_int]
    L.SZxG_get_launch_shapes.restype = C.c_int
    L.SZxG_get_launch_shapes.argtypes = [C.c_void_p, C.c_int]
    L.SZxG_batch_create.restype = C.c_void_p
    L.SZxG_batch_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    L.SZxG_batch_run.restype = C.c_int
    L.SZxG_batch_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.SZxG_batch_status.restype = C.c_int
    L.SZxG_batch_status.argtypes = [C.c_void_p, C.c_void_p]
    L.SZxG_batch_destroy.restype = None
    L.SZxG_batch_destroy.argtypes = [C.c_void_p]
    return L


def set_shapes(entries):
    """entries: [(maxValues, encTileVariant, encCtasPerSm, decCtasPerSm)]; [] reloads the tuning file."""
    L = _declare(lib())
    tab = (LaunchShape * max(1, len(entries)))()
    for k, (m, tv, ec, dc) in enumerate(entries):
        tab[k] = LaunchShape(m, tv, ec, dc, 0)
    rc = L.SZxG_set_launch_shapes(C.cast(tab, C.c_void_p) if entries else None, len(entries))
    if rc:
        raise RuntimeError(f"SZxG_set_launch_shapes: {rc}")


def get_shapes():
    L = _declare(lib())
    tab = (LaunchShape * 8)()
    n = L.SZxG_get_launch_shapes(C.cast(tab, C.c_void_p), 8)
    return [(t.maxValues, t.encTileVariant, t.encCtasPerSm, t.decCtasPerSm) for t in tab[:n]]


def time_batch(xs, ebs, outs, mode=3, bs=128, reps=5):
    """(compress ms, decompress ms) of one batch of device fields, each the
    median of `reps` CUDA-graph replays; outs: per-field stream buffers."""
    import torch
    L = _declare(lib())
    nf = len(xs)
    s = torch.cuda.Stream()
    res = []
    fields = (Field * nf)()
    for k, (x, eb, o) in enumerate(zip(xs, ebs, outs)):
        fields[k] = Field(x.data_ptr(), x.numel(), 0, eb, 0, o.data_ptr(), o.numel())
    info = torch.zeros(nf * C.sizeof(StreamInfo), dtype=torch.uint8, device="cuda")
    ys = [torch.empty_like(x) for x in xs]
    for direction in (0, 1):
        if direction == 1:
            raw = info.cpu().numpy().tobytes()
            sz = C.sizeof(StreamInfo)
            infos = [StreamInfo.from_buffer_copy(raw[k * sz:(k + 1) * sz]) for k in range(nf)]
            for k in range(nf):
                fields[k] = Field(outs[k].data_ptr() + infos[k].offset, xs[k].numel(), infos[k].size, 0.0, 0,
                                  ys[k].data_ptr(), ys[k].numel() * 4)
        b = L.SZxG_batch_create(direction, mode, 0, bs, nf, C.cast(fields, C.c_void_p))
        if not b:
            raise RuntimeError(f"SZxG_batch_create failed: {L.SZxG_get_last_error()}")
        try:
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                for _ in range(2):
                    assert L.SZxG_batch_run(b, C.c_void_p(info.data_ptr() if direction == 0 else 0),
                                            C.c_void_p(s.cuda_stream)) == 0
            torch.cuda.current_stream().wait_stream(s)
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                assert L.SZxG_batch_run(b, C.c_void_p(info.data_ptr() if direction == 0 else 0),
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
            ts = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                g.replay()
                e1.record()
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            st = L.SZxG_batch_status(b, C.c_void_p(torch.cuda.current_stream().cuda_stream))
            if st:
                raise RuntimeError(f"batch status {st}")
            res.append(statistics.median(ts))
        finally:
            L.SZxG_batch_destroy(b)
    return res[0], res[1]


def tune(out=DEFAULT_OUT, quick=False, seed=777):
    import torch

    from . import synth
    from ._lib import lib as _l
    L = _declare(_l())
    rows, table = [], []
    for ci, (cmax, (lo, hi), nf) in enumerate(CLASSES):
        if quick:
            nf = max(4, nf // 8)
        xs, ebs = synth.batch_fields(nf, seed + ci, np.log2(lo), np.log2(hi), "cuda")
        outs = [torch.empty(L.SZxG_compress_bound(3, 0, x.numel(), 128), dtype=torch.uint8, device="cuda")
                for x in xs]
        nbytes = sum(x.numel() for x in xs) * 4
        enc_t, dec_t = {}, {}
        for tv, ec in ENC_CANDIDATES:
            set_shapes([((1 << 64) - 1, tv, ec, 0)])   # one class: every field takes the candidate
            enc_t[(tv, ec)], _ = time_batch(xs, ebs, outs)
        best_e = min(enc_t, key=enc_t.get)
        for dc in DEC_CANDIDATES:
            set_shapes([((1 << 64) - 1, best_e[0], best_e[1], dc)])
            _, dec_t[dc] = time_batch(xs, ebs, outs)
        best_d = min(dec_t, key=dec_t.get)
        table.append((cmax, best_e[0], best_e[1], best_d))
        rows.append((ci, lo, hi, nf, nbytes, enc_t, dec_t, best_e, best_d))
        del xs, outs
        torch.cuda.empty_cache()
    set_shapes([])
    os.makedirs(os.path.dirname(out), exist_ok=True)
    with open(out, "w") as f:
        f.write("# Launch shapes of batched fields by size class, written by szx_gb300/tune.py\n")
        f.write(f"# {datetime.datetime.now(datetime.timezone.utc):%Y-%m-%d} on {torch.cuda.get_device_name(0)}; float32, fastMode 3, "
                "blockSize 128; batched compress / decompress GB/s per candidate\n")
        for ci, lo, hi, nf, nbytes, enc_t, dec_t, be, bd in rows:
            f.write(f"# class {ci}: {nf} fields of {lo}..{hi} values ({nbytes / 1e9:.2f} GB)\n")
            f.write("#   encoder (tile variant, CTAs/SM): " +
                    ", ".join(f"{k}={nbytes / (v / 1e3) / 1e9:.0f}" for k, v in enc_t.items()) + "\n")
            f.write("#   decoder CTAs/SM: " + ", ".join(f"{k}={nbytes / (v / 1e3) / 1e9:.0f}" for k, v in dec_t.items())
                    + "\n")
        f.write("# max_values enc_tile_variant enc_ctas_per_sm dec_ctas_per_sm\n")
        for cmax, tv, ec, dc in table:
            f.write(f"{cmax} {tv} {ec} {dc}\n")
    return table, rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--quick", action="store_true", help="fewer fields per class")
    args = ap.parse_args()
    table, _ = tune(args.out, args.quick)
    print(open(args.out).read())


if __name__ == "__main__":
    main()
