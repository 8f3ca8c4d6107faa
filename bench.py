#!/usr/bin/env python3
"""Benchmark: SZx blocked codec on GB300, compress + decompress GB/s.

Workload (default ``c2``): 512^3 float32 Gaussian random field with a k^-5/3
spectrum (seeded FFT synthesis, unit variance) plus 5% zero-valued z-slabs,
REL bound 1e-3, fastMode 3 (random-access layout), blockSize 128.

A step is one compress and one decompress of the whole field.
  value      = 2 * field bytes / (compress time + decompress time)   [GB/s]
               device-resident input/output, SZxG_compress / SZxG_decompress,
               CUDA events on the launching stream
  e2e        = the same metric through the reference-facing C entry points
               SZx_fast_compress_args / SZx_fast_decompress with host buffers
               (pageable numpy input, as a drop-in caller passes it; malloc'd
               outputs as the reference API returns them), host<->device
               copies inside the timed region (wall clock: the calls are
               synchronous)
  roofline   = the dominant kernel's algorithmic bytes per launch / its mean
               launch time (CUDA events the library records around each launch)
               against the measured HBM copy bandwidth; roofline_decode the
               same for the decoder
  stream_equal / decode_equal = after the timed region, the benchmarked
               stream and decoded field compared byte for byte with the
               oracle's
  cpu_baseline / --impl reference = the oracle's block-parallel (OpenMP) port of
               the reference codec on the host cores

The same run adds the rest of the headline metric as extra keys (``--extras``,
on by default at N=1): ``mode1`` (the same field through fastMode 1),
``batched`` (mixed-size fields in one persistent launch replayed from a CUDA
graph, against per-field launches) and ``fixed_rate`` (learned fixed-rate
fields/s against plain bisection).  ``--workload c4`` / ``c5`` print those
alone as their own line.

Multi-GPU: replicas only (one independent field per rank), value summed.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

REL = 1
WORKLOADS = {
    "c2": dict(shape=(512, 512, 512), mode=3, bs=128, rel=1e-3,
               desc="512^3 float32 k^-5/3 Gaussian random field + 5% zero slabs, REL 1e-3, fastMode 3, blockSize 128"),
    "c2s": dict(shape=(384, 384, 384), mode=3, bs=128, rel=1e-3,
                desc="384^3 float32 k^-5/3 Gaussian random field + 5% zero slabs, REL 1e-3, fastMode 3, blockSize 128 "
                     "(profiling size: 216 MiB, above L2)"),
    "c2m1": dict(shape=(512, 512, 512), mode=1, bs=128, rel=1e-3,
                 desc="512^3 float32 k^-5/3 Gaussian random field + 5% zero slabs, REL 1e-3, fastMode 1"),
    "c2sm1": dict(shape=(384, 384, 384), mode=1, bs=128, rel=1e-3,
                  desc="384^3 float32 k^-5/3 Gaussian random field + 5% zero slabs, REL 1e-3, fastMode 1 "
                       "(profiling size: 216 MiB, above L2)"),
    "c5": dict(mode=2, bs=128,
               desc="learned fixed rate: 500 float32 fields, sizes log-uniform 2^20..2^26, seeded mix of spectral / "
                    "piecewise-constant (+1e-3 noise) / white noise, targets 8, 16, 32 within 5%, fastMode-2 "
                    "streams, blockSize 128; network trained on the GPU from 20 real compress passes of 1000 "
                    "other fields of the same distribution"),
    "c4": dict(mode=3, bs=128,
               desc="batched: float32 fields, sizes log-uniform 2^14..2^26, seeded mix of spectral / "
                    "piecewise-constant / white noise, per-field ABS bound log-uniform 1e-5..1e-2 x range, "
                    "fastMode 3, blockSize 128"),
}


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def read_traffic(kernel: str):
    """(DRAM bytes per value, where that figure was measured) from the
    committed ncu summary, or (None, None)."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(p):
        return None, None
    with open(p) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 3 and parts[0] == kernel and parts[1] == "bytes_per_element":
                return float(parts[2]), " ".join(parts[3:]) or None
    return None, None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.rows = []
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 3 + k and r[3 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


FIELD_SEED = 1234


def common_config(wl, n, world):
    """The `config` both arms print (same workload, size, seed and L2 note)."""
    return {"workload": wl["desc"], "elements": int(n), "seed": FIELD_SEED,
            "l2": f"inputs ({n * 4 >> 20} MiB) larger than L2; no flush needed",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


def make_field(wl, seed, device):
    import torch

    from szx_gb300 import synth
    return synth.spectral_field(wl["shape"], seed=seed, device=device, dtype=torch.float32)


def cpu_codec_gbs(x_np, eb, bs, reps, threads):
    """The oracle's OpenMP port of the reference mode-3 codec: GB/s of
    2*bytes/(t_compress + t_decompress), best of `reps`."""
    import numpy as np

    import oracle as O
    if not os.path.exists(O.ORACLE_SO):
        O.build(reference=False)
    buf = np.empty(O.capacity(3, 0, x_np.size, bs), np.uint8)
    out = np.empty_like(x_np)
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        _, n = O.compress_m3_omp(x_np, eb, bs, threads=threads, out=buf)
        t1 = time.perf_counter()
        O.decompress_m3_omp(np.float32, buf, n, x_np.size, threads=threads, out=out)
        t2 = time.perf_counter()
        t = t2 - t0
        best = t if best is None or t < best else best
    return 2 * x_np.nbytes / best / 1e9, best


def run_reference(args, wl, rank, world):
    import numpy as np
    import torch
    if rank != 0:
        return
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    x = make_field(wl, FIELD_SEED, dev).cpu().numpy()
    import oracle as O
    r = O.value_range(x)[0]
    eb = float(np.float32(np.float32(r) * np.float32(wl["rel"])))
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_codec_gbs(x, eb, wl["bs"], 1, threads)
    times = []
    for _ in range(args.steps):
        _, t = cpu_codec_gbs(x, eb, wl["bs"], 1, threads)
        times.append(t)
    ms = 1000 * sum(times) / len(times)
    val = 2 * x.nbytes / (sum(times) / len(times)) / 1e9
    sample = f"whole field ({x.size} float32 values, {x.nbytes >> 20} MiB), compress+decompress per step"
    line = {
        "metric": "compress/decompress GB/s (fp32 REL 1e-3)", "value": round(val, 3), "unit": "GB/s",
        "impl": "reference", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded on-device FFT synthesis; no dataset ships with the reference)",
        "config": common_config(wl, x.size, world),
        "cpu_baseline": {"value": round(val, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(val, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def reduce_over_ranks(maxes, sums, device):
    """The replicas' only cross-rank step (timing, never data): each value of
    `maxes` becomes its maximum over the ranks (a job ends with its slowest
    rank) and each value of `sums` its sum.  Needs an initialised
    torch.distributed process group (NCCL on GPUs; gloo in the CPU tests)."""
    import torch
    import torch.distributed as D
    m = torch.tensor([float(v) for v in maxes], dtype=torch.float64, device=device)
    s = torch.tensor([float(v) for v in sums], dtype=torch.float64, device=device)
    if m.numel():
        D.all_reduce(m, op=D.ReduceOp.MAX)
    if s.numel():
        D.all_reduce(s, op=D.ReduceOp.SUM)
    return m.tolist(), s.tolist()


def timed_steps(L, codec, x, y, sv, n, rel, steps, ev_stream_sync=True):
    """`steps` compress+decompress steps of `codec` on field x (REL rel),
    bracketed by CUDA events on the current stream, with the library's launch
    trace on.  Returns (total ms, compress ms, decompress ms, {kernel: (ms, launches)})."""
    import torch
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3 * steps)]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    L.SZxG_trace_enable(1)
    torch.cuda.synchronize()
    t_start.record()
    for k in range(steps):
        ev[3 * k].record()
        codec.compress(x, REL, 0.0, rel)
        ev[3 * k + 1].record()
        codec.decompress(sv, n, out=y)
        ev[3 * k + 2].record()
    t_end.record()
    torch.cuda.synchronize()
    names = C.create_string_buffer(4096)
    tms = (C.c_double * 32)()
    cnt = (C.c_ulonglong * 32)()
    nk = L.SZxG_trace_collect(names, 4096, tms, cnt, 32)
    L.SZxG_trace_enable(0)
    kern = {nm: (tms[i], int(cnt[i])) for i, nm in enumerate(names.value.decode().split("\n")[:nk])}
    tc = sum(ev[3 * k].elapsed_time(ev[3 * k + 1]) for k in range(steps))
    td = sum(ev[3 * k + 1].elapsed_time(ev[3 * k + 2]) for k in range(steps))
    return t_start.elapsed_time(t_end), tc, td, kern


def traffic_of(kernel: str, n: int):
    """DRAM bytes per launch of `kernel` on n values from the committed ncu
    summary (scaled by the value count), or None."""
    tb, _ = read_traffic(kernel)
    return round(tb * n) if tb else None


def kernel_roofline(kern, name, alg_bytes, peak, peak_kind, traffic=None):
    """Roofline entry of one kernel: algorithmic bytes per launch / mean launch time."""
    ms, cnt = kern[name]
    achieved = alg_bytes / (ms / cnt / 1000) / 1e9
    return {"kernel": name, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_kind": peak_kind, "traffic": traffic,
            "algorithmic_bytes": int(alg_bytes), "ms_per_launch": round(ms / cnt, 5)}


def prepare(codec, x, rel):
    """One compress to learn where the stream lands (the same every step)."""
    import szx_gb300 as S
    codec.compress(x, REL, 0.0, rel)
    info = codec.stream_info()
    if info.status:
        raise S.SZxError(info.status, "compress")
    off, size = int(info.offset), int(info.size)
    return info, off, size, codec.out[off:off + size]


def run_mode1(args, L, x, rel, peak, peak_kind):
    """The same field through the non-blocked layout (fastMode 1): GB/s,
    kernel rooflines and stream equality with the oracle's serial mode 1."""
    import numpy as np
    import torch

    import szx_gb300 as S
    n = x.numel()
    in_bytes = n * 4
    codec = S.DeviceCodec(1, np.float32, n, 128)
    y = torch.empty_like(x)
    info, off, size, sv = prepare(codec, x, rel)
    for _ in range(args.warmup):
        codec.compress(x, REL, 0.0, rel)
        codec.decompress(sv, n, out=y)
    steps = max(3, args.steps // 2)
    total, tc, td, kern = timed_steps(L, codec, x, y, sv, n, rel, steps)
    got = sv.cpu().numpy().tobytes()
    dec = y.cpu().numpy()
    del codec, y
    torch.cuda.empty_cache()
    import oracle as O
    xh = x.cpu().numpy()
    want = O.fast_compress_args(1, xh, 1, 0.0, rel, 128)
    equal = got == want
    dec_equal = bool(equal and np.array_equal(dec.view(np.uint32),
                                              O.decompress(1, np.float32, want, n).view(np.uint32)))
    enc, decn = kern["nonblocked_encode"], kern["nonblocked_decode"]
    return {
        "workload": "the same 512^3 float32 field, REL 1e-3, fastMode 1 (non-blocked layout)",
        "steps": steps, "value": round(2 * in_bytes * steps / ((tc + td) / 1000) / 1e9, 2), "unit": "GB/s",
        "compress_gbs": round(in_bytes * steps / (tc / 1000) / 1e9, 2),
        "decompress_gbs": round(in_bytes * steps / (td / 1000) / 1e9, 2),
        "stream_bytes": size, "ratio": round(in_bytes / size, 4),
        "kernels_ms_per_step": {k: round(v[0] / steps, 4) for k, v in kern.items()},
        "roofline_encode": kernel_roofline(kern, "nonblocked_encode", in_bytes + size, peak, peak_kind,
                                           traffic_of("nonblocked_encode", n)),
        "roofline_decode": kernel_roofline(kern, "nonblocked_decode", in_bytes + size, peak, peak_kind,
                                           traffic_of("nonblocked_decode", n)),
        "stream_equal": equal, "decode_equal": dec_equal,
        "gpu_launches": sum(c for _, c in kern.values()),
    }


def run_ours(args, wl, rank, world, local_rank):
    import numpy as np
    import torch

    import szx_gb300 as S
    from szx_gb300._lib import lib, libc

    dist = world > 1
    if dist:
        import torch.distributed as D
    torch.cuda.set_device(local_rank)
    L = lib()
    x = make_field(wl, FIELD_SEED + rank, "cuda")
    n = x.numel()
    in_bytes = n * 4
    mode, bs, rel = wl["mode"], wl["bs"], wl["rel"]
    codec = S.DeviceCodec(mode, np.float32, n, bs)
    y = torch.empty_like(x)
    info, off, size, sv = prepare(codec, x, rel)

    for _ in range(args.warmup):
        codec.compress(x, REL, 0.0, rel)
        codec.decompress(sv, n, out=y)
    torch.cuda.synchronize()
    if dist:
        D.barrier()
    clocks = ClockSampler(local_rank) if rank == 0 else None
    time.sleep(0.3)
    total_ms, tc, td, kern = timed_steps(L, codec, x, y, sv, n, rel, args.steps)
    clk = clocks.stop() if clocks else None
    launches = sum(c for _, c in kern.values())
    info2 = codec.stream_info()
    assert (int(info2.offset), int(info2.size), info2.status) == (off, size, 0)

    # the decoded field honours the bound (size-independent property)
    eb = float(info.eb)
    err = (x.double() - y.double()).abs()
    ulp = torch.nextafter(x.abs(), torch.full_like(x, float("inf"))) - x.abs()
    bound_ok = bool((err <= eb + 2 * ulp.double()).all().item())
    del err, ulp

    if dist:
        (total_ms, tc, td), (launches,) = reduce_over_ranks([total_ms, tc, td], [launches], "cuda")
        launches = int(launches)

    # ---- e2e through the reference-facing entry points, pageable host buffers
    # ordinary (pageable) host memory written by the CPU, as a drop-in
    # caller's array is: allocated by numpy, filled by a CPU copy
    xh = np.empty(n, np.float32)
    np.copyto(xh, x.cpu().numpy())
    free = libc().free
    sz = C.c_size_t()

    def e2e_step():
        p = L.SZx_fast_compress_args(mode, 0, C.c_void_p(xh.ctypes.data), C.byref(sz), REL, 0.0, rel, 0.0, 0.0,
                                     0, 0, 0, 0, n)
        if not p:
            raise S.SZxError(S.api.last_error(), "SZx_fast_compress_args")
        q = L.SZx_fast_decompress(mode, 0, C.c_void_p(p), sz.value, 0, 0, 0, 0, n)
        if not q:
            raise S.SZxError(S.api.last_error(), "SZx_fast_decompress")
        free(p)
        free(q)
        return sz.value

    for _ in range(args.warmup):
        e2e_step()
    if dist:
        D.barrier()
    e2e_steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    if dist:
        (e2e_s,), _ = reduce_over_ranks([e2e_s], [], "cuda")

    if rank != 0:
        return
    K = args.steps
    value = world * 2 * in_bytes * K / ((tc + td) / 1000) / 1e9
    peak, peak_kind = read_peaks()
    enc = "blocked_encode" if mode != 1 else "nonblocked_encode"
    dec = "blocked_decode" if mode != 1 else "nonblocked_decode"
    dom = max((enc, dec), key=lambda k: kern.get(k, (0, 0))[0])
    alg = in_bytes + size          # encode: read field, write stream; decode: read stream, write field
    tb, tb_note = read_traffic(dom)
    roofline = kernel_roofline(kern, dom, alg, peak, peak_kind, round(tb * n) if tb else None)
    if tb:
        roofline["traffic_source"] = tb_note
    other = dec if dom == enc else enc
    to, to_note = read_traffic(other)
    roofline_other = kernel_roofline(kern, other, alg, peak, peak_kind, round(to * n) if to else None)
    if to:
        roofline_other["traffic_source"] = to_note

    # parity of what was timed: the stream and the decoded field against the
    # oracle's block-parallel port of the reference codec (outside the timing)
    import oracle as O
    got = sv.cpu().numpy()
    threads = os.cpu_count() or 1
    if mode == 3:
        want, wlen = O.compress_m3_omp(xh, np.float32(eb), bs, threads=threads)
    else:   # the serial oracle for the other layouts
        want = np.frombuffer(O.fast_compress_args(mode, xh, REL, 0.0, rel, bs), np.uint8)
        wlen = want.size
    stream_equal = bool(wlen == size and np.array_equal(got, want[:wlen]))
    decode_equal = bool(stream_equal and np.array_equal(
        y.cpu().numpy().view(np.uint32),
        (O.decompress_m3_omp(np.float32, want, wlen, n, threads=threads) if mode == 3
         else O.decompress(mode, np.float32, want.tobytes(), n)).view(np.uint32)))
    del want, got
    del codec, y
    torch.cuda.empty_cache()

    # CPU baseline: the same field on the host cores
    cpu_val, _ = cpu_codec_gbs(xh, eb, bs, 2, threads)
    line = {
        "metric": "compress/decompress GB/s (fp32 REL 1e-3)",
        "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": round(total_ms / K, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded on-device FFT synthesis; no dataset ships with the reference)",
        "config": common_config(wl, n, world),
        "stream_bytes": size, "ratio": round(in_bytes / size, 4), "bound": eb,
        "compress_gbs": round(world * in_bytes * K / (tc / 1000) / 1e9, 2),
        # the REL range pass hoisted out, as the reference CLI converts REL to ABS first
        "compress_codec_only_gbs": round(world * in_bytes * K / ((tc - kern.get("range", (0.0, 0))[0]) / 1000) / 1e9,
                                         2),
        "decompress_gbs": round(world * in_bytes * K / (td / 1000) / 1e9, 2),
        "kernels_ms_per_step": {k: round(v[0] / K, 4) for k, v in kern.items()},
        "gpu_launches": launches,
        "bound_ok": bound_ok,
        "stream_equal": stream_equal,
        "decode_equal": decode_equal,
        "clocks": clk,
        "e2e": {"value": round(world * 2 * in_bytes / e2e_s / 1e9, 3), "unit": "GB/s",
                "h2d_bytes_per_step": in_bytes + size, "d2h_bytes_per_step": size + in_bytes,
                "api": "SZx_fast_compress_args + SZx_fast_decompress (pageable host input)"},
        "roofline": roofline,
        "roofline_" + ("decode" if other == dec else "encode"): roofline_other,
        "cpu_baseline": {"value": round(cpu_val, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"the same field ({n} float32 values), compress+decompress, best of 2"},
    }
    if args.extras and world == 1 and mode == 3:
        line["mode1"] = run_mode1(args, L, x, rel, peak, peak_kind)
        del x
        torch.cuda.empty_cache()
        line["batched"] = run_batched(args, WORKLOADS["c4"], fields=args.extra_fields)
        torch.cuda.empty_cache()
        line["fixed_rate"] = run_fixed_rate(args, WORKLOADS["c5"])
    print(json.dumps(line), flush=True)


def make_batch_fields(nf, seed, device):
    """C4 fields on the device: sizes log-uniform 2^14..2^26, each a seeded
    1-D spectral field (k^-5/3), piecewise-constant levels or white noise,
    with an ABS bound log-uniform in 1e-5..1e-2 of its range."""
    from szx_gb300 import synth
    return synth.batch_fields(nf, seed, 14, 26, device)


def run_fixed_rate(args, wl):
    """C5: fixed-rate selection for 500 fields x 3 targets -- the learned path
    (sampled model + network, judged by real compress passes) against plain
    bisection over real compress passes, on the same GPU and plan."""
    import numpy as np
    import torch

    from szx_gb300 import learned as LR
    t0 = time.perf_counter()
    tf, _ = LR.synthetic_fields(1000, 20, 26, seed=101)
    tb = LR.Batch(tf)
    X, y, _ = LR.training_set(tb, passes=20, seed=102)
    tb.close()
    del tf, tb
    torch.cuda.empty_cache()
    t1 = time.perf_counter()
    model, loss = LR.train(X, y, seed=103, epochs=100, batch=512)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    rows, var = int(X.shape[0]), float(y.var())
    del X, y
    zero = LR.Mlp(0, params=np.concatenate([np.zeros(32), np.ones(32),
                                            np.zeros(model.count - 64)]).astype(np.float32))
    fields, _ = LR.synthetic_fields(500, 20, 26, seed=202)
    b = LR.Batch(fields)
    nbytes = float(b.n.sum() * 4)
    b.fixed_rate(8.0, model, 0.05, 20)   # warm-up
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    time.sleep(0.3)
    per = {}
    tot = {"bisection": 0.0, "learned": 0.0, "zero_network": 0.0}
    jobs = 0
    methods = (("bisection", None), ("zero_network", zero), ("learned", model))
    reps = 3   # each method timed 3 times per target in rotated order; the median time counts
    for target in (8.0, 16.0, 32.0):
        per[target] = {}
        times = {name: [] for name, _ in methods}
        for r in range(reps):
            for name, m in methods[r % 3:] + methods[:r % 3]:
                torch.cuda.synchronize()
                ts = time.perf_counter()
                eb, cr, ps = b.fixed_rate(target, m, 0.05, 20)
                torch.cuda.synchronize()
                times[name].append(time.perf_counter() - ts)
                if r == 0:
                    ok = np.abs(cr / target - 1) <= 0.05
                    per[target][name] = {"ok": round(float(ok.mean()), 4), "passes_mean": round(float(ps.mean()), 3),
                                         "first_pass_hits": round(float((ps == 1).mean()), 4),
                                         "median_abs_miss": round(float(np.median(np.abs(cr / target - 1))), 4)}
        for name, _ in methods:
            dt = statistics.median(times[name])
            tot[name] += dt
            per[target][name] = {"fields_per_s": round(b.nf / dt, 2),
                                 "fields_per_s_runs": [round(b.nf / t, 1) for t in times[name]], **per[target][name]}
        jobs += b.nf
    clk = clocks.stop()
    b.close()
    fps = {k: jobs / v for k, v in tot.items()}
    line = {
        "metric": "fixed-rate fields/s at +/-5% ratio", "value": round(fps["learned"], 2), "unit": "fields/s",
        "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": round(1000 * tot["learned"], 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded on-device fields)",
        "config": {"workload": wl["desc"], "fields": 500, "targets": [8, 16, 32], "tolerance": 0.05,
                   "max_passes": 20, "field_bytes": int(nbytes),
                   "timing": "per target, each method run 3 times in rotated order; the median run counts"},
        "bisection_fields_per_s": round(fps["bisection"], 2),
        "speedup_vs_bisection": round(fps["learned"] / fps["bisection"], 2),
        "zero_network_fields_per_s": round(fps["zero_network"], 2),
        "learned_gbs": round(nbytes * 3 / tot["learned"] / 1e9, 1),
        "per_target": {str(int(k)): v for k, v in per.items()},
        "training": {"rows": rows, "label_var": round(var, 5), "final_mse": round(loss, 5),
                     "corpus_s": round(t1 - t0, 1), "train_s": round(t2 - t1, 2)},
        "clocks": clk,
    }
    return line


def run_batched(args, wl, fields=None):
    """C4: one batch (one persistent launch per kernel, replayed from a CUDA
    graph) against the same fields compressed by per-field calls."""
    import numpy as np
    import torch

    from szx_gb300._lib import StreamInfo, lib

    class Field(C.Structure):
        _fields_ = [("in_", C.c_void_p), ("nbEle", C.c_size_t), ("inBytes", C.c_size_t),
                    ("absErrBound", C.c_float), ("reserved", C.c_int), ("out", C.c_void_p), ("outCapacity", C.c_size_t)]

    L = lib()
    L.SZxG_batch_create.restype = C.c_void_p
    L.SZxG_batch_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    L.SZxG_batch_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.SZxG_batch_status.argtypes = [C.c_void_p, C.c_void_p]
    L.SZxG_batch_destroy.argtypes = [C.c_void_p]
    mode, bs = wl["mode"], wl["bs"]
    nfields = fields or args.fields
    xs, ebs = make_batch_fields(nfields, 4242, "cuda")
    nf = len(xs)
    total_in = sum(x.numel() for x in xs) * 4
    outs, fields = [], (Field * nf)()
    for k, (x, eb) in enumerate(zip(xs, ebs)):
        cap = L.SZxG_compress_bound(mode, 0, x.numel(), bs)
        o = torch.empty(cap, dtype=torch.uint8, device="cuda")
        outs.append(o)
        fields[k] = Field(x.data_ptr(), x.numel(), 0, eb, 0, o.data_ptr(), cap)
    b = L.SZxG_batch_create(0, mode, 0, bs, nf, C.cast(fields, C.c_void_p))
    assert b, L.SZxG_error_string(L.SZxG_get_last_error())
    info = torch.zeros(nf * C.sizeof(StreamInfo), dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(args.warmup):
            assert L.SZxG_batch_run(b, C.c_void_p(info.data_ptr()), C.c_void_p(s.cuda_stream)) == 0
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        assert L.SZxG_batch_run(b, C.c_void_p(info.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    graph.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    time.sleep(0.3)
    e0.record()
    for _ in range(args.steps):
        graph.replay()
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    batched_ms = e0.elapsed_time(e1) / args.steps
    assert L.SZxG_batch_status(b, C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    raw = info.cpu().numpy().tobytes()
    sizes_out = [StreamInfo.from_buffer_copy(raw[k * C.sizeof(StreamInfo):(k + 1) * C.sizeof(StreamInfo)]).size
                 for k in range(nf)]
    # per-field launches of the same fields (one reused workspace)
    wsb = max(L.SZxG_workspace_size(mode, 0, x.numel(), bs) for x in xs)
    ws = torch.zeros(wsb, dtype=torch.uint8, device="cuda")
    inf1 = torch.zeros(C.sizeof(StreamInfo), dtype=torch.uint8, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def one(k):
        x = xs[k]
        return L.SZxG_compress(mode, 0, C.c_void_p(x.data_ptr()), x.numel(), bs, 0, ebs[k], 0.0,
                               C.c_void_p(outs[k].data_ptr()), outs[k].numel(), C.c_void_p(ws.data_ptr()), wsb,
                               C.c_void_p(inf1.data_ptr()), st)
    for k in range(nf):
        assert one(k) == 0
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(nf + 1)]
    per_field = []
    loop_ms = []
    for _ in range(max(1, args.steps // 2)):
        evs[0].record()
        for k in range(nf):
            one(k)
            evs[k + 1].record()
        torch.cuda.synchronize()
        loop_ms.append(evs[0].elapsed_time(evs[nf]))
        per_field = [evs[k].elapsed_time(evs[k + 1]) for k in range(nf)]
    loop_ms = statistics.median(loop_ms)
    # one large field alone (the single-field reference point for the batch)
    big = max(range(nf), key=lambda k: xs[k].numel())
    e0.record()
    for _ in range(args.steps):
        one(big)
    e1.record()
    torch.cuda.synchronize()
    big_gbs = xs[big].numel() * 4 / (e0.elapsed_time(e1) / args.steps / 1000) / 1e9
    L.SZxG_batch_destroy(b)
    pf = np.array(per_field)

    # the same streams decoded as one batch (graph replay) and by per-field calls
    offs = [StreamInfo.from_buffer_copy(raw[k * C.sizeof(StreamInfo):(k + 1) * C.sizeof(StreamInfo)]).offset
            for k in range(nf)]
    ys, dfields = [], (Field * nf)()
    for k in range(nf):
        y = torch.empty_like(xs[k])
        ys.append(y)
        dfields[k] = Field(outs[k].data_ptr() + offs[k], xs[k].numel(), sizes_out[k], 0.0, 0, y.data_ptr(),
                           y.numel() * 4)
    bd = L.SZxG_batch_create(1, mode, 0, bs, nf, C.cast(dfields, C.c_void_p))
    assert bd, L.SZxG_error_string(L.SZxG_get_last_error())
    dinfo = torch.zeros(nf * C.sizeof(StreamInfo), dtype=torch.uint8, device="cuda")
    with torch.cuda.stream(s):
        for _ in range(args.warmup):
            assert L.SZxG_batch_run(bd, C.c_void_p(dinfo.data_ptr()), C.c_void_p(s.cuda_stream)) == 0
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    dgraph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(dgraph):
        assert L.SZxG_batch_run(bd, C.c_void_p(dinfo.data_ptr()),
                                C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    dgraph.replay()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        dgraph.replay()
    e1.record()
    torch.cuda.synchronize()
    dec_ms = e0.elapsed_time(e1) / args.steps
    dec_status = L.SZxG_batch_status(bd, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    L.SZxG_batch_destroy(bd)
    assert dec_status == 0, dec_status
    bad = sum(int(not bool((ys[k] - xs[k]).abs().max() <= ebs[k] * 1.001)) for k in range(nf))

    def one_dec(k):
        return L.SZxG_decompress(mode, 0, C.c_void_p(outs[k].data_ptr() + offs[k]), sizes_out[k], xs[k].numel(), bs,
                                 C.c_void_p(ys[k].data_ptr()), C.c_void_p(ws.data_ptr()), wsb, st)
    for k in range(nf):
        assert one_dec(k) == 0
    torch.cuda.synchronize()
    dloop = []
    for _ in range(max(1, args.steps // 2)):
        evs[0].record()
        for k in range(nf):
            one_dec(k)
            evs[k + 1].record()
        torch.cuda.synchronize()
        dloop.append(evs[0].elapsed_time(evs[nf]))
        dper = [evs[k].elapsed_time(evs[k + 1]) for k in range(nf)]
    dloop = statistics.median(dloop)
    dpf = np.array(dper)
    # the launch shapes the autotuner chose per size class against the fixed
    # default shape, same fields, median of graph replays each
    from szx_gb300 import tune
    del ys
    torch.cuda.empty_cache()
    tuned_table = tune.get_shapes()
    t_ms = tune.time_batch(xs, ebs, outs, mode, bs)
    tune.set_shapes([((1 << 64) - 1, 0, 0, 0)])
    try:
        f_ms = tune.time_batch(xs, ebs, outs, mode, bs)
    finally:
        tune.set_shapes([])
    shapes = {"table": [list(e) for e in tuned_table],
              "tuned_compress_gbs": round(total_in / (t_ms[0] / 1000) / 1e9, 2),
              "tuned_decompress_gbs": round(total_in / (t_ms[1] / 1000) / 1e9, 2),
              "fixed_compress_gbs": round(total_in / (f_ms[0] / 1000) / 1e9, 2),
              "fixed_decompress_gbs": round(total_in / (f_ms[1] / 1000) / 1e9, 2),
              "note": "table: per size class (max values, encoder tile variant, encoder CTAs/SM, decoder CTAs/SM; "
                      "0 = as many as fit); fixed: one class, default shape"}
    line = {
        "metric": "batched compress GB/s (mixed float32 fields, ABS)", "value": round(total_in / (batched_ms / 1000) / 1e9, 2),
        "unit": "GB/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(batched_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded on-device fields)",
        "config": {"workload": wl["desc"], "fields": nf, "elements": total_in // 4,
                   "stream_bytes": int(sum(sizes_out)), "graph": True,
                   "l2": "total input far above L2; no flush needed"},
        "per_field_launches": {"value": round(total_in / (loop_ms / 1000) / 1e9, 2), "unit": "GB/s",
                               "ms_per_step": round(loop_ms, 3), "p50_ms": round(float(np.percentile(pf, 50)), 4),
                               "p99_ms": round(float(np.percentile(pf, 99)), 4)},
        "single_field_gbs": round(big_gbs, 2), "single_field_elements": xs[big].numel(),
        "batched_vs_single": round(total_in / (batched_ms / 1000) / 1e9 / big_gbs, 3),
        "launch_shapes": shapes,
        "decompress": {"batched_gbs": round(total_in / (dec_ms / 1000) / 1e9, 2), "ms_per_step": round(dec_ms, 4),
                       "per_field_gbs": round(total_in / (dloop / 1000) / 1e9, 2),
                       "p50_ms": round(float(np.percentile(dpf, 50)), 4),
                       "p99_ms": round(float(np.percentile(dpf, 99)), 4),
                       "fields_over_bound": bad},
        "clocks": clk,
    }
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--fields", type=int, default=2000, help="c4: number of fields")
    ap.add_argument("--extras", dest="extras", action="store_true", default=True,
                    help="c2 at N=1: add the mode1, batched and fixed_rate keys (default)")
    ap.add_argument("--no-extras", dest="extras", action="store_false")
    ap.add_argument("--extra-fields", type=int, default=2000, help="fields of the batched extra key")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        if "rel" not in wl:
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": f"no CPU arm for workload {args.workload}; "
                                  "the reference arm times the single-field codec"}), flush=True)
            return
        run_reference(args, wl, rank, world)
        return
    if args.workload == "c4":
        print(json.dumps(run_batched(args, wl)), flush=True)
        return
    if args.workload == "c5":
        print(json.dumps(run_fixed_rate(args, wl)), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as D
        torch.cuda.set_device(local_rank)
        D.init_process_group("nccl")
    run_ours(args, wl, rank, world, local_rank)
    if world > 1:
        import torch.distributed as D
        D.destroy_process_group()


if __name__ == "__main__":
    main()
