"""Batched fields: one persistent launch per kernel over a work queue of
(field, block-range) tiles.  Every field's stream must equal what the
single-field entry point produces for it (which the parity tests pin to the
reference), for uneven sizes down to one value, and replaying the batch from
a captured CUDA graph must reproduce it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class Field(C.Structure):
    _fields_ = [("in_", C.c_void_p), ("nbEle", C.c_size_t), ("inBytes", C.c_size_t), ("absErrBound", C.c_float),
                ("reserved", C.c_int), ("out", C.c_void_p), ("outCapacity", C.c_size_t)]


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a CUDA device is required")
    from szx_gb300 import build
    build.build()
    from szx_gb300._lib import StreamInfo, lib
    L = lib()
    L.SZxG_batch_create.restype = C.c_void_p
    L.SZxG_batch_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    L.SZxG_batch_run.restype = C.c_int
    L.SZxG_batch_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.SZxG_batch_status.restype = C.c_int
    L.SZxG_batch_status.argtypes = [C.c_void_p, C.c_void_p]
    L.SZxG_batch_destroy.restype = None
    L.SZxG_workspace_status.restype = C.c_int
    L.SZxG_batch_destroy.argtypes = [C.c_void_p]
    return torch, L, StreamInfo


def _single(env, mode, x, bs, eb):
    torch, L, StreamInfo = env
    code = 0 if x.dtype == torch.float32 else 1
    n = x.numel()
    cap = L.SZxG_compress_bound(mode, code, n, bs)
    wsb = L.SZxG_workspace_size(mode, code, n, bs)
    out = torch.empty(cap, dtype=torch.uint8, device="cuda")
    ws = torch.zeros(wsb, dtype=torch.uint8, device="cuda")
    info = torch.zeros(C.sizeof(StreamInfo), dtype=torch.uint8, device="cuda")
    rc = L.SZxG_compress(mode, code, C.c_void_p(x.data_ptr()), n, bs, 0, eb, 0.0, C.c_void_p(out.data_ptr()), cap,
                         C.c_void_p(ws.data_ptr()), wsb, C.c_void_p(info.data_ptr()),
                         C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    i = StreamInfo.from_buffer_copy(info.cpu().numpy().tobytes())
    return out[i.offset: i.offset + i.size].cpu().numpy().tobytes()


def _batch(env, mode, xs, bs, ebs, graph=False):
    torch, L, StreamInfo = env
    code = 0 if xs[0].dtype == torch.float32 else 1
    outs, fields = [], (Field * len(xs))()
    for k, (x, eb) in enumerate(zip(xs, ebs)):
        cap = L.SZxG_compress_bound(mode, code, x.numel(), bs)
        o = torch.empty(cap, dtype=torch.uint8, device="cuda")
        outs.append(o)
        fields[k] = Field(x.data_ptr(), x.numel(), 0, eb, 0, o.data_ptr(), cap)
    b = L.SZxG_batch_create(0, mode, code, bs, len(xs), C.cast(fields, C.c_void_p))
    assert b, L.SZxG_error_string(L.SZxG_get_last_error())
    info = torch.zeros(len(xs) * C.sizeof(StreamInfo), dtype=torch.uint8, device="cuda")
    try:
        if graph:
            g = torch.cuda.CUDAGraph()
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                assert L.SZxG_batch_run(b, C.c_void_p(info.data_ptr()), C.c_void_p(s.cuda_stream)) == 0   # warm
            torch.cuda.current_stream().wait_stream(s)
            torch.cuda.synchronize()
            for o in outs:
                o.zero_()
            info.zero_()
            with torch.cuda.graph(g):
                rc = L.SZxG_batch_run(b, C.c_void_p(info.data_ptr()),
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
                assert rc == 0
            torch.cuda.synchronize()
            for o in outs:
                o.zero_()
            g.replay()
            g.replay()
        else:
            assert L.SZxG_batch_run(b, C.c_void_p(info.data_ptr()),
                                    C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
        assert L.SZxG_batch_status(b, C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
        torch.cuda.synchronize()
        raw = info.cpu().numpy().tobytes()
        res = []
        for k, o in enumerate(outs):
            i = StreamInfo.from_buffer_copy(raw[k * C.sizeof(StreamInfo):(k + 1) * C.sizeof(StreamInfo)])
            assert i.status == 0
            res.append(o[i.offset: i.offset + i.size].cpu().numpy().tobytes())
        return res
    finally:
        L.SZxG_batch_destroy(b)


def _fields(torch, dt, sizes, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    xs, ebs = [], []
    for k, n in enumerate(sizes):
        kind = k % 3
        if kind == 0:      # smooth random walk
            x = torch.randn(n, generator=g, device="cuda", dtype=torch.float64).cumsum(0) * 1e-2
        elif kind == 1:    # piecewise constant
            x = torch.repeat_interleave(torch.randn(n // 300 + 1, generator=g, device="cuda",
                                                    dtype=torch.float64), 300)[:n]
        else:              # white noise
            x = torch.randn(n, generator=g, device="cuda", dtype=torch.float64)
        x = x.to(dt).contiguous()
        rng = float((x.max() - x.min()).item()) or 1.0
        ebs.append(float(np.float32(rng * 10 ** (-2 - 3 * ((k * 7919) % 97) / 96.0))))
        xs.append(x)
    return xs, ebs


@pytest.mark.parametrize("mode,dtname,bs", [(3, "float32", 128), (4, "float64", 64), (2, "float32", 128),
                                            (3, "float64", 256)])
def test_batch_streams_equal_single_field_streams(env, mode, dtname, bs):
    torch = env[0]
    dt = getattr(torch, dtname)
    rng = np.random.default_rng(5)
    sizes = [1, 2, 127, 128, 129, 4097, 65536] + [int(v) for v in np.exp(rng.uniform(np.log(1 << 14),
                                                                                       np.log(1 << 21), 40))]
    xs, ebs = _fields(torch, dt, sizes, 7)
    got = _batch(env, mode, xs, bs, ebs)
    for k, (x, eb) in enumerate(zip(xs, ebs)):
        assert got[k] == _single(env, mode, x, bs, eb), (k, x.numel())


def test_batch_replays_from_a_cuda_graph(env):
    torch = env[0]
    xs, ebs = _fields(torch, torch.float32, [5000, 1 << 20, 333, 1 << 18, 70001], 11)
    want = _batch(env, 3, xs, 128, ebs)
    got = _batch(env, 3, xs, 128, ebs, graph=True)
    assert got == want


def _single_decompress(env, mode, stream, n, bs, dt):
    torch, L, StreamInfo = env
    code = 0 if dt == torch.float32 else 1
    wsb = L.SZxG_workspace_size(mode, code, n, bs)
    ws = torch.zeros(wsb, dtype=torch.uint8, device="cuda")
    out = torch.empty(n, dtype=dt, device="cuda")
    rc = L.SZxG_decompress(mode, code, C.c_void_p(stream.data_ptr()), stream.numel(), n, bs,
                           C.c_void_p(out.data_ptr()), C.c_void_p(ws.data_ptr()), wsb,
                           C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    assert L.SZxG_workspace_status(C.c_void_p(ws.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    return out


def _batch_decompress(env, mode, streams, ns, bs, dt, graph=False):
    """Decode device streams as one batch; returns (values per field, status per field, batch status)."""
    torch, L, StreamInfo = env
    code = 0 if dt == torch.float32 else 1
    outs, fields = [], (Field * len(streams))()
    for k, (s, n) in enumerate(zip(streams, ns)):
        o = torch.full((n,), 7.0, dtype=dt, device="cuda")
        outs.append(o)
        fields[k] = Field(s.data_ptr(), n, s.numel(), 0.0, 0, o.data_ptr(), o.numel() * o.element_size())
    b = L.SZxG_batch_create(1, mode, code, bs, len(streams), C.cast(fields, C.c_void_p))
    assert b, L.SZxG_error_string(L.SZxG_get_last_error())
    info = torch.zeros(len(streams) * C.sizeof(StreamInfo), dtype=torch.uint8, device="cuda")
    try:
        if graph:
            g = torch.cuda.CUDAGraph()
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                assert L.SZxG_batch_run(b, C.c_void_p(info.data_ptr()), C.c_void_p(s.cuda_stream)) == 0
            torch.cuda.current_stream().wait_stream(s)
            torch.cuda.synchronize()
            with torch.cuda.graph(g):
                assert L.SZxG_batch_run(b, C.c_void_p(info.data_ptr()),
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
            torch.cuda.synchronize()
            for o in outs:
                o.fill_(7.0)
            info.zero_()
            g.replay()
            g.replay()
        else:
            assert L.SZxG_batch_run(b, C.c_void_p(info.data_ptr()),
                                    C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
        st = L.SZxG_batch_status(b, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        raw = info.cpu().numpy().tobytes()
        infos = [StreamInfo.from_buffer_copy(raw[k * C.sizeof(StreamInfo):(k + 1) * C.sizeof(StreamInfo)])
                 for k in range(len(streams))]
        return outs, infos, st
    finally:
        L.SZxG_batch_destroy(b)


def _same(a, b):
    """Bitwise equality of two float tensors."""
    import torch
    it = torch.int32 if a.element_size() == 4 else torch.int64
    return a.shape == b.shape and bool((a.view(it) == b.view(it)).all())


@pytest.mark.parametrize("mode,dtname,bs", [(3, "float32", 128), (4, "float64", 64), (3, "float64", 256),
                                            (4, "float32", 16), (3, "float32", 1)])
def test_batch_decompress_equals_single_stream_decompress(env, mode, dtname, bs):
    torch = env[0]
    dt = getattr(torch, dtname)
    rng = np.random.default_rng(9)
    hi = 1 << 17 if bs == 1 else 1 << 21
    sizes = [1, 2, 127, 128, 129, 4097, 65536] + [int(v) for v in np.exp(rng.uniform(np.log(1 << 14),
                                                                                       np.log(hi), 30))]
    xs, ebs = _fields(torch, dt, sizes, 13)
    streams = [torch.tensor(np.frombuffer(s, np.uint8).copy(), device="cuda")
               for s in _batch(env, mode, xs, bs, ebs)]
    outs, infos, st = _batch_decompress(env, mode, streams, sizes, bs, dt)
    assert st == 0
    for k, (s, n) in enumerate(zip(streams, sizes)):
        assert infos[k].status == 0 and infos[k].size == n * xs[k].element_size()
        want = _single_decompress(env, mode, s, n, bs, dt)
        assert _same(outs[k], want), (k, n)


def test_batch_decompress_isolates_bad_streams_and_replays(env):
    """A truncated stream and one of another block size fail alone; the rest
    decode exactly, also when the batch is replayed from a CUDA graph."""
    torch = env[0]
    sizes = [70001, 1 << 18, 5000, 1 << 20, 333]
    xs, ebs = _fields(torch, torch.float32, sizes, 17)
    streams = [torch.tensor(np.frombuffer(s, np.uint8).copy(), device="cuda")
               for s in _batch(env, 3, xs, 128, ebs)]
    other_bs = torch.tensor(np.frombuffer(_single(env, 3, xs[2], 64, ebs[2]), np.uint8).copy(), device="cuda")
    bad = [streams[0], streams[1][: streams[1].numel() // 2].clone(), other_bs, streams[3], streams[4]]
    for graph in (False, True):
        outs, infos, st = _batch_decompress(env, 3, bad, sizes, 128, torch.float32, graph=graph)
        assert st == 3
        assert [i.status for i in infos] == [0, 3, 3, 0, 0]
        for k in (0, 3, 4):
            assert _same(outs[k], _single_decompress(env, 3, streams[k], sizes[k], 128, torch.float32)), k


@pytest.mark.parametrize("mode,dtname,bs", [(3, "float32", 128), (3, "float64", 64)])
def test_batch_streams_and_decodes_match_the_oracle(env, mode, dtname, bs):
    """64 fields drawn like the mixed-size batch workload (sizes log-uniform
    2^14..2^22, spectral / piecewise-constant / white noise, ABS bound
    log-uniform 1e-5..1e-2 x range): every batched stream equals the oracle's
    stream of that field (szx/src/szx_float.cc:1407-1489, double
    szx/src/szx_double.cc:1509-1590) byte for byte, and the batched decode
    equals the oracle's decode bit for bit."""
    import oracle as O
    from szx_gb300 import synth
    torch = env[0]
    dt = getattr(torch, dtname)
    xs, ebs = synth.batch_fields(64, 2024 + bs, 14, 22, "cuda", dt)
    got = _batch(env, mode, xs, bs, ebs)
    hosts = [x.cpu().numpy() for x in xs]
    for k, (xh, eb) in enumerate(zip(hosts, ebs)):
        assert got[k] == O.compress(mode, xh, eb, bs), (k, xh.size)
    streams = [torch.tensor(np.frombuffer(s, np.uint8).copy(), device="cuda") for s in got]
    outs, infos, st = _batch_decompress(env, mode, streams, [x.numel() for x in xs], bs, dt)
    assert st == 0
    it = np.uint32 if dt == torch.float32 else np.uint64
    for k, xh in enumerate(hosts):
        z = O.decompress(mode, xh.dtype, got[k], xh.size)
        assert np.array_equal(outs[k].cpu().numpy().view(it), z.view(it)), (k, xh.size)


def test_every_launch_shape_gives_the_same_streams(env):
    """Fields grouped by size class, each class one persistent launch with its
    own shape (encoder tile size and threads per CTA, CTAs per SM of encoder
    and decoder): for every shape the tuner may choose, and for a table that
    splits the fields into three classes, every stream equals the single-field
    stream and every batched decode equals the single-field decode."""
    from szx_gb300 import tune
    torch = env[0]
    rng = np.random.default_rng(31)
    sizes = [1, 129, 4097, 65536] + [int(v) for v in np.exp(rng.uniform(np.log(1 << 12), np.log(1 << 21), 20))]
    xs, ebs = _fields(torch, torch.float32, sizes, 37)
    want = [_single(env, 3, x, 128, eb) for x, eb in zip(xs, ebs)]
    want_dec = None
    M = (1 << 64) - 1
    tables = [[(M, tv, ec, dc)] for tv, ec in tune.ENC_CANDIDATES for dc in tune.DEC_CANDIDATES[:2]]
    tables.append([(1 << 14, 1, 4, 2), (1 << 18, 0, 2, 3), (M, 1, 0, 0)])
    try:
        for table in tables:
            tune.set_shapes(table)
            assert tune.get_shapes() == table
            got = _batch(env, 3, xs, 128, ebs)
            assert got == want, table
            streams = [torch.tensor(np.frombuffer(s, np.uint8).copy(), device="cuda") for s in got]
            outs, infos, st = _batch_decompress(env, 3, streams, sizes, 128, torch.float32)
            assert st == 0 and all(i.status == 0 for i in infos), table
            if want_dec is None:
                want_dec = [_single_decompress(env, 3, s, n, 128, torch.float32) for s, n in zip(streams, sizes)]
            for k in range(len(sizes)):
                assert _same(outs[k], want_dec[k]), (table, k)
    finally:
        tune.set_shapes([])
