"""SZxG_compress_noalloc: the compress entry point for callers that may not
allocate device memory (applications whose own pool allocator owns the GPU's
memory, loops that cannot pay for cudaMalloc's device-wide synchronisation).

It must produce exactly the stream of the allocating entry point
(SZxG_compress), call after call, although every call reuses the same fixed
device scratch array.  Kept in a file of its own, collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_BLOCKS = 1 << 20   # the fixed scratch's limit, in blocks of blockSize values


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a CUDA device is required")
    from szx_gb300 import build
    build.build()
    from szx_gb300._lib import StreamInfo, lib
    L = lib()
    L.SZxG_compress_noalloc.restype = C.c_int
    L.SZxG_compress_noalloc.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_int, C.c_int, C.c_float,
                                        C.c_float, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
    return torch, L, StreamInfo


def _info(torch, t, StreamInfo):
    return StreamInfo.from_buffer_copy(t.cpu().numpy().tobytes())


def _run(env, fastMode, x, bs, err_mode, eb, rel):
    """(allocating stream, no-alloc stream) for the same input."""
    torch, L, StreamInfo = env
    code = 0 if x.dtype == torch.float32 else 1
    n = x.numel()
    cap = L.SZxG_compress_bound(fastMode, code, n, bs)
    wsb = L.SZxG_workspace_size(fastMode, code, n, bs)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    out_a = torch.empty(cap, dtype=torch.uint8, device="cuda")
    ws = torch.zeros(wsb, dtype=torch.uint8, device="cuda")
    info_a = torch.zeros(C.sizeof(StreamInfo), dtype=torch.uint8, device="cuda")
    rc = L.SZxG_compress(fastMode, code, C.c_void_p(x.data_ptr()), n, bs, err_mode, eb, rel,
                         C.c_void_p(out_a.data_ptr()), cap, C.c_void_p(ws.data_ptr()), wsb,
                         C.c_void_p(info_a.data_ptr()), stream)
    assert rc == 0
    out_b = torch.empty(cap, dtype=torch.uint8, device="cuda")
    info_b = torch.zeros(C.sizeof(StreamInfo), dtype=torch.uint8, device="cuda")
    rc = L.SZxG_compress_noalloc(fastMode, code, C.c_void_p(x.data_ptr()), n, bs, err_mode, eb, rel,
                                 C.c_void_p(out_b.data_ptr()), cap, C.c_void_p(info_b.data_ptr()), stream)
    assert rc == 0, L.SZxG_error_string(rc)
    torch.cuda.synchronize()
    ia, ib = _info(torch, info_a, StreamInfo), _info(torch, info_b, StreamInfo)
    assert ia.status == 0 and ib.status == 0
    a = out_a[ia.offset: ia.offset + ia.size].cpu().numpy().tobytes()
    b = out_b[ib.offset: ib.offset + ib.size].cpu().numpy().tobytes()
    return a, b


def test_noalloc_matches_allocating_entry_point_on_two_calls_in_a_row(env):
    torch = env[0]
    from szx_gb300 import synth
    g = torch.Generator(device="cuda").manual_seed(5)
    first = synth.spectral_field((64, 64, 128), seed=3, device="cuda")              # 524,288 float32
    second = (torch.randn(1_000_003, generator=g, device="cuda", dtype=torch.float64)
              .cumsum(0) * 1e-3).contiguous()                                       # different type and size
    # call 1: float32, REL, random-access layout; call 2: float64, ABS, native-endian layout
    a, b = _run(env, 3, first, 128, 1, 0.0, 1e-3)
    assert a == b and len(a) > 20
    a, b = _run(env, 4, second, 64, 0, 1e-4, 0.0)
    assert a == b and len(a) > 20
    # call 3: smaller again, a block count that is not a multiple of the tile,
    # after a larger call left its contents in the shared array
    third = (torch.randn(77_777, generator=g, device="cuda") * 3).contiguous()
    a, b = _run(env, 3, third, 128, 0, 1e-2, 0.0)
    assert a == b and len(a) > 20
    torch_, L, _ = env
    assert L.SZxG_get_last_error() == 0


def test_noalloc_at_its_full_block_count(env):
    torch = env[0]
    g = torch.Generator(device="cuda").manual_seed(9)
    n = MAX_BLOCKS * 8 - 3            # exactly MAX_BLOCKS blocks of 8 values, the last one short
    x = (torch.randn(n, generator=g, device="cuda").cumsum(0) * 1e-3).contiguous()
    a, b = _run(env, 3, x, 8, 0, 1e-3, 0.0)
    assert a == b and len(a) > 20


def test_noalloc_rejects_inputs_beyond_its_scratch(env):
    torch, L, StreamInfo = env
    x = torch.zeros(16, dtype=torch.float32, device="cuda")
    out = torch.empty(64, dtype=torch.uint8, device="cuda")
    info = torch.zeros(C.sizeof(StreamInfo), dtype=torch.uint8, device="cuda")
    too_many = MAX_BLOCKS * 128 + 1     # rejected from its size alone, before any GPU work
    rc = L.SZxG_compress_noalloc(3, 0, C.c_void_p(x.data_ptr()), too_many, 128, 0, 1e-3, 0.0,
                                 C.c_void_p(out.data_ptr()), 1 << 40, C.c_void_p(info.data_ptr()),
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 7
    assert L.SZxG_get_last_error() == 7
    assert b"fixed scratch" in L.SZxG_error_string(rc)
    rc = L.SZxG_compress_noalloc(1, 0, C.c_void_p(x.data_ptr()), 16, 128, 0, 1e-3, 0.0,
                                 C.c_void_p(out.data_ptr()), 1 << 20, C.c_void_p(info.data_ptr()),
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 6 and L.SZxG_get_last_error() == 6
