"""File I/O (include/szx_rw.h) and the `szx` command-line tool.

CPU: the SZx_read*/write* functions of the library (raw bytes, native and
swapped byte order, text output, status codes) and the tool's option
handling.  GPU: files compressed by the tool hold the reference's streams
(checked against the oracle), decompression writes the oracle's values, and
-a prints the reference tool's statistics.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def rw():
    from szx_gb300 import build
    build.build()
    L = C.CDLL(build.LIB)
    cp, vp, szp, ip = C.c_char_p, C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_int)
    for name, res, args in [
        ("SZx_checkFileExistance", C.c_int, [cp]),
        ("SZx_checkFileSize", C.c_size_t, [cp, ip]),
        ("SZx_readByteData", vp, [cp, szp, ip]),
        ("SZx_readFloatData", vp, [cp, szp, ip]),
        ("SZx_readDoubleData", vp, [cp, szp, ip]),
        ("SZx_readFloatData_systemEndian", vp, [cp, szp, ip]),
        ("SZx_writeByteData", None, [vp, C.c_size_t, cp, ip]),
        ("SZx_writeFloatData", None, [vp, C.c_size_t, cp, ip]),
        ("SZx_writeDoubleData", None, [vp, C.c_size_t, cp, ip]),
        ("SZx_writeIntData", None, [vp, C.c_size_t, cp, ip]),
        ("SZx_writeData", None, [vp, C.c_int, C.c_size_t, cp, ip]),
        ("SZx_writeFloatData_inBytes", None, [vp, C.c_size_t, cp, ip]),
        ("SZx_writeDoubleData_inBytes", None, [vp, C.c_size_t, cp, ip]),
    ]:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    libc = C.CDLL(None)
    libc.free.argtypes = [vp]
    return L, libc, build.CLI


def _take(libc, p, nbytes, dtype):
    a = np.frombuffer(C.string_at(p, nbytes), dtype).copy()
    libc.free(p)
    return a


def test_raw_files_round_trip_and_byte_order(rw, tmp_path):
    L, libc, _ = rw
    st = C.c_int(7)
    n = C.c_size_t()
    x = np.random.default_rng(1).normal(size=1001).astype(np.float32)
    path = str(tmp_path / "x.f32").encode()
    L.SZx_writeFloatData_inBytes(x.ctypes.data, x.size, path, C.byref(st))
    assert st.value == 0 and L.SZx_checkFileExistance(path) == 1
    assert L.SZx_checkFileSize(path, C.byref(st)) == x.nbytes and st.value == 0
    p = L.SZx_readFloatData(path, C.byref(n), C.byref(st))
    assert st.value == 0 and n.value == x.size
    assert np.array_equal(_take(libc, p, x.nbytes, np.float32), x)
    # a big-endian file read with dataEndianType = BIG_ENDIAN_DATA
    d = np.random.default_rng(2).normal(size=77)
    pathd = str(tmp_path / "x.be").encode()
    be = d.astype(">f8").tobytes()
    L.SZx_writeByteData(be, len(be), pathd, C.byref(st))
    flag = C.c_int.in_dll(L, "dataEndianType")
    flag.value = 1
    try:
        p = L.SZx_readDoubleData(pathd, C.byref(n), C.byref(st))
        assert st.value == 0 and n.value == d.size
        assert np.array_equal(_take(libc, p, d.nbytes, np.float64), d)
    finally:
        flag.value = 0
    p = L.SZx_readByteData(pathd, C.byref(n), C.byref(st))
    assert _take(libc, p, n.value, np.uint8).tobytes() == be


def test_text_output_and_status_codes(rw, tmp_path):
    L, libc, _ = rw
    st = C.c_int(7)
    x = np.array([1.5, -0.1, 3e-30], np.float32)
    p = str(tmp_path / "x.txt").encode()
    L.SZx_writeFloatData(x.ctypes.data, x.size, p, C.byref(st))
    assert st.value == 0
    assert open(p, "rb").read().decode() == "".join("%.30G\n" % float(v) for v in x)
    d = np.array([2.0 / 3.0, -1e300])
    L.SZx_writeData(d.ctypes.data, 1, d.size, p, C.byref(st))
    assert open(p, "rb").read().decode() == "".join("%.20G\n" % v for v in d)
    i = np.array([3, -4], np.int32)
    L.SZx_writeIntData(i.ctypes.data, i.size, p, C.byref(st))
    assert open(p, "rb").read().decode() == "3\n-4\n"
    L.SZx_writeData(d.ctypes.data, 7, d.size, p, C.byref(st))
    assert st.value == -3   # SZx_TERR
    n = C.c_size_t()
    missing = str(tmp_path / "missing").encode()
    assert L.SZx_readFloatData(missing, C.byref(n), C.byref(st)) is None and st.value == -2   # SZx_FERR
    assert L.SZx_checkFileExistance(missing) == 0


def test_tool_version_and_usage(rw):
    cli = rw[2]
    r = subprocess.run([cli, "-v"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "version: 1.1.0"
    for args in ([], ["-h"], ["-q"], ["-zz"]):
        r = subprocess.run([cli, *args], capture_output=True, text=True)
        assert r.returncode == 0 and r.stdout.startswith("Usage: szx")


# ------------------------------------------------------------------ GPU

def _run(cli, *args):
    r = subprocess.run([cli, *map(str, args)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("dt,flag,mode", [(np.float32, "-f", 3), (np.float32, "-f", 1), (np.float64, "-d", 3),
                                          (np.float32, "-f", 2), (np.float64, "-d", 4)])
def test_tool_streams_and_values_match_the_oracle(rw, tmp_path, dt, flag, mode):
    cli = rw[2]
    rng = np.random.default_rng(3)
    x = (np.cumsum(rng.normal(size=(16, 32, 70)), axis=2) * 1e-2).astype(dt)
    raw = tmp_path / "field.raw"
    x.tofile(raw)
    eb = 1e-3
    out = _run(cli, "-z", flag, "-i", raw, "-m", mode, "-M", "ABS", "-A", eb, "-3", 70, 32, 16)
    assert "compressed data file: %s.szx" % raw in out
    s = open(f"{raw}.szx", "rb").read()
    want = O.fast_compress_args(mode, x.ravel(), 0, eb, 0.0, 128)
    assert s == want
    out = _run(cli, "-x", flag, "-s", f"{raw}.szx", "-m", mode, "-3", 70, 32, 16, "-i", raw, "-a")
    y = np.fromfile(f"{raw}.szx.out", dt)
    z = O.decompress(mode, dt, want, x.size)
    assert np.array_equal(y.view(np.uint8), z.view(np.uint8))
    assert "compressionRatio=%f" % (x.nbytes / len(s)) in out
    assert "Max absolute error" in out and "PSNR" in out


@pytest.mark.gpu
def test_tool_rel_fxr_and_text_output(rw, tmp_path):
    cli = rw[2]
    rng = np.random.default_rng(4)
    x = (np.sin(np.arange(200000) / 500.0) + rng.normal(size=200000) * 1e-3).astype(np.float32)
    raw = tmp_path / "sig.f32"
    x.tofile(raw)
    # REL: the tool converts the bound with the value range, then compresses with ABS
    _run(cli, "-z", tmp_path / "rel.szx", "-f", "-i", raw, "-m", 3, "-M", "REL", "-R", 1e-3, "-1", x.size)
    eb = float(np.float32(np.float32(x.max() - x.min()) * np.float32(1e-3)))
    assert open(tmp_path / "rel.szx", "rb").read() == O.fast_compress_args(3, x, 0, eb, 0.0, 128)
    # fixed rate: the stream the library's FXR path writes
    from szx_gb300 import api
    _run(cli, "-z", tmp_path / "fxr.szx", "-f", "-i", raw, "-M", "FXR", "-C", 8, "-T", 0.1, "-1", x.size)
    assert open(tmp_path / "fxr.szx", "rb").read() == api.fast_compress_args(2, x, 2, compressionRatio=8.0,
                                                                            tolerance=0.1)
    # text output
    _run(cli, "-x", tmp_path / "rel.txt", "-f", "-s", tmp_path / "rel.szx", "-m", 3, "-t", "-1", x.size)
    y = O.decompress(3, np.float32, open(tmp_path / "rel.szx", "rb").read(), x.size)
    lines = open(tmp_path / "rel.txt").read().splitlines()
    assert lines == ["%.30G" % float(v) for v in y]
