"""Build recipe for libszx_gb300.so (CUDA kernels + C ABI) for sm_103a, and
the `szx` command-line tool (bin/szx) on top of it.

Each translation unit in csrc/ is compiled in parallel by nvcc with one
-gencode (compute_103a -> sm_103a), FMA contraction off (the reference does
plain IEEE adds/subtracts, and bit-exact streams depend on it) and -lineinfo
for the profiler; objects go to _build/ and are linked into
szx_gb300/libszx_gb300.so.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libszx_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-O3,-ffp-contract=off",
              "-Xptxas", "-O3", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build szx_gb300")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps += [os.path.join(os.path.dirname(PKG), "include", h) for h in ("szx_gb300.h", "szx_rw.h", "cuszx_entry.h")]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps if os.path.exists(d)):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile every .cu under csrc/ and link libszx_gb300.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if not (os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs)):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print("built", LIB)
    build_cli(verbose)
    return LIB


CLI_SRC = os.path.join(PKG, "cli", "szx.cpp")
CLI = os.path.join(PKG, "bin", "szx")


def build_cli(verbose: bool = False) -> str:
    """The `szx` command-line tool, linked against libszx_gb300.so (found next
    to bin/ through its rpath)."""
    inc = os.path.join(os.path.dirname(PKG), "include")
    deps = [CLI_SRC, LIB, os.path.join(inc, "szx_gb300.h"), os.path.join(inc, "szx_rw.h")]
    if os.path.exists(CLI) and all(os.path.getmtime(CLI) >= os.path.getmtime(d) for d in deps):
        return CLI
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", CLI_SRC, "-o", CLI, "-L" + PKG, "-lszx_gb300", "-lm",
           "-Wl,-rpath,$ORIGIN/.."]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the szx tool failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", CLI)
    return CLI


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
