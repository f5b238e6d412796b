"""Compile the probebwa_gb300 native library (CUDA for sm_103a + host C++).

Produces probebwa_gb300/_lib/libprobebwa_gb300.so with the C ABI declared in
include/probebwa_gpu.h. Translation units compile in parallel; the link is
one nvcc call. -fmad=false and -ffp-contract=off keep FP64 sums and products
unfused, matching the reference's (Rust) arithmetic.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libprobebwa_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-Xptxas", "-v"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def headers():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))) + [
        os.path.join(os.path.dirname(HERE), "include", "probebwa_gpu.h")]


def _compile(src: str) -> tuple[str, str]:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    newest_dep = max(os.path.getmtime(p) for p in [src] + headers())
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj, ""
    cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [_nvcc(), "-x", "cu", *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(_compile, srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_cli()
    return LIB


CLI_SRC = os.path.join(HERE, "cli", "probebwa.cpp")
CLI = os.path.join(LIBDIR, "probebwa")


def build_cli() -> str:
    """The `probebwa` command line (host C++ over the C ABI), linked against
    the library in the same folder."""
    deps = [CLI_SRC, LIB, os.path.join(os.path.dirname(HERE), "include", "probebwa_gpu.h")]
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(p) for p in deps):
        return CLI
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-Wall", "-o", CLI, CLI_SRC, "-L" + LIBDIR,
           "-lprobebwa_gb300", "-Wl,-rpath,$ORIGIN", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{r.stdout}\n{r.stderr}")
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
