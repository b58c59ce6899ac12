"""Build libchfft_gb300.so in-tree with nvcc for sm_103a.

Each CUDA translation unit under csrc/ compiles in parallel to an object
file in _build/, then nvcc links the shared library into _lib/. Only the
C ABI symbols of include/chfft_gpu.h are exported (-fvisibility=hidden).
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
LIB = os.path.join(LIBDIR, "libchfft_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-I", INCLUDE, "-I", BUILD]
# Kernel headers the plan-time compiler (csrc/jit.cu) hands to NVRTC.
JIT_HEADERS = ["common.cuh", "engine.cuh", "kernels.cuh", "k_complex.cuh", "k_real.cuh", "tc.cuh", "tc_core.cuh"]


def _gen_jit_headers() -> None:
    """Write _build/jit_headers.inc: the kernel headers as C++ raw strings."""
    names, srcs = [], []
    for h in JIT_HEADERS:
        text = open(os.path.join(CSRC, h)).read()
        if ")CHFFT_SRC\"" in text:
            raise RuntimeError(f"{h} contains the raw-string delimiter")
        names.append(f'"{h}"')
        srcs.append('R"CHFFT_SRC(' + text + ')CHFFT_SRC"')
    body = (f"static const int kJitHeaderCount = {len(JIT_HEADERS)};\n"
            f"static const char* const kJitHeaderNames[] = {{{', '.join(names)}}};\n"
            f"static const char* const kJitHeaderSrc[] = {{\n" + ",\n".join(srcs) + "};\n")
    out = os.path.join(BUILD, "jit_headers.inc")
    if not os.path.exists(out) or open(out).read() != body:
        with open(out, "w") as f:
            f.write(body)


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _compile(src: str, nvcc: str, header_mtime: float) -> str:
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), header_mtime):
        return obj
    tmp = obj + f".tmp{os.getpid()}"
    cmd = [nvcc, *ARCH, *FLAGS, "-c", src, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}")
    os.replace(tmp, obj)
    return obj


def build(force: bool = False, jobs: int | None = None) -> str:
    """Compile every .cu under csrc/ and link libchfft_gb300.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    if force:
        for f in os.listdir(BUILD):
            if f.endswith(".o"):
                os.remove(os.path.join(BUILD, f))
    _gen_jit_headers()
    hm = max(os.path.getmtime(h) for h in _headers())
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc, hm), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link of libchfft_gb300.so failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
