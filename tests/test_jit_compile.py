"""CPU: the plan compiler's kernel instances compile with NVRTC for sm_103a.

The library compiles these at plan time on the GPU host (csrc/jit.cu), and a
failed compile there falls back to the run-time-stage library kernels, so a
header change that breaks them would only show as slower plans. This test
hands NVRTC the same headers, options and name expressions (the instances
of the benchmark's plans, the four-step passes, the Bluestein middle pass
and the Rader rows) and checks that each compiles, and that the
hot ones stay free of register spills. NVRTC needs no GPU.
"""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "chfft_gb300", "csrc")
HEADERS = ["common.cuh", "engine.cuh", "kernels.cuh", "k_complex.cuh", "k_real.cuh", "tc.cuh", "tc_core.cuh"]
OPTS = ["--gpu-architecture=sm_103a", "--std=c++17", "-lineinfo", "-DCHFFT_PLAN_TIME=1", "-Xptxas=-v"]


def _nvrtc():
    for name in ("libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                 "/usr/local/cuda/lib64/libnvrtc.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.skip("NVRTC not available")


def compile_expr(expr):
    lib = _nvrtc()
    srcs = [open(os.path.join(CSRC, h)).read().encode() for h in HEADERS]
    names = [h.encode() for h in HEADERS]
    prog = ctypes.c_void_p()
    main = b'#include "k_complex.cuh"\n#include "k_real.cuh"\n#include "tc_core.cuh"\n'
    n = len(HEADERS)
    rc = lib.nvrtcCreateProgram(ctypes.byref(prog), main, b"chfft_plan.cu", n, (ctypes.c_char_p * n)(*srcs),
                                (ctypes.c_char_p * n)(*names))
    assert rc == 0
    assert lib.nvrtcAddNameExpression(prog, expr.encode()) == 0
    opts = [o.encode() for o in OPTS]
    rc = lib.nvrtcCompileProgram(prog, len(opts), (ctypes.c_char_p * len(opts))(*opts))
    size = ctypes.c_size_t()
    lib.nvrtcGetProgramLogSize(prog, ctypes.byref(size))
    log = ctypes.create_string_buffer(size.value)
    lib.nvrtcGetProgramLog(prog, log)
    lib.nvrtcDestroyProgram(ctypes.byref(prog))
    return rc, log.value.decode(errors="replace")


A_2P20 = "chfft::StatCore<false,true,false,1024,1024,8,1058,32,256,2,0,32,32>"
CASES = [
    # (name expression, must be spill-free)
    ("&chfft::kern::k_c2c<float, chfft::StatCore<false,false,true,1000,1000,2,1101,10,224,6,0,10,10,10>>", True),
    ("&chfft::kern::k_c2c<float, chfft::StatCore<true,false,false,2048,1009,1,2177,16,128,8,16,16,16,8>>", True),
    ("&chfft::kern::k_c2c<float, chfft::StatCore<false,false,false,2048,2048,1,2177,16,128,8,16,16,16,8>>", True),
    ("&chfft::kern::k_cols<float, chfft::StatCore<false,true,false,2048,2048,8,2178,16,512,1,0,16,16,8>>", True),
    (f"&chfft::kern::k_cols_tw<float, {A_2P20}, 8>", True),
    (f"&chfft::kern::k_rows_t<float, {A_2P20}, 0>", True),
    (f"&chfft::kern::k_rows_t<float, {A_2P20}, 2>", False),
    ("&chfft::kern::k_rows_bb<float, chfft::StatCore<false,true,true,512,512,8,546,16,256,4,0,16,16,2>, 3>", True),
    # Rader rows of N = 1009 (the 1008-point core, one sequence per CTA)
    ("&chfft::kern::k_c2c_rader<float, chfft::StatCore<false,false,true,1008,1008,1,1071,16,352,2,0,16,3,3,7>>", True),
    # ... and its two-pass order (1008 = 28 x 36), six sequences per CTA
    ("&chfft::kern::k_c2c_rader<float, chfft::StatCore<false,false,true,1008,1008,6,1045,28,224,2,0,28,36>>", True),
    ("&chfft::kern::k_rows_bb<double, chfft::StatCore<false,true,false,256,256,4,274,16,256,1,0,16,16>, 7>", False),
]


@pytest.mark.parametrize("expr,spill_free", CASES)
def test_plan_time_instance_compiles(expr, spill_free):
    rc, log = compile_expr(expr)
    assert rc == 0, log[-2000:]
    spills = [int(v) for v in re.findall(r"(\d+) bytes spill stores", log)]
    assert spills, log[-500:]
    if spill_free:
        assert max(spills) == 0, log[-1000:]
