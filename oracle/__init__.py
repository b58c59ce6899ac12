"""CPU oracle for the chfft transforms (test infrastructure only).

A C++17 restatement of chfft 0.3.4's algorithms (chfft_oracle.hpp) exposed
through ctypes. Only tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline leg use it, as the checker and the CPU baseline; the product
library under chfft_gb300/ never imports it.

Parity status: bit-level parity with the Rust reference is unpinned (the
crate cannot be compiled here); the restatement is pinned to the
reference's own test identities and tolerances and cross-checked against
numpy.fft (tests/test_oracle.py).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "liboracle.so")
_SRC = [os.path.join(_HERE, "chfft_oracle.cpp"), os.path.join(_HERE, "chfft_oracle.hpp")]

# Method ids shared with the C side (chfft_oracle.hpp `Method`).
METHODS = {
    "forward": 0, "forward0": 1, "forwardu": 2, "forwardn": 3,
    "backward": 4, "backward0": 5, "backwardu": 6, "backwardn": 7,
    "forward0i": 8, "backward0i": 9, "forwardui": 10, "backwardui": 11,
}

_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with g++ (-O3 -ffp-contract=off, no -march)."""
    os.makedirs(_BUILD, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in _SRC)
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < newest:
        tmp = _SO + f".tmp{os.getpid()}"
        cmd = ["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
               _SRC[0], "-o", tmp]
        subprocess.run(cmd, check=True)
        os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        sz = ctypes.c_size_t
        vp = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        i = ctypes.c_int
        _lib.orc_factorize.argtypes = [sz, sz, vp, vp, sz]
        _lib.orc_bitreverse.argtypes = [sz, vp, vp, sz, vp]
        _lib.orc_bitreverse2inplace.argtypes = [vp, sz, vp, i]
        _lib.orc_chirp_index.argtypes = [sz, vp]
        _lib.orc_omega.argtypes = [i, sz, vp]
        _lib.orc_cfft1d_mode.argtypes = [sz, vp]
        _lib.orc_cfft1d.argtypes = [i, sz, i, vp, vp, sz, i, dp]
        _lib.orc_cfft2d.argtypes = [i, sz, sz, i, vp, vp, sz, i, dp]
        _lib.orc_rfft1d.argtypes = [i, sz, i, vp, vp, sz, i, dp]
        _lib.orc_dct1d.argtypes = [i, i, sz, i, i, vp, vp, sz, i, dp]
        _lib.orc_mdct1d.argtypes = [i, sz, i, vp, i, vp, vp, sz, i, dp]
    return _lib


def _dt(a) -> int:
    return 0 if a.dtype in (np.float32, np.complex64) else 1


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleError(ValueError):
    pass


def _check(rc):
    if rc == 1:
        raise OracleError("invalid length")
    if rc != 0:
        raise OracleError(f"oracle error {rc}")


def factorize(n: int, max_prime: int = 7):
    v = np.zeros(64, np.uint64)
    c = np.zeros(64, np.uint64)
    k = lib().orc_factorize(n, max_prime, _ptr(v), _ptr(c), 64)
    return [(int(v[i]), int(c[i])) for i in range(k)]


def bitreverse(n: int, factors):
    total = 1
    for v, c in factors:
        total *= v ** c
    vals = np.array([f[0] for f in factors] or [0], np.uint64)
    cnts = np.array([f[1] for f in factors] or [0], np.uint64)
    out = np.zeros(total, np.uint64)
    lib().orc_bitreverse(n, _ptr(vals), _ptr(cnts), len(factors), _ptr(out))
    return out


def bitreverse2inplace(ids, literal: bool = False):
    src = np.ascontiguousarray(ids, np.uint64)
    out = np.zeros_like(src)
    lib().orc_bitreverse2inplace(_ptr(src), src.size, _ptr(out), int(literal))
    return out


def chirp_index(n: int):
    out = np.zeros(n, np.uint64)
    lib().orc_chirp_index(n, _ptr(out))
    return out


def omega(n: int, dtype=np.complex128):
    out = np.zeros(n + 1, dtype)
    lib().orc_omega(_dt(out), n, _ptr(out))
    return out


def cfft1d_mode(n: int):
    m = ctypes.c_size_t(0)
    mode = lib().orc_cfft1d_mode(n, ctypes.byref(m))
    return ("chirpz" if mode else "mixed"), m.value


def _secs():
    return ctypes.c_double(0.0)


def cfft1d(x, method: str = "forward", nthreads: int = 1, timing: bool = False):
    """x: (..., N) complex64/complex128; each row is one transform."""
    x = np.ascontiguousarray(x)
    n = x.shape[-1]
    out = np.empty_like(x)
    s = _secs()
    _check(lib().orc_cfft1d(_dt(x), n, METHODS[method], _ptr(x), _ptr(out), x.size // max(n, 1) if n else 0,
                            nthreads, ctypes.byref(s)))
    return (out, s.value) if timing else out


def cfft2d(x, method: str = "forward", nthreads: int = 1, timing: bool = False):
    """x: (..., M, N) complex; row-major M x N per transform."""
    x = np.ascontiguousarray(x)
    m, n = x.shape[-2], x.shape[-1]
    out = np.empty_like(x)
    s = _secs()
    b = x.size // (m * n) if m * n else 0
    _check(lib().orc_cfft2d(_dt(x), m, n, METHODS[method], _ptr(x), _ptr(out), b, nthreads, ctypes.byref(s)))
    return (out, s.value) if timing else out


def rfft1d(x, method: str = "forward", nthreads: int = 1, timing: bool = False, n: int | None = None):
    """Forward methods: real (..., N) -> complex (..., N/2+1). Backward: the reverse."""
    x = np.ascontiguousarray(x)
    s = _secs()
    if METHODS[method] <= 3:
        n = x.shape[-1]
        b = x.size // n
        out = np.empty(x.shape[:-1] + (n // 2 + 1,), np.complex64 if x.dtype == np.float32 else np.complex128)
    else:
        h = x.shape[-1]
        n = n if n is not None else 2 * (h - 1)
        b = x.size // h
        out = np.empty(x.shape[:-1] + (n,), np.float32 if x.dtype == np.complex64 else np.float64)
        if h != n // 2 + 1:
            raise OracleError("invalid length")
    _check(lib().orc_rfft1d(_dt(x), n, METHODS[method], _ptr(x), _ptr(out), b, nthreads, ctypes.byref(s)))
    return (out, s.value) if timing else out


def dct1d(x, dct_type: int = 2, ortho: bool = False, method: str = "forward", nthreads: int = 1,
          timing: bool = False):
    x = np.ascontiguousarray(x)
    n = x.shape[-1]
    out = np.empty_like(x)
    s = _secs()
    _check(lib().orc_dct1d(_dt(x), dct_type, n, int(ortho), METHODS[method], _ptr(x), _ptr(out), x.size // n,
                           nthreads, ctypes.byref(s)))
    return (out, s.value) if timing else out


WINDOWS = {"sine": 0, "vorbis": 1, "custom": 2}


def mdct1d(x, n: int, window="sine", method: str = "forward", nthreads: int = 1, timing: bool = False):
    """Forward: (..., n) -> (..., n/2). Backward: (..., n/2) -> (..., n)."""
    x = np.ascontiguousarray(x)
    if isinstance(window, str):
        kind, win = WINDOWS[window], None
    else:
        kind, win = 2, np.ascontiguousarray(window, x.dtype)
    fwd = METHODS[method] <= 3
    if (x.shape[-1] != (n if fwd else n // 2)) or n % 4:
        raise OracleError("invalid length")
    b = x.size // x.shape[-1]
    out = np.empty(x.shape[:-1] + ((n // 2) if fwd else n,), x.dtype)
    s = _secs()
    _check(lib().orc_mdct1d(_dt(x), n, kind, _ptr(win) if win is not None else None, METHODS[method], _ptr(x),
                            _ptr(out), b, nthreads, ctypes.byref(s)))
    return (out, s.value) if timing else out
