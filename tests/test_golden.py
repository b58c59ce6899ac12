"""Golden fixtures (tests/golden/golden.npz, made by tests/golden/make_golden.py).

CPU: the oracle still reproduces its recorded outputs (libm may differ in the
last bit between hosts, hence the tight relative tolerance rather than
equality). GPU: the CUDA path through the C ABI matches them within the
parity tolerances (f64 1e-12, f32 5e-6 relative L2).
"""
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = np.load(os.path.join(HERE, "golden", "golden.npz"))
KEYS = sorted({k.split("|")[0] for k in GOLDEN.files})


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run(key, x, impl):
    kind, tag, *rest = key.split("/")
    if impl == "oracle":
        if kind == "cfft1d":
            return oracle.cfft1d(x, rest[1])
        if kind == "cfft2d":
            return oracle.cfft2d(x, rest[1])
        if kind == "rfft1d":
            return oracle.rfft1d(x, rest[1])
        if kind == "dct1d":
            return oracle.dct1d(x, int(rest[1]), bool(int(rest[2])), "forward")
        n, w, m = int(rest[0]), rest[1], rest[2]
        return oracle.mdct1d(x, n, w, m)
    import chfft_gb300 as cg

    dt = np.float64 if tag == "f64" else np.float32
    if kind == "cfft1d":
        return cg.CFft1D.with_len(int(rest[0]), dt).execute_batch(rest[1], x)
    if kind == "cfft2d":
        m, n = map(int, rest[0].split("x"))
        return getattr(cg.CFft2D.with_len(m, n, dt), rest[1])(x)
    if kind == "rfft1d":
        return cg.RFft1D(int(rest[0]), dt).execute_batch(rest[1], x)
    if kind == "dct1d":
        p = cg.Dct1D(cg.DctType(int(rest[1])), int(rest[0]), bool(int(rest[2])), dt)
        return p.execute_batch("forward", x)
    n, w, m = int(rest[0]), rest[1], rest[2]
    p = cg.Mdct1D.with_sine(n, dt) if w == "sine" else cg.Mdct1D.with_vorbis(n, dt)
    return p.execute_batch(m, x)


@pytest.mark.parametrize("key", KEYS)
def test_oracle_reproduces_golden(key):
    x, y = GOLDEN[key + "|in"], GOLDEN[key + "|out"]
    tol = 1e-13 if "/f64/" in key else 2e-6
    assert rel(run(key, x, "oracle"), y) <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("key", KEYS)
def test_gpu_matches_golden(key):
    pytest.importorskip("chfft_gb300")
    x, y = GOLDEN[key + "|in"], GOLDEN[key + "|out"]
    tol = 1e-12 if "/f64/" in key else 5e-6
    assert rel(run(key, x, "gpu"), y) <= tol
