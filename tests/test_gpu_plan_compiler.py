"""Plan-time specialised kernels (NVRTC) against the library kernels.

The same kernel templates are instantiated with compile-time stages
(CHFFT_JIT=1) or run-time stages (CHFFT_JIT=0); both must match the oracle
and each other for every kind, dtype and core (mixed radix / Bluestein).
"""
import os

import numpy as np
import pytest

import oracle

cg = pytest.importorskip("chfft_gb300")

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture
def jit_env():
    old = os.environ.get("CHFFT_JIT")
    yield
    if old is None:
        os.environ.pop("CHFFT_JIT", None)
    else:
        os.environ["CHFFT_JIT"] = old


def run_both(fn):
    os.environ["CHFFT_JIT"] = "0"
    a = fn()
    os.environ["CHFFT_JIT"] = "1"
    b = fn()
    return a, b


def test_plan_compiler_available():
    assert cg.plan_compiler_available(), cg.lib().chfft_last_error().decode()


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n", [8, 60, 128, 1000, 1009, 2048, 4096, 97, 4000])
def test_cfft1d_specialised_matches(jit_env, dt, n):
    rng = np.random.default_rng(n)
    x = (rng.standard_normal((64, n)) + 1j * rng.standard_normal((64, n))).astype(np.complex64 if dt == np.float32
                                                                                   else np.complex128)
    p = cg.CFft1D.with_len(n, dt)
    before = cg.plan_compiler_cache_size()
    for meth in ("forward", "backwardu"):
        a, b = run_both(lambda: p.execute_batch(meth, x))
        tol = 1e-12 if dt == np.float64 else 5e-6
        assert rel(b, a) <= tol
        assert rel(b, oracle.cfft1d(x.astype(np.complex128), meth)) <= tol
    assert cg.plan_compiler_cache_size() >= max(before, 1)  # an earlier batch may have compiled it


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_real_kinds_specialised_match(jit_env, dt):
    rng = np.random.default_rng(5)
    tol = 1e-12 if dt == np.float64 else 5e-6
    for n in (64, 1000, 2048, 22):
        x = rng.uniform(-1, 1, (32, n)).astype(dt)
        r = cg.RFft1D(n, dt)
        a, b = run_both(lambda: r.execute_batch("forward", x))
        assert rel(b, a) <= tol and rel(b, oracle.rfft1d(x.astype(np.float64), "forward")) <= tol
        s = a.astype(np.complex128)
        a, b = run_both(lambda: r.execute_batch("backward", s.astype(a.dtype)))
        assert rel(b, a) <= tol
        for t in (cg.DctType.Two, cg.DctType.Three):
            d = cg.Dct1D(t, n, False, dt)
            a, b = run_both(lambda: d.execute_batch("forward", x))
            assert rel(b, a) <= tol and rel(b, oracle.dct1d(x.astype(np.float64), int(t))) <= tol
    for n in (2048, 64, 44):
        x = rng.uniform(-1, 1, (32, n)).astype(dt)
        m = cg.Mdct1D.with_sine(n, dt)
        a, b = run_both(lambda: m.execute_batch("forward", x))
        assert rel(b, a) <= tol and rel(b, oracle.mdct1d(x.astype(np.float64), n, "sine")) <= tol
        y = a
        a, b = run_both(lambda: m.execute_batch("backward", y))
        assert rel(b, a) <= tol


def test_cfft2d_specialised_matches(jit_env):
    rng = np.random.default_rng(9)
    for m, n in ((2048, 2048), (64, 1000), (1009, 16)):
        x = (rng.uniform(-1, 1, (m, n)) + 1j * rng.uniform(-1, 1, (m, n))).astype(np.complex64)
        p = cg.CFft2D.with_len(m, n, np.float32)
        a, b = run_both(lambda: p.forward(x))
        assert rel(b, a) <= 5e-6
        assert rel(b, np.fft.fft2(x.astype(np.complex128))) <= 5e-6
