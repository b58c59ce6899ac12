"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Restates the reference's unit tests (src/cfft1d.rs:470-604, src/cfft2d.rs:
378-489, src/rfft1d.rs:315-423, src/dct1d.rs:412-539, src/mdct1d.rs:294-487)
with the oracle as the expected value: the same lengths, the same method /
round-trip identities, the same invalid-length panics. Tolerances:
f64 relative L2 <= 1e-12 against the oracle's f64 output; f32 relative L2
<= 5e-6 against the oracle's f64 output (the GPU's f32 tables are rounded
from FP64) and, as in the reference, absolute error <= 1e-2.
"""
import numpy as np
import pytest

import oracle

cg = pytest.importorskip("chfft_gb300")

pytestmark = pytest.mark.gpu

TOL = {np.float64: 1e-12, np.float32: 5e-6}
CPLX = {np.float64: np.complex128, np.float32: np.complex64}


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a))


def close(actual, expected, dt):
    r = rel(actual, expected)
    assert r <= TOL[dt], f"rel-L2 {r:.3e} > {TOL[dt]:.0e}"
    if dt == np.float32:
        assert np.max(np.abs(np.asarray(actual, np.complex128) - expected), initial=0) <= 1e-2


def rng_vectors(n, count=10, seed=0, complex_=True):
    rng = np.random.default_rng(seed + 1000 * n)
    if complex_:
        return rng.random((count, n)) + 1j * rng.random((count, n))
    return rng.random((count, n))


DTYPES = [np.float64, np.float32]


# ---------------------------------------------------------------- CFft1D
SCALED = [("forward", "backward"), ("forward0", "backwardn"), ("forwardu", "backwardu"), ("forwardn", "backward0")]


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("use_new", [False, True])
def test_cfft1d_lengths_1_to_99(dt, use_new):
    """f64_new / f32_new / f64_with_len / f32_with_len (src/cfft1d.rs:566-592)."""
    plan = cg.CFft1D.new(dt) if use_new else None
    for n in range(1, 100):
        p = plan if use_new else cg.CFft1D.with_len(n, dt)
        for x in rng_vectors(n, count=3):
            xs = x.astype(CPLX[dt])
            xd = xs.astype(np.complex128)
            for fwd, bwd in SCALED:
                exp = oracle.cfft1d(xd, fwd)
                act = p.__getattribute__(fwd)(xs)
                close(act, exp, dt)
                close(p.__getattribute__(bwd)(act), xd, dt)
            # in-place variants equal the out-of-place ones
            y = xs.copy()
            p.forward0i(y)
            close(y, oracle.cfft1d(xd, "forward0"), dt)
            y = p.forwardn(xs)
            p.backward0i(y)
            close(y, xd, dt)
            y = xs.copy()
            p.forwardui(y)
            close(y, oracle.cfft1d(xd, "forwardu"), dt)
            p.backwardui(y)
            close(y, xd, dt)


def test_cfft1d_primes_reuse_plan():
    """f64_primes (src/cfft1d.rs:594-603): one plan re-planned across primes."""
    p = cg.CFft1D.new(np.float64)
    for n in [2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89, 97]:
        for x in rng_vectors(n, count=2):
            close(p.forward(x), oracle.cfft1d(x, "forward"), np.float64)
            close(p.backward(p.forward(x)), x, np.float64)


@pytest.mark.parametrize("dt", DTYPES)
def test_cfft1d_batch_matches_single(dt):
    for n in (16, 60, 128, 1000, 1009, 4096):
        x = rng_vectors(n, count=5).astype(CPLX[dt])
        p = cg.CFft1D.with_len(n, dt)
        yb = p.execute_batch("forward", x)
        exp = oracle.cfft1d(x.astype(np.complex128), "forward")
        close(yb, exp, dt)
        for i in range(5):
            np.testing.assert_array_equal(yb[i], p.forward(x[i]))


# ---------------------------------------------------------------- CFft2D
@pytest.mark.parametrize("dt", DTYPES)
def test_cfft2d_small(dt):
    """src/cfft2d.rs:454-489: M, N in 1..9, forward then backward."""
    for m in range(1, 10):
        for n in range(1, 10):
            p = cg.CFft2D.with_len(m, n, dt)
            rng = np.random.default_rng(m * 31 + n)
            x = (rng.random((m, n)) + 1j * rng.random((m, n))).astype(CPLX[dt])
            xd = x.astype(np.complex128)
            y = p.forward(x)
            close(y, oracle.cfft2d(xd, "forward"), dt)
            close(p.backward(y), xd, dt)
            for meth in ("forwardu", "forwardn", "backward0", "backwardu"):
                close(p.__getattribute__(meth)(x), oracle.cfft2d(xd, meth), dt)


# ---------------------------------------------------------------- RFft1D
@pytest.mark.parametrize("dt", DTYPES)
def test_rfft1d_even_lengths(dt):
    """src/rfft1d.rs:390-402: N = 2..198 even, all scalings round trip."""
    for n in range(2, 200, 2):
        p = cg.RFft1D(n, dt)
        for x in rng_vectors(n, count=2, complex_=False):
            xs = x.astype(dt)
            xd = xs.astype(np.float64)
            for fwd, bwd in SCALED + [("forward", "backwardn")]:
                act = p.__getattribute__(fwd)(xs)
                close(act, oracle.rfft1d(xd, fwd), dt)
                close(p.__getattribute__(bwd)(act), xd, dt)


def test_rfft1d_invalid_length():
    """invalid_length / invalid_length_convert(_back) (src/rfft1d.rs:404-422)."""
    with pytest.raises(cg.InvalidLength, match="invalid length"):
        cg.RFft1D(11)
    p = cg.RFft1D(4)
    with pytest.raises(cg.InvalidLength, match="invalid length"):
        p.forward(np.arange(5, dtype=np.float64))
    with pytest.raises(cg.InvalidLength, match="invalid length"):
        p.backward(np.arange(5, dtype=np.complex128))


# ---------------------------------------------------------------- Dct1D
def _dct_pair_checks(d2, d3, x, dt):
    xd = x.astype(np.float64)
    for m2, m3 in (("forwardu", "forwardu"), ("forwardn", "forward0"), ("forward0", "forwardn")):
        y = d2.__getattribute__(m2)(x)
        close(y, oracle.dct1d(xd, 2, False, m2), dt)
        close(d3.__getattribute__(m3)(y), xd, dt)


@pytest.mark.parametrize("dt", DTYPES)
def test_dct1d_even_lengths(dt):
    """f64_new / f32_new (src/dct1d.rs:483-503): DCT-II <-> DCT-III round trips."""
    for n in range(2, 200, 2):
        d2 = cg.Dct1D(cg.DctType.Two, n, False, dt)
        d3 = cg.Dct1D(cg.DctType.Three, n, False, dt)
        for x in rng_vectors(n, count=2, complex_=False):
            _dct_pair_checks(d2, d3, x.astype(dt), dt)


@pytest.mark.parametrize("dt", DTYPES)
def test_dct1d_setup_and_ortho(dt):
    """f64_with_setup / f32_with_setup (src/dct1d.rs:505-525) and the ortho flag."""
    for i in range(1, 40):
        d2 = cg.Dct1D(cg.DctType.Two if dt == np.float64 else cg.DctType.Three, i << 2, True, dt)
        d3 = cg.Dct1D(cg.DctType.Two if dt == np.float64 else cg.DctType.Three, i << 2, True, dt)
        d2.setup(cg.DctType.Two, i << 1, False)
        d3.setup(cg.DctType.Three, i << 1, False)
        for x in rng_vectors(i << 1, count=2, complex_=False):
            _dct_pair_checks(d2, d3, x.astype(dt), dt)
    for n in (2, 6, 8, 30, 64):
        x = rng_vectors(n, count=1, complex_=False)[0]
        for t in (2, 3):
            p = cg.Dct1D(cg.DctType(t), n, True, dt)
            for meth in ("forward", "forwardu", "forwardn"):
                close(p.__getattribute__(meth)(x.astype(dt)), oracle.dct1d(x, t, True, meth), dt)


def test_dct1d_invalid_length():
    """src/dct1d.rs:527-538."""
    with pytest.raises(cg.InvalidLength, match="invalid length"):
        cg.Dct1D(cg.DctType.Two, 11, False)
    p = cg.Dct1D(cg.DctType.Two, 8, False)
    with pytest.raises(cg.InvalidLength, match="invalid length"):
        p.forward(np.arange(10, dtype=np.float64))


# ---------------------------------------------------------------- Mdct1D
@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("window", ["sine", "vorbis", "custom"])
def test_mdct1d_lengths(dt, window):
    """src/mdct1d.rs:384-466: N = 4..396 step 4, sine / vorbis / custom windows."""
    for i in range(1, 100, 3):
        n = i << 2
        if window == "sine":
            p = cg.Mdct1D.with_sine(n, dt)
        elif window == "vorbis":
            p = cg.Mdct1D.with_vorbis(n, dt)
        else:
            p = cg.Mdct1D(cg.sine_window, n, dt)
        wname = "vorbis" if window == "vorbis" else "sine"
        for x in rng_vectors(n, count=2, complex_=False):
            xs = x.astype(dt)
            xd = xs.astype(np.float64)
            y = p.forward(xs)
            close(y, oracle.mdct1d(xd, n, wname, "forward"), dt)
            yd = np.asarray(y, np.float64)
            close(p.backward(y), oracle.mdct1d(yd, n, wname, "backward"), dt)
            yu = p.forwardu(xs)
            close(yu, oracle.mdct1d(xd, n, wname, "forwardu"), dt)
            close(p.backwardu(yu), oracle.mdct1d(np.asarray(yu, np.float64), n, wname, "backwardu"), dt)


@pytest.mark.parametrize("dt", DTYPES)
def test_mdct1d_setup_shrink(dt):
    """f32_with_setup / f64_with_setup (src/mdct1d.rs:450-466): 16i -> 4i."""
    for i in range(1, 30, 4):
        p = cg.Mdct1D(cg.sine_window, i << 4, dt)
        p.setup(i << 2)
        x = rng_vectors(i << 2, count=1, complex_=False)[0]
        close(p.forward(x.astype(dt)), oracle.mdct1d(x, i << 2, "sine", "forward"), dt)


def test_mdct1d_invalid_length():
    """src/mdct1d.rs:468-486."""
    with pytest.raises(cg.InvalidLength, match="invalid length"):
        cg.Mdct1D.with_sine(10)
    p = cg.Mdct1D.with_sine(8)
    with pytest.raises(cg.InvalidLength, match="invalid length"):
        p.forward(np.arange(10, dtype=np.float64))
    with pytest.raises(cg.InvalidLength, match="invalid length"):
        p.backward(np.arange(8, dtype=np.float64))


# ---------------------------------------------------------------- configurations
def test_config_cfft1d_f64_1024():
    """N = 1024 f64 forward + backward, re/im uniform[-1, 1): rel-L2 <= 1e-12."""
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, 1024) + 1j * rng.uniform(-1, 1, 1024)
    p = cg.CFft1D.with_len(1024, np.float64)
    y = p.forward(x)
    assert rel(y, oracle.cfft1d(x, "forward")) <= 1e-12
    assert rel(p.backward(y), oracle.cfft1d(oracle.cfft1d(x, "forward"), "backward")) <= 1e-12


@pytest.mark.parametrize("n", [1000, 1009])
def test_config_batch_f32(n):
    """4096 transforms of N = 1000 (mixed radix) and N = 1009 (Bluestein), f32, N(0,1)."""
    rng = np.random.default_rng(2)
    x = (rng.standard_normal((4096, n)) + 1j * rng.standard_normal((4096, n))).astype(np.complex64)
    p = cg.CFft1D.with_len(n, np.float32)
    y = p.execute_batch("forward", x)
    sel = slice(0, 4096, 97)
    exp = oracle.cfft1d(x[sel].astype(np.complex128), "forward")
    assert rel(y[sel], exp) <= 5e-6


def test_config_cfft2d_2048_f32():
    """CFft2D 2048 x 2048 f32, uniform[-1, 1), against numpy's FP64 FFT."""
    rng = np.random.default_rng(3)
    x = (rng.uniform(-1, 1, (2048, 2048)) + 1j * rng.uniform(-1, 1, (2048, 2048))).astype(np.complex64)
    p = cg.CFft2D.with_len(2048, 2048, np.float32)
    y = p.forward(x)
    assert rel(y, np.fft.fft2(x.astype(np.complex128))) <= 5e-6


# ---------------------------------------------------------------- beyond one CTA (four-step)
@pytest.mark.parametrize("n,dt", [(32768, np.float32), (65536, np.float32), (1 << 20, np.float32), (16384, np.float64),
                                  (3 * 5 * 7 * 2 ** 9, np.float32), (65521, np.float32), (20011, np.float64)])
def test_cfft1d_four_step(n, dt):
    """Lengths beyond one CTA: four-step (7-smooth) or four-step Bluestein (primes)."""
    rng = np.random.default_rng(n)
    x = (rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))).astype(CPLX[dt])
    p = cg.CFft1D.with_len(n, dt)
    info = p.info()
    assert info.algorithm in (2, 3)
    ref = np.fft.fft(x.astype(np.complex128), axis=-1)
    tol = 1e-11 if dt == np.float64 else 5e-6
    for meth, r in (("forward", ref), ("forwardn", ref / n)):
        assert rel(p.execute_batch(meth, x), r) <= tol
    y = p.execute_batch("forward", x)
    assert rel(p.execute_batch("backward", y), x) <= tol
    assert rel(p.forward(x[0]), ref[0]) <= tol


def test_config_1m_x64_f32():
    """N = 2^20 x 64 f32, N(0,1) with 1% of entries x 1e3: rel-L2 against FP64."""
    n, b = 1 << 20, 64
    rng = np.random.default_rng(4)
    x = (rng.standard_normal((b, n), dtype=np.float32) + 1j * rng.standard_normal((b, n), dtype=np.float32))
    spikes = rng.random((b, n)) < 0.01
    x[spikes] *= 1e3
    x = x.astype(np.complex64)
    p = cg.CFft1D.with_len(n, np.float32)
    y = p.execute_batch("forward", x)
    for i in (0, 31, 63):
        assert rel(y[i], np.fft.fft(x[i].astype(np.complex128))) <= 1e-6


# ---------------------------------------------------------------- index work on the GPU
@pytest.mark.parametrize("n", [1009, 20011, 65521, 65537, 99991, 1000003])
def test_chirp_index_device_bit_exact(n):
    """chfft_chirp_index_device: (i*i) % 2N for i < N (src/cfft1d.rs:123-128),
    bit for bit against the oracle; N = 65537 and above overflow 32 bits."""
    torch = pytest.importorskip("torch")
    d = torch.zeros(n, dtype=torch.int64, device="cuda")
    cg.chirp_index_device(n, d.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d.cpu().numpy().view(np.uint64), oracle.chirp_index(n))


def test_config_4096x16384_fp32_outliers_every_row():
    """N = 4096 x 16384 f32, N(0,1) with 1% of entries x 1e3: every row
    within 1e-6 rel-L2 of numpy's FP64 FFT (the precision configuration)."""
    n, b = 4096, 16384
    rng = np.random.default_rng(5)
    x = rng.standard_normal((b, n), dtype=np.float32) + 1j * rng.standard_normal((b, n), dtype=np.float32)
    x[rng.random((b, n)) < 0.01] *= 1e3
    x = x.astype(np.complex64)
    y = cg.CFft1D.with_len(n, np.float32).execute_batch("forward", x)
    for lo in range(0, b, 2048):
        ref = np.fft.fft(x[lo:lo + 2048].astype(np.complex128), axis=-1)
        err = np.linalg.norm(y[lo:lo + 2048] - ref, axis=-1) / np.linalg.norm(ref, axis=-1)
        assert err.max() <= 1e-6, (lo, float(err.max()))


# ---------------------------------------------------------------- Rader
@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n", [17, 31, 1009, 7681, 12289])
def test_rader_lengths(n, dt):
    """With CHFFT_RADER=1, primes whose n - 1 is 7-smooth run Rader's
    algorithm (two (n-1)-point FFTs) instead of Chirp-Z; same results as the
    oracle's Chirp-Z (src/chirpz.rs) within the tolerances, every method, and
    the same as this library's Chirp-Z path (the default)."""
    import os

    os.environ["CHFFT_RADER"] = "1"
    try:
        p = cg.CFft1D.with_len(n, dt)
    finally:
        os.environ.pop("CHFFT_RADER", None)
    info = p.info()
    if dt == np.float64 and n >= 7681:
        assert info.algorithm in (1, 3)  # tile and staged row do not fit a CTA in f64: Chirp-Z
    else:
        assert info.algorithm == 4
    x = rng_vectors(n, count=3).astype(CPLX[dt])
    xd = x.astype(np.complex128)
    for fwd, bwd in SCALED:
        y = p.execute_batch(fwd, x)
        for i in range(3):
            close(y[i], oracle.cfft1d(xd[i], fwd), dt)
        z = p.execute_batch(bwd, y)
        close(z, xd, dt)
    y = x.copy()
    p.forward0i(y[0])
    close(y[0], oracle.cfft1d(xd[0], "forward0"), dt)
    q = cg.CFft1D.with_len(n, dt)
    assert q.info().algorithm in (1, 3)
    close(q.execute_batch("forward", x), p.execute_batch("forward", x).astype(np.complex128), dt)
