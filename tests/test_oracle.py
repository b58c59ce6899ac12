"""The CPU oracle pinned to the reference's own test criteria (no GPU).

chfft's unit tests compare every transform with a naive DFT in the same
precision, absolute tolerance 1e-10 (f64) / 1e-2 (f32) (src/lib.rs:48-58),
plus round trips and invalid-length panics. The same identities run here on
the oracle at the reference's lengths (src/cfft1d.rs:566-603,
src/cfft2d.rs:454-489, src/rfft1d.rs:390-422, src/dct1d.rs:483-538,
src/mdct1d.rs:384-486). The reference's rand/XorShift stream is not
available, so inputs are numpy-seeded uniform [0, 1) like rng.gen::<T>().
Independent checks: numpy.fft at larger lengths, exact known answers, and the
bit-exact index arithmetic (factor lists, digit reversal, swap lists, chirp
indices).
"""
import numpy as np
import pytest

import oracle

EPS = {np.float64: 1e-10, np.float32: 1e-2}
CPLX = {np.float64: np.complex128, np.float32: np.complex64}


def naive_dft(x, sign=-1.0, scale=1.0):
    x = np.asarray(x, np.complex128)
    n = x.shape[-1]
    k = np.arange(n)
    w = np.exp(sign * 2j * np.pi * np.outer(k, k) / n)
    return (x @ w.T) * scale


def appro(expected, actual, dt):
    d = np.max(np.abs(np.asarray(expected, np.complex128) - np.asarray(actual, np.complex128)), initial=0.0)
    assert d <= EPS[dt], f"max abs error {d:.3e} > {EPS[dt]}"


def vecs(n, count, dt, complex_=True, seed=0):
    rng = np.random.default_rng(seed * 7919 + n)
    if complex_:
        return (rng.random((count, n)) + 1j * rng.random((count, n))).astype(CPLX[dt])
    return rng.random((count, n)).astype(dt)


# ---------------------------------------------------------------- CFft1D
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_cfft1d_reference_identities(dt):
    """test_with_source (src/cfft1d.rs:496-543) for N = 1..99, 10 vectors each."""
    for n in range(1, 100):
        x = vecs(n, 10, dt)
        xd = x.astype(np.complex128)
        exp = naive_dft(xd)
        for meth, sc in (("forward", 1.0), ("forward0", 1.0), ("forwardu", 1 / np.sqrt(n)), ("forwardn", 1.0 / n)):
            appro(exp * sc, oracle.cfft1d(x, meth), dt)
        appro(x, oracle.cfft1d(oracle.cfft1d(x, "forward"), "backward"), dt)
        appro(x, oracle.cfft1d(oracle.cfft1d(x, "forward0"), "backwardn"), dt)
        appro(x, oracle.cfft1d(oracle.cfft1d(x, "forwardu"), "backwardu"), dt)
        appro(x, oracle.cfft1d(oracle.cfft1d(x, "forwardn"), "backward0"), dt)
        # in-place forms equal the out-of-place ones
        appro(oracle.cfft1d(x, "forward0"), oracle.cfft1d(x, "forward0i"), dt)
        appro(x, oracle.cfft1d(oracle.cfft1d(x, "forwardn"), "backward0i"), dt)
        appro(oracle.cfft1d(x, "forwardu"), oracle.cfft1d(x, "forwardui"), dt)
        appro(x, oracle.cfft1d(oracle.cfft1d(x, "forwardu"), "backwardui"), dt)


def test_cfft1d_primes_f64():
    """f64_primes (src/cfft1d.rs:594-603): Chirp-Z for every prime below 100."""
    for n in [2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89, 97]:
        x = vecs(n, 10, np.float64)
        appro(naive_dft(x), oracle.cfft1d(x, "forward"), np.float64)
        appro(x, oracle.cfft1d(oracle.cfft1d(x, "forward"), "backward"), np.float64)


@pytest.mark.parametrize("n", [1000, 1009, 1024, 2048, 4096, 65536, 65521, 12345])
def test_cfft1d_against_numpy(n):
    x = vecs(n, 2, np.float64)
    y = oracle.cfft1d(x, "forward")
    assert np.linalg.norm(y - np.fft.fft(x)) / np.linalg.norm(np.fft.fft(x)) < 1e-13


def test_cfft1d_known_answer():
    """The doc example input (src/cfft1d.rs:43-44): its 4-point DFT is exact."""
    x = np.array([2 + 0j, 1 + 1j, 0 + 3j, 2 + 4j])
    np.testing.assert_array_equal(oracle.cfft1d(x, "forward"), [5 + 8j, -1 - 2j, -1 - 2j, 5 - 4j])
    np.testing.assert_array_equal(oracle.cfft1d(np.ones(8, np.complex128), "forward"), [8] + [0] * 7)
    imp = np.zeros(6, np.complex128)
    imp[0] = 1
    np.testing.assert_array_equal(oracle.cfft1d(imp, "forward"), np.ones(6))


# ---------------------------------------------------------------- CFft2D
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_cfft2d_reference_identities(dt):
    """src/cfft2d.rs:454-489: M, N in 1..9, forward against the 2-D DFT, backward round trip."""
    for m in range(1, 10):
        for n in range(1, 10):
            rng = np.random.default_rng(m * 10 + n)
            x = (rng.random((m, n)) + 1j * rng.random((m, n))).astype(CPLX[dt])
            appro(np.fft.fft2(x.astype(np.complex128)), oracle.cfft2d(x, "forward"), dt)
            appro(x, oracle.cfft2d(oracle.cfft2d(x, "forward"), "backward"), dt)


# ---------------------------------------------------------------- RFft1D
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_rfft1d_reference_identities(dt):
    """src/rfft1d.rs:390-402: N = 2..198 even; bins 0..=N/2 against the DFT."""
    for n in range(2, 200, 2):
        x = vecs(n, 4, dt, complex_=False)
        exp = naive_dft(x.astype(np.complex128))[:, : n // 2 + 1]
        for meth, sc in (("forward", 1.0), ("forwardu", 1 / np.sqrt(n)), ("forwardn", 1.0 / n)):
            appro(exp * sc, oracle.rfft1d(x, meth), dt)
        for fwd, bwd in (("forward", "backward"), ("forward0", "backwardn"), ("forwardu", "backwardu"),
                         ("forwardn", "backward0")):
            appro(x, oracle.rfft1d(oracle.rfft1d(x, fwd), bwd), dt)


# ---------------------------------------------------------------- Dct1D
def naive_dct2(x):
    n = x.shape[-1]
    j = np.arange(n)
    return x @ np.cos(np.pi / (2 * n) * np.outer(2 * j + 1, j))


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_dct1d_reference_identities(dt):
    """src/dct1d.rs:436-503: DCT-II against its definition, DCT-III round trips at three scalings."""
    for n in range(2, 200, 2):
        x = vecs(n, 3, dt, complex_=False)
        xd = x.astype(np.float64)
        appro(naive_dct2(xd) * np.sqrt(2 / n), oracle.dct1d(x, 2, False, "forwardu"), dt)
        appro(naive_dct2(xd) * 2 / n, oracle.dct1d(x, 2, False, "forwardn"), dt)
        appro(naive_dct2(xd), oracle.dct1d(x, 2, False, "forward0"), dt)
        appro(x, oracle.dct1d(oracle.dct1d(x, 2, False, "forwardu"), 3, False, "forwardu"), dt)
        appro(x, oracle.dct1d(oracle.dct1d(x, 2, False, "forwardn"), 3, False, "forward0"), dt)
        appro(x, oracle.dct1d(oracle.dct1d(x, 2, False, "forward0"), 3, False, "forwardn"), dt)


def test_dct1d_ortho_definition():
    """is_ortho scales the first INPUT value: DCT-II by sqrt(1/2) instead of 1 (src/dct1d.rs:220-224,
    :248-250), DCT-III by sqrt(1/2) instead of 1/2 (src/dct1d.rs:343-347, :366)."""
    for n in (2, 8, 30, 64):
        x = vecs(n, 2, np.float64, complex_=False)
        xs = x.copy()
        xs[:, 0] *= np.sqrt(0.5)
        appro(naive_dct2(xs) * np.sqrt(2 / n), oracle.dct1d(x, 2, True, "forwardu"), np.float64)
        j = np.arange(n)
        c = np.cos(np.pi / (2 * n) * np.outer(j, 2 * j + 1))  # [k, j]
        d3 = x[:, :1] * np.sqrt(0.5) + x[:, 1:] @ c[1:]
        appro(d3, oracle.dct1d(x, 3, True, "forward"), np.float64)


# ---------------------------------------------------------------- Mdct1D
def naive_mdct(x, w):
    n = x.shape[-1]
    k = np.arange(n)
    m = np.arange(n // 2)
    return (w * x) @ np.cos(np.pi / (2 * n) * np.outer(1 + n // 2 + 2 * k, 1 + 2 * m))


def naive_imdct(y, w):
    n = 2 * y.shape[-1]
    k = np.arange(n)
    m = np.arange(n // 2)
    return 4.0 * w / n * (y @ np.cos(np.pi / (2 * n) * np.outer(1 + 2 * m, 1 + n // 2 + 2 * k)))


def sine_w(n):
    return np.sin(np.pi * (np.arange(n) + 0.5) / n)


def vorbis_w(n):
    return np.sin(np.sin(np.pi * (np.arange(n) + 0.5) / n) ** 2 * np.pi * 0.5)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("window", ["sine", "vorbis", "custom"])
def test_mdct1d_reference_identities(dt, window):
    """src/mdct1d.rs:341-466: MDCT against its definition, IMDCT against the windowed naive IMDCT."""
    for i in range(1, 100, 2):
        n = i << 2
        w = vorbis_w(n) if window == "vorbis" else sine_w(n)
        x = vecs(n, 2, dt, complex_=False)
        win = w.astype(dt) if window == "custom" else window
        y = oracle.mdct1d(x, n, win, "forward")
        appro(naive_mdct(x.astype(np.float64), w), y, dt)
        appro(naive_imdct(y.astype(np.float64), w), oracle.mdct1d(y, n, win, "backward"), dt)
        yu = oracle.mdct1d(x, n, win, "forwardu")
        appro(naive_imdct(y.astype(np.float64), w), oracle.mdct1d(yu, n, win, "backwardu"), dt)


# ---------------------------------------------------------------- invalid lengths
def test_invalid_lengths():
    """src/rfft1d.rs:404-422, src/dct1d.rs:527-538, src/mdct1d.rs:468-486."""
    with pytest.raises(oracle.OracleError, match="invalid length"):
        oracle.rfft1d(np.zeros(11), "forward")
    with pytest.raises(oracle.OracleError, match="invalid length"):
        oracle.rfft1d(np.zeros(5, np.complex128), "backward", n=4)
    with pytest.raises(oracle.OracleError, match="invalid length"):
        oracle.dct1d(np.zeros(11), 2)
    with pytest.raises(oracle.OracleError, match="invalid length"):
        oracle.mdct1d(np.zeros(10), 10, "sine")
    with pytest.raises(oracle.OracleError, match="invalid length"):
        oracle.mdct1d(np.zeros(8), 8, "sine", "backward")


# ---------------------------------------------------------------- index arithmetic
def test_factorization_known_lists():
    """prime_factorization (src/prime_factorization.rs:66-113): chfft's idiosyncratic order."""
    assert oracle.factorize(1024) == [(4, 5)]
    assert oracle.factorize(1000) == [(2, 1), (5, 3), (4, 1)]
    assert oracle.factorize(2048) == [(2, 1), (4, 5)]
    assert oracle.factorize(4096) == [(4, 6)]
    assert oracle.factorize(1 << 20) == [(4, 10)]
    assert oracle.factorize(512) == [(2, 1), (4, 4)]
    assert oracle.factorize(60) == [(3, 1), (5, 1), (4, 1)]
    assert oracle.factorize(140) == [(4, 1), (5, 1), (7, 1)]
    assert oracle.factorize(1009) == []
    assert oracle.factorize(1) == []
    assert oracle.factorize(22) == []  # 11 > 7: Chirp-Z


def test_digit_reversal_known():
    """calc_bitreverse (src/precompute_utils.rs:70-91): N = 8 with factors [2, 4]."""
    np.testing.assert_array_equal(oracle.bitreverse(8, [(2, 1), (4, 1)]), [0, 4, 1, 5, 2, 6, 3, 7])


def test_swap_list_fast_equals_literal():
    """calc_bitreverse2inplace (src/precompute_utils.rs:93-104): O(n) form == literal O(n^2) form."""
    for n in list(range(1, 200)) + [1000, 1024, 2048]:
        f = oracle.factorize(n)
        if not f:
            continue
        ids = oracle.bitreverse(n, f)
        np.testing.assert_array_equal(oracle.bitreverse2inplace(ids), oracle.bitreverse2inplace(ids, literal=True))


def test_chirp_index():
    """(i*i) % 2N in integers (src/cfft1d.rs:123-128)."""
    for n in (11, 1009, 65521):
        i = np.arange(n, dtype=np.uint64)
        np.testing.assert_array_equal(oracle.chirp_index(n), (i * i) % np.uint64(2 * n))


def test_omega_table_symmetry():
    """calc_omega (src/precompute_utils.rs:23-68): len+1 entries, quarter / half turn symmetry, omega[N] = 1."""
    for n in (4, 6, 7, 16, 1000, 1009):
        o = oracle.omega(n)
        assert o.shape == (n + 1,)
        assert o[0] == 1 and o[n] == 1
        np.testing.assert_allclose(o[:n], np.exp(-2j * np.pi * np.arange(n) / n), atol=1e-15)


@pytest.mark.parametrize("n", [16, 64, 1000, 2048])
def test_bench_checkers_agree_with_the_oracle(n):
    """bench.py checks its results against FP64 numpy / scipy (the oracle is
    only timed there): chfft's DCT-II / DCT-III are half of scipy's types 2
    / 3, and its MDCT is bench.mdct_def, the sine-windowed definition."""
    import scipy.fft

    import bench

    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, n)
    for t in (2, 3):
        ref = oracle.dct1d(x, t, False, "forward")
        got = scipy.fft.dct(x, type=t) / 2
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-13, t
    if n % 4 == 0:
        ref = oracle.mdct1d(x, n, "sine", "forward")
        assert np.linalg.norm(bench.mdct_def(x, n) - ref) / np.linalg.norm(ref) < 1e-12
    z = x + 1j * rng.uniform(-1, 1, n)
    assert np.linalg.norm(np.fft.ifft(np.fft.fft(z)) - oracle.cfft1d(oracle.cfft1d(z, "forward"), "backward")) < 1e-12
