"""The C ABI without a GPU: the library loads, exports every entry point that
include/chfft_gpu.h declares, and its host-only index arithmetic is
bit-exact with the oracle's restatement of chfft's plan code."""
import os
import re

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "chfft_gpu.h")


@pytest.fixture(scope="module")
def cg():
    import chfft_gb300

    if not os.path.exists(chfft_gb300.LIB_PATH):
        from chfft_gb300 import _build

        _build.build()
    chfft_gb300.lib()
    return chfft_gb300


def declared_symbols():
    text = open(HEADER).read()
    return re.findall(r"CHFFT_API\s+[\w\s\*]+?\b(chfft_\w+)\s*\(", text)


def test_header_declares_the_api():
    names = declared_symbols()
    for must in ("chfft_cfft1d_create", "chfft_cfft2d_create", "chfft_rfft1d_create", "chfft_dct1d_create",
                 "chfft_mdct1d_create", "chfft_execute", "chfft_execute_device", "chfft_plan_destroy",
                 "chfft_execute_device_noalloc"):
        assert must in names


def test_library_exports_every_declared_symbol(cg):
    lib = cg.lib()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_status_strings(cg):
    assert "sm_103a" in cg.version()
    assert cg.lib().chfft_status_string(1) == b"invalid length"


def test_factorize_bit_exact(cg):
    """chfft_factorize == prime_factorization (src/prime_factorization.rs:66-113) for 1..6000 and large N."""
    for n in list(range(1, 6000)) + [1 << 20, 3 ** 12, 5 ** 8, 7 ** 7, 2 * 3 * 5 * 7 * 11 * 13, 65521 * 4, 1000003]:
        for mx in (7, 5, 3, 13):
            assert cg.factorize(n, mx) == oracle.factorize(n, mx), (n, mx)


def test_digit_reversal_bit_exact(cg):
    """chfft_digit_reversal == calc_bitreverse (src/precompute_utils.rs:70-91)."""
    for n in (8, 60, 140, 1000, 1024, 2048, 4096, 5040):
        f = oracle.factorize(n)
        np.testing.assert_array_equal(cg.digit_reversal(f), oracle.bitreverse(n, f))
    # Chirp-Z's power-of-two list (src/cfft1d.rs:163-175)
    for lv in range(1, 14):
        f = [(2, lv & 1), (4, lv >> 1)]
        np.testing.assert_array_equal(cg.digit_reversal(f), oracle.bitreverse(1, f))


def test_swap_list_bit_exact(cg):
    """chfft_swap_list == calc_bitreverse2inplace (src/precompute_utils.rs:93-104)."""
    for n in (8, 60, 140, 1000, 1024, 2048, 4096):
        ids = oracle.bitreverse(n, oracle.factorize(n))
        np.testing.assert_array_equal(cg.swap_list(ids), oracle.bitreverse2inplace(ids, literal=n <= 1024))


def test_invalid_lengths_need_no_gpu(cg):
    """Constructor panics are decided on the host (src/rfft1d.rs:75, src/dct1d.rs:55, src/mdct1d.rs:103)."""
    with pytest.raises(cg.InvalidLength, match="invalid length"):
        cg.RFft1D(11)
    with pytest.raises(cg.InvalidLength, match="invalid length"):
        cg.Dct1D(cg.DctType.Two, 11, False)
    with pytest.raises(cg.InvalidLength, match="invalid length"):
        cg.Mdct1D.with_sine(10)


def test_plan_compiler_query_is_safe_without_gpu(cg):
    ok = cg.plan_compiler_available()
    assert ok in (True, False)
    if not ok:
        assert cg.lib().chfft_last_error()
