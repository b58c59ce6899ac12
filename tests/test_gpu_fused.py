"""GPU: the fused four-step launch (k_fourstep_fused) against the two-launch path.

Both run the same specialised column and row cores with the same modes, so
the fused launch must reproduce the two-launch output bit for bit; both are
also checked against numpy's FP64 FFT. CHFFT_FUSED="lead,ring,hints" selects
the fused launch (ring slots of intermediates, pass-A transforms ahead of
pass B, L2 eviction hints); lead/ring larger than the batch are clamped.
"""
import os

import numpy as np
import pytest

cg = pytest.importorskip("chfft_gb300")

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run(p, meth, x, fused):
    old = os.environ.pop("CHFFT_FUSED", None)
    try:
        if fused:
            os.environ["CHFFT_FUSED"] = fused
        return p.execute_batch(meth, x)
    finally:
        os.environ.pop("CHFFT_FUSED", None)
        if old is not None:
            os.environ["CHFFT_FUSED"] = old


@pytest.mark.parametrize("n,batch,fused", [
    (1 << 20, 8, "2,4,1"),
    (1 << 20, 1, "2,4,1"),
    (65536, 33, "1,2,0"),
    (3 * 5 * 7 * 2 ** 9, 5, "3,3,1"),
    (1 << 16, 12, "4,5,1"),
])
def test_fused_matches_two_launch(n, batch, fused):
    rng = np.random.default_rng(n + batch)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    p = cg.CFft1D.with_len(n, np.float32)
    assert p.info().algorithm == 2  # plain four-step
    ref = np.fft.fft(x.astype(np.complex128), axis=-1)
    for meth, r in (("forward", ref), ("forwardn", ref / n)):
        two = run(p, meth, x, None)
        one = run(p, meth, x, fused)
        assert np.array_equal(one, two), f"{meth}: fused differs from two-launch ({rel(one, two):.2e})"
        assert rel(one, r) <= 5e-6
    y = run(p, "backward", ref.astype(np.complex64), fused)
    assert rel(y, x) <= 5e-6  # backward carries the 1/N


def test_fused_device_pointers_repeat():
    """Device buffers, repeated launches on one plan (the ticket and tile
    counters are cleared before every launch)."""
    torch = pytest.importorskip("torch")
    n, b = 1 << 18, 16
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(b, n, dtype=torch.complex64, device="cuda", generator=g)
    y0 = torch.empty_like(x)
    y1 = torch.empty_like(x)
    p = cg.CFft1D.with_len(n, np.float32)
    p.execute_device("forward", x.data_ptr(), y0.data_ptr(), b)
    os.environ["CHFFT_FUSED"] = "2,3,1"
    try:
        for _ in range(3):
            y1.zero_()
            p.execute_device("forward", x.data_ptr(), y1.data_ptr(), b)
            torch.cuda.synchronize()
            assert torch.equal(y0, y1)
    finally:
        os.environ.pop("CHFFT_FUSED", None)
