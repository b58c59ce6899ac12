"""GPU: radix-16 passes on the tensor cores (tcgen05, FP32 accumulation).

f32 C2C through the tensor-core precision knob against float64 numpy.fft:
FP16 hi+lo and BF16 hi+mid+lo must stay at FP32-path accuracy (relative L2
<= 2e-6 on N(0,1) data, <= 5e-6 with 1% entries scaled by 1e3); BF16 hi+lo
carries 16 significant bits (relative L2 <= 1e-4). The FP32 path's own error
is printed beside them.
"""
import numpy as np
import pytest

cg = pytest.importorskip("chfft_gb300")
from chfft_gb300 import tuning  # noqa: E402

pytestmark = pytest.mark.gpu

BOUND = {1: 2e-6, 2: 1e-4, 3: 2e-6}
BOUND_SPIKY = {1: 5e-6, 2: 1e-4, 3: 5e-6}


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.complex128) - b) / np.linalg.norm(b))


def data(n, batch, seed, spiky=False):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))
    if spiky:
        x[rng.random((batch, n)) < 0.01] *= 1e3
    return x.astype(np.complex64)


def config(prec):
    c = tuning.default_config()
    c.tc_precision = prec
    return c


@pytest.mark.parametrize("prec", [1, 2, 3])
@pytest.mark.parametrize("n,batch", [(4096, 24), (256, 40), (1024, 12), (16, 300), (512, 9), (2048, 5),
                                     (65536, 2)])
def test_tc_rows_match_fp64(prec, n, batch):
    x = data(n, batch, n + prec)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    plan = cg.CFft1D.with_len(n, np.float32)
    base = rel(plan.execute_batch("forward", x), ref)
    tuning.set_config(plan, config(prec))
    y = plan.execute_batch("forward", x)
    r = rel(y, ref)
    print(f"n={n} prec={prec}: tc {r:.2e}, fp32 {base:.2e}")
    assert r <= BOUND[prec]
    # Backward (conjugation trick) with its 1/N scale.
    xb = plan.execute_batch("backward", y)
    assert rel(xb, x.astype(np.complex128)) <= 2 * BOUND[prec]


@pytest.mark.parametrize("prec", [1, 3])
def test_tc_dynamic_range(prec):
    n, batch = 4096, 64
    x = data(n, batch, 99, spiky=True)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    plan = cg.CFft1D.with_len(n, np.float32)
    tuning.set_config(plan, config(prec))
    assert rel(plan.execute_batch("forward", x), ref) <= BOUND_SPIKY[prec]


@pytest.mark.parametrize("prec", [1, 2, 3])
def test_tc_four_step(prec):
    n, batch = 1 << 20, 2
    x = data(n, batch, 5, spiky=True)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    plan = cg.CFft1D.with_len(n, np.float32)
    tuning.set_config(plan, config(prec))
    r = rel(plan.execute_batch("forward", x), ref)
    print(f"2^20 prec={prec}: {r:.2e}")
    assert r <= (1e-4 if prec == 2 else 1e-5)


def test_tc_rejects_unsupported_plans():
    plan = cg.CFft1D.with_len(1000, np.float32)
    with pytest.raises(cg.ChfftError):
        tuning.set_config(plan, config(1))
        plan.execute_batch("forward", data(1000, 2, 1))
    p64 = cg.CFft1D.with_len(4096, np.float64)
    with pytest.raises(cg.ChfftError):
        tuning.set_config(p64, config(1))
        p64.execute_batch("forward", data(4096, 2, 1).astype(np.complex128))
