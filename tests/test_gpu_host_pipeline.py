"""GPU: the host-memory pipeline of chfft_execute_batch.

Batches above 8 MiB run as a chunked copy-in / transform / copy-out
pipeline over two copy streams. Repeated calls on the same page-locked
buffers must read the buffers' current contents (new input each call), and
pageable and page-locked buffers, and method changes, mix freely; outputs
are checked against numpy's FP64 FFT.
"""
import numpy as np
import pytest

cg = pytest.importorskip("chfft_gb300")
torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n,batch", [(1000, 4096), (1009, 2048), (4096, 1024)])
def test_repeated_pinned_calls_see_new_input(n, batch):
    p = cg.CFft1D.with_len(n, np.float32)
    h_in = torch.empty(batch * n * 2, dtype=torch.float32).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    rng = np.random.default_rng(n)
    for call in range(4):
        x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
        h_in.numpy()[:] = x.view(np.float32).ravel()
        h_out.zero_()
        rc = cg.lib().chfft_execute_batch(p.handle, cg.METHODS["forward"], h_in.data_ptr(), h_out.data_ptr(), batch)
        assert rc == 0, cg.lib().chfft_last_error().decode()
        y = h_out.numpy().view(np.complex64).reshape(batch, n)
        for i in (0, batch // 2, batch - 1):
            assert rel(y[i], np.fft.fft(x[i].astype(np.complex128))) <= 5e-6, (call, i)


def test_pageable_then_pinned_then_method_change():
    n, batch = 1000, 2048
    p = cg.CFft1D.with_len(n, np.float32)
    rng = np.random.default_rng(7)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    ref = np.fft.fft(x.astype(np.complex128), axis=-1)
    # pageable numpy buffers
    for _ in range(3):
        assert rel(p.execute_batch("forward", x), ref) <= 5e-6
    h_in = torch.from_numpy(x.view(np.float32).ravel().copy()).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    for meth, r in (("forward", ref), ("forward", ref), ("forward", ref), ("forwardn", ref / n), ("forwardn", ref / n),
                    ("forward", ref)):
        rc = cg.lib().chfft_execute_batch(p.handle, cg.METHODS[meth], h_in.data_ptr(), h_out.data_ptr(), batch)
        assert rc == 0
        y = h_out.numpy().view(np.complex64).reshape(batch, n)
        assert rel(y, r) <= 5e-6, meth
