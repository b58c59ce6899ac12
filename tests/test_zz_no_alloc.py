"""chfft_execute_device_noalloc against chfft_execute_device and numpy's FP64 FFT.

The no-allocation entry point serves callers that cannot allocate device
memory when a transform runs (stream capture, real-time loops, pooled
device memory): it runs four-step CFft1D plans with their workspace in a
fixed array the library holds per device. This file runs last so a failure
here leaves every other test already run; it also passes on its own in a
fresh process.
"""
import ctypes

import numpy as np
import pytest

cg = pytest.importorskip("chfft_gb300")
torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _entry():
    L = cg.lib()
    fn = L.chfft_execute_device_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n,dt,batch", [(65536, np.float32, 40), (65521, np.float32, 12), (32768, np.float64, 20)])
def test_noalloc_matches_execute_device(n, dt, batch):
    fn = _entry()
    cdt = np.complex64 if dt == np.float32 else np.complex128
    tol = 5e-6 if dt == np.float32 else 1e-12
    p = cg.CFft1D.with_len(n, dt)
    assert p.info().algorithm in (2, 3)
    rng = np.random.default_rng(n + batch)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(cdt)
    rdt = torch.float32 if dt == np.float32 else torch.float64
    d_in = torch.from_numpy(x.view(np.float32 if dt == np.float32 else np.float64)).cuda()
    d_ref = torch.empty_like(d_in)
    d_out = torch.empty_like(d_in)
    assert d_in.dtype == rdt
    stream = torch.cuda.current_stream().cuda_stream
    xd = x.astype(np.complex128)
    fp64 = {"forward": np.fft.fft(xd, axis=-1), "backwardu": np.fft.ifft(xd, axis=-1) * np.sqrt(n)}
    ftol = 5e-6 if dt == np.float32 else 1e-11
    for method in ("forward", "backwardu"):
        p.execute_device(method, d_in.data_ptr(), d_ref.data_ptr(), batch, stream)
        ref = d_ref.cpu().numpy().view(cdt)
        for call in range(2):  # two calls in a row share the scratch
            d_out.zero_()
            rc = fn(p.handle, cg.METHODS[method], d_in.data_ptr(), d_out.data_ptr(), batch, stream)
            assert rc == 0, cg.lib().chfft_last_error().decode()
            out = d_out.cpu().numpy().view(cdt)
            assert rel(out, ref) <= tol, (method, call)
            assert rel(out, fp64[method]) <= ftol, (method, call)  # independent FP64 check


def test_noalloc_rejects_oversized_and_small_plans():
    fn = _entry()
    big = cg.CFft1D.with_len(1 << 22, np.float32)  # 32 MiB of workspace per transform
    d = torch.zeros(2 * (1 << 22), dtype=torch.float32, device="cuda")
    rc = fn(big.handle, cg.METHODS["forward"], d.data_ptr(), d.data_ptr(), 1, 0)
    assert rc == cg.EUNSUPPORTED
    assert "scratch" in cg.lib().chfft_last_error().decode()
    small = cg.CFft1D.with_len(1024, np.float32)  # single-CTA plan: needs no scratch
    rc = fn(small.handle, cg.METHODS["forward"], d.data_ptr(), d.data_ptr(), 1, 0)
    assert rc == cg.EINVAL


def test_noalloc_captures_into_a_graph():
    """After one warm-up call, the entry point runs inside a global-mode
    stream capture (where a cudaMalloc would fail the capture) and the
    replayed graph gives numpy's FP64 result."""
    fn = _entry()
    n, batch = 65536, 8
    p = cg.CFft1D.with_len(n, np.float32)
    rng = np.random.default_rng(7)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    d_in = torch.from_numpy(x.view(np.float32)).cuda()
    d_out = torch.empty_like(d_in)
    rc = fn(p.handle, cg.METHODS["forward"], d_in.data_ptr(), d_out.data_ptr(), batch,
            torch.cuda.current_stream().cuda_stream)
    assert rc == 0, cg.lib().chfft_last_error().decode()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, capture_error_mode="global"):
        rc = fn(p.handle, cg.METHODS["forward"], d_in.data_ptr(), d_out.data_ptr(), batch,
                torch.cuda.current_stream().cuda_stream)
    assert rc == 0, cg.lib().chfft_last_error().decode()
    d_out.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert rel(d_out.cpu().numpy().view(np.complex64), np.fft.fft(x.astype(np.complex128), axis=-1)) <= 5e-6
    assert torch.cuda.mem_get_info()[0] >= free_before - (64 << 20)  # no workspace growth beyond the graph's own pool
