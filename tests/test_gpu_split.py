"""GPU: CFft1D on split-complex device arrays (chfft_execute_device_split),
a native layout the reference does not offer (its Complex<T> is
interleaved), against numpy's FP64 FFT and the interleaved entry point.

Tolerances as the parity tests: f64 relative L2 <= 1e-12, f32 <= 5e-6.
"""
import numpy as np
import pytest

cg = pytest.importorskip("chfft_gb300")
torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = {np.float64: 1e-12, np.float32: 5e-6}
TDT = {np.float64: torch.float64, np.float32: torch.float32}


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run_split(p, method, x, dt, in_place=False):
    s = torch.cuda.current_stream().cuda_stream
    re = torch.from_numpy(np.ascontiguousarray(x.real.astype(dt))).cuda()
    im = torch.from_numpy(np.ascontiguousarray(x.imag.astype(dt))).cuda()
    ore, oim = (re, im) if in_place else (torch.empty_like(re), torch.empty_like(im))
    p.execute_device_split(method, re.data_ptr(), im.data_ptr(), ore.data_ptr(), oim.data_ptr(), x.shape[0], s)
    p.wait(s)
    return ore.cpu().numpy() + 1j * oim.cpu().numpy()


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n", [16, 60, 1000, 1009, 1024, 4096])
@pytest.mark.parametrize("batch", [1, 7])
def test_split_matches_fft(dt, n, batch):
    rng = np.random.default_rng(n + batch)
    x = rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))
    x = x.astype(np.complex128 if dt == np.float64 else np.complex64).astype(np.complex128)
    p = cg.CFft1D.with_len(n, dt)
    ref = np.fft.fft(x, axis=-1)
    assert rel(run_split(p, "forward", x, dt), ref) <= TOL[dt]
    assert rel(run_split(p, "backward", ref, dt), x) <= 2 * TOL[dt]
    assert rel(run_split(p, "forwardu", x, dt, in_place=True), ref / np.sqrt(n)) <= TOL[dt]
    inter = p.execute_batch("forward", x.astype(np.complex128 if dt == np.float64 else np.complex64))
    assert rel(run_split(p, "forward", x, dt), inter) <= TOL[dt]


def test_split_refuses_four_step_plans():
    p = cg.CFft1D.with_len(1 << 20, np.float32)
    d = torch.zeros(1 << 20, dtype=torch.float32, device="cuda")
    with pytest.raises(cg.ChfftError) as e:
        p.execute_device_split("forward", d.data_ptr(), d.data_ptr(), d.data_ptr(), d.data_ptr(), 1, 0)
    assert e.value.status == cg.EUNSUPPORTED
