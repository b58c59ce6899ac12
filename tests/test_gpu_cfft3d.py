"""GPU: CFft3D, the native 3-D layout (no reference counterpart; CFft2D's
methods and scales extended by one axis), against numpy's FP64 fftn.

Rows of len_n, then the len_m axis and the len_l axis through the column-tile
kernels, every axis with the one-CTA engine (mixed radix or Bluestein).
Tolerances as the parity tests: f64 relative L2 <= 1e-12, f32 <= 5e-6.
"""
import numpy as np
import pytest

cg = pytest.importorskip("chfft_gb300")
torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = {np.float64: 1e-12, np.float32: 5e-6}
CPLX = {np.float64: np.complex128, np.float32: np.complex64}


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def vol(shape, dt, seed):
    rng = np.random.default_rng(seed)
    return (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(CPLX[dt])


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("shape", [(8, 16, 32), (64, 64, 64), (5, 7, 9), (3, 100, 1009), (17, 2, 48)])
def test_cfft3d_methods_match_fftn(dt, shape):
    p = cg.CFft3D.with_len(*shape, dtype=dt)
    x = vol(shape, dt, sum(shape))
    xd = x.astype(np.complex128)
    n = x.size
    ref = np.fft.fftn(xd)
    assert rel(p.forward(x), ref) <= TOL[dt]
    assert rel(p.forward0(x), ref) <= TOL[dt]
    assert rel(p.forwardu(x), ref / np.sqrt(n)) <= TOL[dt]
    assert rel(p.forwardn(x), ref / n) <= TOL[dt]
    assert rel(p.backward(x), np.fft.ifftn(xd)) <= TOL[dt]
    assert rel(p.backward0(x), np.fft.ifftn(xd) * n) <= TOL[dt]
    assert rel(p.backwardu(x), np.fft.ifftn(xd) * np.sqrt(n)) <= TOL[dt]
    assert rel(p.backward(p.forward(x)), xd) <= 2 * TOL[dt]


def test_cfft3d_replans_rejects_and_runs_batches_on_device():
    p = cg.CFft3D.with_len(4, 4, 4, dtype=np.float64)
    x = vol((6, 10, 12), np.float64, 1)
    assert rel(p.forward(x), np.fft.fftn(x)) <= 1e-12  # a new shape re-plans
    assert p.info().len_l == 6 and p.info().len_m == 10 and p.info().len_n == 12
    assert p.forward(np.zeros((0, 3, 3), np.complex128)).size == 0
    with pytest.raises(cg.ChfftError):  # no BACKWARDN, as CFft2D
        p._run("backwardn", x)
    batch = 3
    xs = vol((batch, 6, 10, 12), np.float64, 2)
    d = torch.from_numpy(xs.view(np.float64)).cuda()
    o = torch.empty_like(d)
    s = torch.cuda.current_stream().cuda_stream
    p.execute_device("forward", d.data_ptr(), o.data_ptr(), batch, s)
    p.wait(s)
    got = o.cpu().numpy().view(np.complex128).reshape(batch, 6, 10, 12)
    assert rel(got, np.fft.fftn(xs, axes=(1, 2, 3))) <= 1e-12
