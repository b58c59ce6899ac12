"""GPU: CFft1D on strided device layouts (chfft_execute_device_strided),
beyond the reference's contiguous slices: matrix columns, padded rows and
interleaved channels, against numpy's FP64 FFT. f64 relative L2 <= 1e-12,
f32 <= 5e-6."""
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


def dev(a, dt):
    return torch.from_numpy(np.ascontiguousarray(a).view(dt)).cuda()


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n", [60, 1000, 1009, 1024])
def test_columns_padded_rows_and_channels(dt, n):
    rng = np.random.default_rng(n)
    s = torch.cuda.current_stream().cuda_stream
    p = cg.CFft1D.with_len(n, dt)
    # columns of an n x 5 matrix -> rows of a padded (5, n + 3) buffer
    m = (rng.uniform(-1, 1, (n, 5)) + 1j * rng.uniform(-1, 1, (n, 5))).astype(CPLX[dt])
    d_in = dev(m, dt)
    d_out = torch.zeros(5 * (n + 3) * 2, dtype=d_in.dtype, device="cuda")
    p.execute_device_strided("forward", d_in.data_ptr(), 5, 1, d_out.data_ptr(), 1, n + 3, 5, s)
    p.wait(s)
    got = d_out.cpu().numpy().view(CPLX[dt]).reshape(5, n + 3)[:, :n]
    assert rel(got, np.fft.fft(m.astype(np.complex128), axis=0).T) <= TOL[dt]
    # in place on interleaved channels (stride 3, distance 1), backward
    c = (rng.uniform(-1, 1, (n, 3)) + 1j * rng.uniform(-1, 1, (n, 3))).astype(CPLX[dt])
    d_c = dev(c, dt)
    p.execute_device_strided("backward", d_c.data_ptr(), 3, 1, d_c.data_ptr(), 3, 1, 3, s)
    p.wait(s)
    got = d_c.cpu().numpy().view(CPLX[dt]).reshape(n, 3)
    assert rel(got, np.fft.ifft(c.astype(np.complex128), axis=0)) <= TOL[dt]


def test_strided_rejects_bad_strides_and_four_step_plans():
    p = cg.CFft1D.with_len(64, np.float32)
    d = torch.zeros(1024, dtype=torch.float32, device="cuda")
    with pytest.raises(cg.ChfftError):
        p.execute_device_strided("forward", d.data_ptr(), 0, 64, d.data_ptr(), 1, 64, 1, 0)
    big = cg.CFft1D.with_len(1 << 20, np.float32)
    with pytest.raises(cg.ChfftError) as e:
        big.execute_device_strided("forward", d.data_ptr(), 1, 0, d.data_ptr(), 1, 0, 1, 0)
    assert e.value.status == cg.EUNSUPPORTED
