"""GPU: the pipelined four-step launch (k_pipe.cuh) of power-of-two f32
CFft1D plans, through the C ABI.

Both four-step passes run in one persistent launch: a producer thread per
CTA loads 64 KiB tiles with the tensor memory accelerator into two
shared-memory stages, eight consumer warps transform them, and
intermediates live in a ring of a few slots. Checked here against numpy's
FP64 FFT (relative L2 <= 5e-6, the f32 bound of the other parity tests) and
against the two-launch path (CHFFT_PIPE=0) for every tile shape, batch
sizes around the ring and lead clamps, in-place calls, an input the tensor
map cannot describe, and the bounded waits running out
(CHFFT_TEST_STALL=1 with a short CHFFT_SPIN_LIMIT: the launch returns, the
call reports CHFFT_ETIMEOUT, and the next call on the same plan and GPU is
correct).
"""
import os

import numpy as np
import pytest

cg = pytest.importorskip("chfft_gb300")
torch = pytest.importorskip("torch")
from chfft_gb300 import tuning  # noqa: E402

pytestmark = pytest.mark.gpu

TOL = 5e-6


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


class env:
    """Temporarily set environment variables (None removes)."""

    def __init__(self, **kv):
        self.kv = kv
        self.old = {}

    def __enter__(self):
        for k, v in self.kv.items():
            self.old[k] = os.environ.get(k)
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        return self

    def __exit__(self, *exc):
        for k, v in self.old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def data(batch, n, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)


def plan_with_split(n, n1):
    p = cg.CFft1D.with_len(n, np.float32)
    if n1:
        cfg = tuning.default_config()
        cfg.fs_n1 = n1
        tuning.set_config(p, cfg)
    assert p.info().algorithm == 2
    return p


SHAPES = [(a, b) for a in (256, 512, 1024) for b in (256, 512, 1024)]


@pytest.mark.parametrize("n1,n2", SHAPES)
def test_pipe_every_tile_shape(n1, n2):
    n = n1 * n2
    p = plan_with_split(n, n1)
    x = data(5, n, n1 + n2)
    ref = np.fft.fft(x.astype(np.complex128), axis=-1)
    y = p.execute_batch("forward", x)
    assert rel(y, ref) <= TOL
    with env(CHFFT_PIPE="0"):
        y2 = p.execute_batch("forward", x)
    assert rel(y, y2) <= TOL
    assert rel(p.execute_batch("backward", y), x) <= TOL
    assert rel(p.execute_batch("forwardu", x), ref / np.sqrt(n)) <= TOL


@pytest.mark.parametrize("batch", [1, 2, 3, 4, 7, 64])
@pytest.mark.parametrize("sched", [None, "1,2,1", "2,4,0", "2,64,1"])
def test_pipe_batches_and_schedules(batch, sched):
    n = 1 << 18
    if batch == 64 and sched not in (None, "2,64,1"):
        pytest.skip("one large batch per schedule family is enough")
    p = cg.CFft1D.with_len(n, np.float32)
    x = data(batch, n, batch)
    with env(CHFFT_PIPE=sched):
        y = p.execute_batch("forward", x)
    for i in sorted({0, batch // 2, batch - 1}):
        assert rel(y[i], np.fft.fft(x[i].astype(np.complex128))) <= TOL


def test_pipe_device_in_place_and_unaligned():
    n, batch = 1 << 20, 6
    p = cg.CFft1D.with_len(n, np.float32)
    x = data(batch, n, 11)
    ref = np.fft.fft(x.astype(np.complex128), axis=-1)
    s = torch.cuda.current_stream().cuda_stream
    d = torch.from_numpy(x.view(np.float32)).cuda()
    p.execute_device("forward0i", d.data_ptr(), d.data_ptr(), batch, s)  # in place
    p.wait(s)
    assert rel(d.cpu().numpy().view(np.complex64), ref) <= TOL
    # an input 8 bytes past a 16-byte boundary cannot be a tensor map: the
    # two-launch path runs instead, with the same result
    buf = torch.zeros(2 * batch * n + 2, dtype=torch.float32, device="cuda")
    src = buf[2:].view(batch, 2 * n)
    assert src.data_ptr() % 16 == 8
    src.copy_(torch.from_numpy(x.view(np.float32)))
    out = torch.empty(batch, 2 * n, dtype=torch.float32, device="cuda")
    p.execute_device("forward", src.data_ptr(), out.data_ptr(), batch, s)
    p.wait(s)
    assert rel(out.cpu().numpy().view(np.complex64), ref) <= TOL


def test_pipe_bounded_wait_runs_out_and_recovers():
    """A dependency nothing satisfies: the bounded wait gives up, the launch
    returns, the call reports CHFFT_ETIMEOUT; the next call is correct."""
    n, batch = 1 << 18, 4
    p = cg.CFft1D.with_len(n, np.float32)
    x = data(batch, n, 3)
    with env(CHFFT_TEST_STALL="1", CHFFT_SPIN_LIMIT="20000"):
        with pytest.raises(cg.ChfftError) as e:
            p.execute_batch("forward", x)
        assert e.value.status == cg.ETIMEOUT
        # device call: the status arrives through chfft_plan_wait
        s = torch.cuda.current_stream().cuda_stream
        d = torch.from_numpy(x.view(np.float32)).cuda()
        o = torch.empty_like(d)
        p.execute_device("forward", d.data_ptr(), o.data_ptr(), batch, s)
        with pytest.raises(cg.ChfftError) as e:
            p.wait(s)
        assert e.value.status == cg.ETIMEOUT
    p.wait(0)  # the error was reported once
    y = p.execute_batch("forward", x)
    assert rel(y, np.fft.fft(x.astype(np.complex128), axis=-1)) <= TOL
