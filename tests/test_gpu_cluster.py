"""GPU: the cluster latency form of small CFft1D batches (k_cluster.cuh),
through the C ABI.

One transform per thread-block cluster of 8 or 16 CTAs, N = n1 x n2 split
over the cluster, the exchange through distributed shared memory. Plans
take it for batches up to chfft_plan_info.cluster_max_batch (CHFFT_CLUSTER=0
at plan creation turns it off, 8 or 16 forces the cluster size). Checked against
the oracle (f64 relative L2 <= 1e-12, f32 <= 5e-6) for every method kind,
lengths one CTA holds and lengths beyond it, both cluster sizes, batches
around the threshold, in-place device calls and a captured CUDA graph.
"""
import os

import numpy as np
import pytest

import oracle

cg = pytest.importorskip("chfft_gb300")
torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = {np.float64: 1e-12, np.float32: 5e-6}
CPLX = {np.float64: np.complex128, np.float32: np.complex64}


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


def data(batch, n, seed, dt):
    rng = np.random.default_rng(seed)
    return (rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))).astype(CPLX[dt])


def plan(n, dt, size=None):
    with env(CHFFT_CLUSTER=size):
        p = cg.CFft1D.with_len(n, dt)
    return p


F64_LENGTHS = [64, 256, 1024, 2304, 4096, 16384]


@pytest.mark.parametrize("n", F64_LENGTHS)
def test_f64_default_takes_cluster_and_matches_oracle(n):
    p = plan(n, np.float64)
    info = p.info()
    assert info.cluster_ctas in (8, 16)
    assert info.cluster_n1 * info.cluster_n2 == n
    assert info.cluster_max_batch >= 1
    x = data(2, n, n, np.float64)
    for b in (1, 2):
        y = p.execute_batch("forward", x[:b])
        for i in range(b):
            assert rel(y[i], oracle.cfft1d(x[i], "forward")) <= 1e-12
    z = p.execute_batch("backward", y)
    assert rel(z, x) <= 1e-12
    assert rel(p.execute_batch("forwardu", x), np.fft.fft(x, axis=-1) / np.sqrt(n)) <= 1e-12
    assert rel(p.execute_batch("backward0", y), x * n) <= 1e-12


@pytest.mark.parametrize("size", ["8", "16"])
@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n", [1024, 4096, 16384])
def test_forced_cluster_sizes(size, dt, n):
    p = plan(n, dt, size)
    info = p.info()
    if info.cluster_ctas == 0:
        pytest.skip(f"no {size}-CTA split of {n} within the shape limits")
    assert info.cluster_ctas == int(size)
    x = data(3, n, 7, dt)
    y = p.execute_batch("forward", x)
    assert rel(y, np.fft.fft(x.astype(np.complex128), axis=-1)) <= TOL[dt]
    assert rel(p.execute_batch("backward", y), x) <= TOL[dt] * 2


def test_threshold_batches_agree_with_row_path():
    """Batches at and just above cluster_max_batch (the second runs the
    one-CTA-per-transform rows) give the same spectra."""
    n = 1024
    p = plan(n, np.float64)
    mb = p.info().cluster_max_batch
    x = data(mb + 1, n, 5, np.float64)
    ref = np.fft.fft(x, axis=-1)
    assert rel(p.execute_batch("forward", x[:mb]), ref[:mb]) <= 1e-12
    assert rel(p.execute_batch("forward", x), ref) <= 1e-12
    off = plan(n, np.float64, "0")
    assert off.info().cluster_ctas == 0
    assert rel(off.execute_batch("forward", x[:1]), ref[:1]) <= 1e-12


def test_max_batch_override_and_in_place_device():
    n, batch = 4096, 40
    with env(CHFFT_CLUSTER_MAX_BATCH="64"):
        p = cg.CFft1D.with_len(n, np.float64)
    assert p.info().cluster_max_batch == 64
    x = data(batch, n, 9, np.float64)
    ref = np.fft.fft(x, axis=-1)
    s = torch.cuda.current_stream().cuda_stream
    d = torch.from_numpy(x.view(np.float64)).cuda()
    p.execute_device("forward0i", d.data_ptr(), d.data_ptr(), batch, s)  # in place
    p.wait(s)
    assert rel(d.cpu().numpy().view(np.complex128), ref) <= 1e-12


def test_graph_capture_replays():
    n = 1024
    p = plan(n, np.float64)
    x = data(1, n, 3, np.float64)
    dev = torch.device("cuda", 0)
    d_x = torch.from_numpy(x.view(np.float64)).to(dev)
    d_y = torch.empty_like(d_x)
    d_z = torch.empty_like(d_x)
    p.execute_device("forward", d_x.data_ptr(), d_y.data_ptr(), 1, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        sp = torch.cuda.current_stream().cuda_stream
        p.execute_device("forward", d_x.data_ptr(), d_y.data_ptr(), 1, sp)
        p.execute_device("backward", d_y.data_ptr(), d_z.data_ptr(), 1, sp)
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    assert rel(d_y.cpu().numpy().view(np.complex128), oracle.cfft1d(x[0], "forward")) <= 1e-12
    assert rel(d_z.cpu().numpy().view(np.complex128), x) <= 1e-12


def test_cluster_bounded_wait_runs_out_and_recovers():
    """Rows waiting for bytes that never come: the bounded wait gives up, the
    launch returns, the call reports CHFFT_ETIMEOUT; the next call is correct."""
    n = 1024
    p = plan(n, np.float64)
    assert p.info().cluster_ctas
    x = data(1, n, 4, np.float64)
    with env(CHFFT_TEST_STALL="1", CHFFT_SPIN_LIMIT="2000"):
        with pytest.raises(cg.ChfftError) as e:
            p.execute_batch("forward", x)
        assert e.value.status == cg.ETIMEOUT
    p.wait(0)
    assert rel(p.execute_batch("forward", x), np.fft.fft(x, axis=-1)) <= 1e-12


@pytest.mark.parametrize("static", ["1", "0"])
@pytest.mark.parametrize("n", [64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384])
def test_compile_time_and_run_time_shapes_agree(n, static):
    """Power-of-two lengths run a compile-time-shape instance of the split;
    CHFFT_CLUSTER_STATIC=0 runs the run-time-shape kernel instead: both
    match the FP64 reference, forward and backward, batches 1 and 3."""
    with env(CHFFT_CLUSTER_STATIC=static):
        p = cg.CFft1D.with_len(n, np.float64)
    assert p.info().cluster_ctas in (8, 16)
    x = data(3, n, n + 1, np.float64)
    for b in (1, 3):
        y = p.execute_batch("forward", x[:b])
        assert rel(y, np.fft.fft(x[:b], axis=-1)) <= 1e-12
        assert rel(p.execute_batch("backward", y), x[:b]) <= 1e-12


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n", [128, 1024, 8192, 2304])
def test_rfft1d_cluster_form_matches_oracle(dt, n):
    """RFft1D runs its half-length FFT on a cluster at small batches (the
    split / merge in their own launches); every method matches the oracle,
    and the plan with CHFFT_CLUSTER=0 gives the same spectra."""
    with env(CHFFT_CLUSTER=None):
        p = cg.RFft1D(n, dt)
    assert p.info().cluster_ctas in (8, 16)
    with env(CHFFT_CLUSTER="0"):
        q = cg.RFft1D(n, dt)
    assert q.info().cluster_ctas == 0
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, (3, n))
    xs = x.astype(dt)
    tol = TOL[dt]
    for method in ("forward", "forwardu", "forwardn"):
        y = p.execute_batch(method, xs)
        ref = np.stack([oracle.rfft1d(xs[i].astype(np.float64), method) for i in range(3)])
        assert rel(y, ref) <= tol, method
        assert rel(y, q.execute_batch(method, xs)) <= tol, method
    spec = np.fft.rfft(xs.astype(np.float64), axis=-1).astype(np.complex128 if dt == np.float64 else np.complex64)
    for method in ("backward", "backwardu"):
        z = p.execute_batch(method, spec)
        ref = np.stack([oracle.rfft1d(spec[i].astype(np.complex128), method) for i in range(3)])
        assert rel(z, ref) <= tol, method
    assert rel(p.execute_batch("backward", p.execute_batch("forward", xs)), xs) <= 2 * tol


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n", [128, 1024, 4096, 1152])
@pytest.mark.parametrize("dct_type,ortho", [(2, False), (3, False), (2, True), (3, True)])
def test_dct1d_cluster_form_matches_oracle(dt, n, dct_type, ortho):
    """Dct1D runs its half-length FFT on a cluster at small batches (packing
    and twiddles in launches of their own); every method matches the oracle
    and the one-CTA plan (CHFFT_CLUSTER=0)."""
    with env(CHFFT_CLUSTER=None):
        p = cg.Dct1D(cg.DctType(dct_type), n, ortho, dt)
    assert p.info().cluster_ctas in (8, 16)
    with env(CHFFT_CLUSTER="0"):
        q = cg.Dct1D(cg.DctType(dct_type), n, ortho, dt)
    assert q.info().cluster_ctas == 0
    rng = np.random.default_rng(n + dct_type)
    xs = rng.uniform(-1, 1, (3, n)).astype(dt)
    tol = TOL[dt]
    for method in ("forward", "forwardu", "forwardn"):
        y = p.execute_batch(method, xs)
        ref = np.stack([oracle.dct1d(xs[i].astype(np.float64), dct_type, ortho, method) for i in range(3)])
        assert rel(y, ref) <= tol, method
        assert rel(y, q.execute_batch(method, xs)) <= tol, method


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n", [256, 1024, 4096, 2304])
@pytest.mark.parametrize("window", ["sine", "vorbis"])
def test_mdct1d_cluster_form_matches_oracle(dt, n, window):
    """Mdct1D runs its quarter-length FFT on a cluster at small batches (fold,
    window and twiddles in launches of their own), both directions, against
    the oracle and the one-CTA plan."""
    make = cg.Mdct1D.with_sine if window == "sine" else cg.Mdct1D.with_vorbis
    with env(CHFFT_CLUSTER=None):
        p = make(n, dt)
    assert p.info().cluster_ctas in (8, 16)
    with env(CHFFT_CLUSTER="0"):
        q = make(n, dt)
    assert q.info().cluster_ctas == 0
    rng = np.random.default_rng(n)
    xs = rng.uniform(-1, 1, (3, n)).astype(dt)
    tol = TOL[dt]
    for method in ("forward", "forwardu"):
        y = p.execute_batch(method, xs)
        ref = np.stack([oracle.mdct1d(xs[i].astype(np.float64), n, window, method) for i in range(3)])
        assert rel(y, ref) <= tol, method
        assert rel(y, q.execute_batch(method, xs)) <= tol, method
    ys = rng.uniform(-1, 1, (3, n // 2)).astype(dt)
    for method in ("backward", "backwardu"):
        z = p.execute_batch(method, ys)
        ref = np.stack([oracle.mdct1d(ys[i].astype(np.float64), n, window, method) for i in range(3)])
        assert rel(z, ref) <= tol, method
        assert rel(z, q.execute_batch(method, ys)) <= tol, method


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_real_kinds_cluster_form_in_place_device_and_graph(dt):
    """Dct1D (II and III) and Mdct1D in the cluster form through
    chfft_execute_device: in place (DCT), and replayed from a captured CUDA
    graph, against the one-CTA plan's results."""
    n, batch = 2048, 4
    tdt = torch.float64 if dt == np.float64 else torch.float32
    tol = TOL[dt]
    rng = np.random.default_rng(11)
    x = rng.uniform(-1, 1, (batch, n)).astype(dt)
    for t in (2, 3):
        with env(CHFFT_CLUSTER=None):
            p = cg.Dct1D(cg.DctType(t), n, False, dt)
        assert p.info().cluster_ctas in (8, 16)
        with env(CHFFT_CLUSTER="0"):
            ref = cg.Dct1D(cg.DctType(t), n, False, dt).execute_batch("forward", x)
        d = torch.from_numpy(x).cuda()
        s = torch.cuda.current_stream().cuda_stream
        p.execute_device("forward", d.data_ptr(), d.data_ptr(), batch, s)  # in place
        torch.cuda.synchronize()
        assert rel(d.cpu().numpy(), ref) <= tol, t
    with env(CHFFT_CLUSTER=None):
        m = cg.Mdct1D.with_sine(n, dt)
    assert m.info().cluster_ctas in (8, 16)
    with env(CHFFT_CLUSTER="0"):
        mref = cg.Mdct1D.with_sine(n, dt).execute_batch("forward", x)
    d_in = torch.from_numpy(x).cuda()
    d_out = torch.empty(batch, n // 2, dtype=tdt, device="cuda")
    m.execute_device("forward", d_in.data_ptr(), d_out.data_ptr(), batch, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        m.execute_device("forward", d_in.data_ptr(), d_out.data_ptr(), batch, torch.cuda.current_stream().cuda_stream)
    d_out.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert rel(d_out.cpu().numpy(), mref) <= tol
