"""Uneven batches: one work-queue launch over mixed kinds and lengths.

Every job's output is checked against the oracle (the reference's call for
that kind and length) at the f32 tolerance (relative L2 <= 5e-6 against the
f64 oracle). Covers one-CTA jobs (mixed radix and Bluestein), four-step jobs
(C2C, four-step Bluestein, R2C / DCT-II with a four-step half length and
their post tasks), the CUDA-graph replay, and the bounded-wait status.
"""
import os

import numpy as np
import pytest

import oracle

cg = pytest.importorskip("chfft_gb300")
torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_inputs(specs, batch, seed=0):
    rng = np.random.default_rng(seed)
    host_in = np.zeros(batch.in_bytes, np.uint8)
    xs = []
    for (kind, n, method, option), (io, _) in zip(specs, batch.offsets):
        if kind == "cfft1d":
            x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
        else:
            x = rng.uniform(-1, 1, n).astype(np.float32)
        host_in[io:io + x.nbytes] = x.view(np.uint8)
        xs.append(x)
    return host_in, xs


def expected(kind, n, method, option, x):
    if kind == "cfft1d":
        return oracle.cfft1d(x.astype(np.complex128), method)
    if kind == "rfft1d":
        return oracle.rfft1d(x.astype(np.float64), method)
    if kind == "dct1d":
        return oracle.dct1d(x.astype(np.float64), 2, bool(option), method)
    return oracle.mdct1d(x.astype(np.float64), n, "vorbis" if option == 1 else "sine", method)


def out_view(kind, n, raw):
    if kind in ("cfft1d",):
        return raw[: 8 * n].view(np.complex64)
    if kind == "rfft1d":
        return raw[: 8 * (n // 2 + 1)].view(np.complex64)
    if kind == "dct1d":
        return raw[: 4 * n].view(np.float32)
    return raw[: 2 * n].view(np.float32)


def run_and_check(specs, graph=False, repeat=1):
    b = cg.Batch(specs)
    host_in, xs = make_inputs(specs, b)
    d_in = torch.from_numpy(host_in).cuda()
    d_out = torch.zeros(max(b.out_bytes, 16), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(repeat):
        d_out.zero_()
        b.execute(d_in.data_ptr(), d_out.data_ptr(), stream, graph=graph)
        b.wait(stream)
        host_out = d_out.cpu().numpy()
        for (kind, n, method, option), (_, oo), x in zip(specs, b.offsets, xs):
            got = out_view(kind, n, host_out[oo:])
            r = rel(got, expected(kind, n, method, option, x))
            assert r <= 5e-6, (kind, n, method, r)
    return b


def test_batch_one_cta_mixed():
    specs = [("cfft1d", n, "forward", 0) for n in (16, 17, 60, 97, 1000, 1009, 2048, 4096, 8192, 3000, 4001)]
    specs += [("rfft1d", n, m, 0) for n, m in ((32, "forward"), (1000, "forwardn"), (2046, "forwardu"), (16384, "forward"))]
    specs += [("dct1d", n, "forward", o) for n, o in ((64, 0), (1000, 1), (4096, 0), (22, 0))]
    specs += [("mdct1d", n, m, o) for n, m, o in ((2048, "forward", 0), (2048, "forwardu", 1), (64, "forward", 0))]
    specs += [("cfft1d", 1000, "forward", 0)] * 9  # grouped into one task
    b = run_and_check(specs)
    assert b.info().four_step_lengths == 0


def test_batch_four_step_mixed():
    specs = [("cfft1d", n, "forward", 0) for n in (16384, 65536, 20000, 10007, 65521, 40000)]
    specs += [("rfft1d", 65536, "forward", 0), ("rfft1d", 40000, "forwardn", 0)]
    specs += [("dct1d", 65536, "forward", 0), ("dct1d", 20000, "forwardu", 1)]
    specs += [("cfft1d", 100, "forward", 0), ("mdct1d", 2048, "forward", 0)]
    b = run_and_check(specs)
    info = b.info()
    assert info.four_step_lengths >= 5 and info.workspace_bytes > 0


def test_batch_graph_replay():
    specs = [("cfft1d", n, "forward", 0) for n in (1000, 1009, 65536, 31)] + [("rfft1d", 40000, "forward", 0)]
    run_and_check(specs, graph=True, repeat=3)


def test_batch_rejects_bad_jobs():
    with pytest.raises(cg.InvalidLength):
        cg.Batch([("rfft1d", 33, "forward", 0)])
    with pytest.raises(cg.ChfftError):
        cg.Batch([("cfft1d", 64, "backward", 0)])


def test_batch_full_uneven_workload():
    """The whole 10,000-job uneven workload of the benchmark (lengths
    log-uniform in [16, 65536], 15% prime, 60/20/10/10 C2C / R2C / DCT-II /
    MDCT): every job against the oracle at 5e-6."""
    import concurrent.futures as cf

    import bench

    specs = bench.uneven_specs()
    b = cg.Batch(specs)
    host_in, xs = make_inputs(specs, b, seed=9)
    d_in = torch.from_numpy(host_in).cuda()
    d_out = torch.zeros(max(b.out_bytes, 16), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    b.execute(d_in.data_ptr(), d_out.data_ptr(), stream, graph=True)
    b.wait(stream)
    host_out = d_out.cpu().numpy()

    def check(i):
        kind, n, method, option = specs[i]
        got = out_view(kind, n, host_out[b.offsets[i][1]:])
        return rel(got, expected(kind, n, method, option, xs[i])), i

    with cf.ThreadPoolExecutor(os.cpu_count() or 4) as ex:
        worst, i = max(ex.map(check, range(len(specs))))
    assert worst <= 5e-6, (specs[i], worst)


def test_batch_bounded_wait_runs_out_and_recovers(monkeypatch):
    """Every dependency unreachable (CHFFT_TEST_STALL=1, short
    CHFFT_SPIN_LIMIT): the four-step tasks' waits give up, the launch
    returns, chfft_batch_wait reports CHFFT_ETIMEOUT; the next launch of the
    same batch on the same GPU is correct."""
    specs = [("cfft1d", 65536, "forward", 0), ("cfft1d", 1000, "forward", 0), ("rfft1d", 40000, "forward", 0)]
    b = cg.Batch(specs)
    host_in, xs = make_inputs(specs, b)
    d_in = torch.from_numpy(host_in).cuda()
    d_out = torch.zeros(max(b.out_bytes, 16), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    monkeypatch.setenv("CHFFT_TEST_STALL", "1")
    monkeypatch.setenv("CHFFT_SPIN_LIMIT", "20000")
    b.execute(d_in.data_ptr(), d_out.data_ptr(), stream)
    with pytest.raises(cg.ChfftError) as e:
        b.wait(stream)
    assert e.value.status == cg.ETIMEOUT
    monkeypatch.delenv("CHFFT_TEST_STALL")
    monkeypatch.delenv("CHFFT_SPIN_LIMIT")
    d_out.zero_()
    b.execute(d_in.data_ptr(), d_out.data_ptr(), stream)
    b.wait(stream)
    host_out = d_out.cpu().numpy()
    for (kind, n, method, option), (_, oo), x in zip(specs, b.offsets, xs):
        assert rel(out_view(kind, n, host_out[oo:]), expected(kind, n, method, option, x)) <= 5e-6


def test_batch_autotune_picks_class_tiles_and_stays_correct():
    """chfft_batch_autotune times tile widths 16 / 32 / 64 per class of
    four-step items on the batch itself; afterwards every used class has a
    width from that set, unused classes report 0, and every job still
    matches the oracle (normal launch and graph replay)."""
    specs = [("cfft1d", n, "forward", 0) for n in (16384, 20000, 40000, 65536, 10007, 65521)] * 3
    specs += [("rfft1d", n, "forward", 0) for n in (40000, 65536)] * 2
    specs += [("cfft1d", 1000, "forward", 0)] * 20
    b = cg.Batch(specs)
    before = list(b.info().class_tile)
    assert all(t in (0, 64) for t in before) and any(before)
    host_in, xs = make_inputs(specs, b)
    d_in = torch.from_numpy(host_in).cuda()
    d_out = torch.zeros(max(b.out_bytes, 16), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    ms = b.autotune(d_in.data_ptr(), d_out.data_ptr(), stream, reps=3)
    assert ms > 0
    after = list(b.info().class_tile)
    for t0, t1 in zip(before, after):
        assert (t0 == 0) == (t1 == 0)
        assert t1 in (0, 16, 32, 64)
    for graph in (False, True):
        d_out.zero_()
        b.execute(d_in.data_ptr(), d_out.data_ptr(), stream, graph=graph)
        b.wait(stream)
        host_out = d_out.cpu().numpy()
        for (kind, n, method, option), (_, oo), x in zip(specs, b.offsets, xs):
            assert rel(out_view(kind, n, host_out[oo:]), expected(kind, n, method, option, x)) <= 5e-6
