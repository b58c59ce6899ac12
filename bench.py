#!/usr/bin/env python3
"""Benchmark: batched FFT GFLOP/s (5 N log2 N) and HBM GB/s with the roofline
fraction, plus the tensor-core form against the FP32 path at its rel-L2.

Default workload (the metric's precision configuration; "step" = one
forward pass over both parts, f32 in and out):
  - CFft1D 64 x N=2^20     (four-step: one pipelined launch)
  - CFft1D 16384 x N=4096  (one CTA per transform)
complex N(0,1) with 1% of the entries (seeded Bernoulli) scaled x1e3; both
inputs are 512 MiB, larger than L2, and sit in HBM before the timed region.
Each step is bracketed by CUDA events on the launch stream. `value` is the
plain FP32 path; `tc_vs_fp32` times the tensor-core form (radix-16 passes as
FP16 / BF16 split-operand products with FP32 accumulation) on the same plans
and inputs, each with its relative L2 error against numpy's FP64 FFT.
`e2e` runs the same workload through the C ABI's host-pointer entry point
(chfft_execute_batch) from pinned host memory, copies included.
`roofline` is the longest single launch (the 2^20 x 64 pipelined launch):
its algorithmic bytes (one read + one write) over its event time against
the measured HBM copy bandwidth; `traffic` is its DRAM read + write bytes
from the committed ncu summary.

`--workload batch` is the other f32 configuration (4096 x N=1000, 4096 x
N=1009 Chirp-Z, CFft2D 2048 x 2048); `uneven`, `costmodel` and `f64` the
rest; `latency` times the cluster form of small batches (RFft1D, Dct1D,
Mdct1D, CFft1D) against the one-CTA plans. `--impl reference` times the CPU oracle (a C++ restatement of chfft's
algorithm; the Rust crate cannot be built here) on a bounded sample of the
same workload with every host thread.

Multi-GPU: every rank runs the workload on its own GPU (independent
replicas, no collective); value = all ranks' work / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "batched FFT GFLOP/s (5N log2N), HBM GB/s; TC vs FP32 path at fixed rel-L2"
WORKLOAD = "cfft1d f32 4096x1000 + cfft1d f32 4096x1009 (chirp-z) + cfft2d f32 2048x2048, forward"
PARTS = [
    # name, kind, shape, batch, seed, distribution
    ("c2c_1000", "cfft1d", (1000,), 4096, 2, "normal"),
    ("c2c_1009", "cfft1d", (1009,), 4096, 2, "normal"),
    ("c2c2d_2048", "cfft2d", (2048, 2048), 1, 3, "uniform"),
]
CPLX_BYTES = 8  # complex f32
FLUSH_BYTES = 256 << 20


def part_elems(shape):
    return int(np.prod(shape))


def part_flops(shape, batch):
    n = part_elems(shape)
    return 5.0 * n * math.log2(n) * batch


def part_bytes(shape, batch):
    return 2.0 * part_elems(shape) * batch * CPLX_BYTES  # one read + one write


TOTAL_FLOPS = sum(part_flops(s, b) for _, _, s, b, _, _ in PARTS)
TOTAL_BYTES = sum(part_bytes(s, b) for _, _, s, b, _, _ in PARTS)


def make_input(shape, batch, seed, dist):
    rng = np.random.default_rng(seed)
    full = (batch,) + tuple(shape)
    if dist == "normal":
        x = rng.standard_normal(full, dtype=np.float32) + 1j * rng.standard_normal(full, dtype=np.float32)
    else:
        x = rng.uniform(-1, 1, full).astype(np.float32) + 1j * rng.uniform(-1, 1, full).astype(np.float32)
    return x.astype(np.complex64)


# ---------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=5)
        rows = []
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5], f[6], f[7], f[8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[2 + i].lower().startswith("active")})
        busy = [r[0] for r in rows if r[0] >= 0.5 * r[1]] or [r[0] for r in rows]
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------------------- traffic
def profiled_traffic():
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "bench_dram_traffic.txt")
    if not os.path.exists(path):
        return {}
    out = {}
    for line in open(path):
        line = line.strip()
        if not line or line.startswith("#") or ":" not in line:
            continue
        k, v = line.split(":", 1)
        try:
            out[k.strip()] = float(v.split()[0])
        except (ValueError, IndexError):
            pass
    return out


# ---------------------------------------------------------------------------- ranks
def reduce_max(values, world, device=None):
    """Element-wise max of per-rank timings over the process group (replicas:
    every rank runs the full workload on its own GPU, no data exchange)."""
    if world <= 1:
        return list(values)
    import torch

    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def aggregate_value(world, seconds):
    """Whole-job GFLOP/s: every rank's work over the slowest rank's time."""
    return world * TOTAL_FLOPS / seconds / 1e9


# ---------------------------------------------------------------------------- CPU
def cpu_run(steps: int, warmup: int, threads: int):
    """The oracle (chfft's algorithm, C++) on the full workload; seconds per step."""
    import oracle

    inputs = [make_input(s, b, seed, d) for _, _, s, b, seed, d in PARTS]
    per_step = []
    for it in range(warmup + steps):
        t = 0.0
        for (name, kind, shape, batch, _, _), x in zip(PARTS, inputs):
            if kind == "cfft1d":
                _, secs = oracle.cfft1d(x, "forward", nthreads=threads, timing=True)
            else:
                _, secs = oracle.cfft2d(x, "forward", nthreads=1, timing=True)
            t += secs
        if it >= warmup:
            per_step.append(t)
    return per_step


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    per_step = cpu_run(args.steps, args.warmup, threads)
    t = statistics.median(per_step)
    v = TOTAL_FLOPS / t / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "GFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": round(v, 3), "unit": "GFLOP/s", "cores": threads, "kind": "port",
                         "sample": "full workload per step; 1-D batches split over all host threads (one plan "
                                   "per thread), CFft2D on one thread"},
        "e2e": {"value": round(v, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "hbm_gbs": round(TOTAL_BYTES / t / 1e9, 3),
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------- GPU
def run_gpu(args, rank, world, local_rank):
    import torch

    import chfft_gb300 as cg

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    plans, d_in, d_out, h_in, h_out = [], [], [], [], []
    for name, kind, shape, batch, seed, dist in PARTS:
        x = make_input(shape, batch, seed, dist)
        if kind == "cfft1d":
            p = cg.CFft1D.with_len(shape[0], np.float32)
        else:
            p = cg.CFft2D.with_len(shape[0], shape[1], np.float32)
        plans.append(p)
        t_in = torch.from_numpy(x.view(np.float32)).to(dev)
        d_in.append(t_in)
        d_out.append(torch.empty_like(t_in))
        hi = torch.from_numpy(x.view(np.float32).reshape(batch, -1)).pin_memory()
        h_in.append(hi)
        h_out.append(torch.empty_like(hi).pin_memory())
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step(events=None):
        for i, (p, (_, _, _, batch, _, _)) in enumerate(zip(plans, PARTS)):
            if events is not None:
                events[i].record(stream)
            p.execute_device("forward", d_in[i].data_ptr(), d_out[i].data_ptr(), batch, sptr)
        if events is not None:
            events[len(plans)].record(stream)

    # correctness guard on the measured buffers (one spot check per part)
    step()
    torch.cuda.synchronize()
    for i, (name, kind, shape, batch, seed, dist) in enumerate(PARTS):
        x = make_input(shape, batch, seed, dist)
        y = d_out[i].cpu().numpy().view(np.complex64).reshape((batch,) + tuple(shape))
        ref = np.fft.fftn(x[0].astype(np.complex128))
        err = np.linalg.norm(y[0] - ref) / np.linalg.norm(ref)
        if err > 1e-5:
            raise SystemExit(f"{name}: rel-L2 {err:.2e} against numpy FP64; refusing to time a wrong result")

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    clocks = ClockSampler(local_rank).start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(len(plans) + 1)] for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()
        step(ev[k])
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    part_ms = [[ev[k][i].elapsed_time(ev[k][i + 1]) for k in range(args.steps)] for i in range(len(plans))]
    step_ms = [sum(part_ms[i][k] for i in range(len(plans))) for k in range(args.steps)]
    ms = statistics.mean(step_ms)

    # end to end through the C ABI from pinned host memory
    def e2e_step():
        for i, (p, (_, _, _, batch, _, _)) in enumerate(zip(plans, PARTS)):
            p_h = p.handle
            rc = cg.lib().chfft_execute_batch(p_h, cg.METHODS["forward"], h_in[i].data_ptr(), h_out[i].data_ptr(),
                                              batch)
            if rc != 0:
                raise SystemExit(f"chfft_execute_batch failed: {cg.lib().chfft_last_error().decode()}")

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    clk = clocks.stop()
    e2e_s = statistics.mean(e2e_times)

    ms, e2e_s = reduce_max([ms, e2e_s], world, device=dev)
    if rank != 0:
        return 0

    # dominant launch: the part with the largest mean time (one kernel each
    # for the 1-D parts; the 2-D part is a row kernel plus a column kernel)
    means = [statistics.mean(pm) for pm in part_ms]
    dom = int(np.argmax(means))
    dname, dkind, dshape, dbatch, _, _ = PARTS[dom]
    dom_launches = 2 if dkind == "cfft2d" else 1
    dom_ms = means[dom] / dom_launches
    dom_bytes = part_bytes(dshape, dbatch) / dom_launches
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured"
    if not peak:
        peak, peak_src = 6800.0, "fallback"
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    traffic = profiled_traffic().get(dname)
    h2d = sum(int(h.numel() * 4) for h in h_in)
    d2h = sum(int(h.numel() * 4) for h in h_out)
    value = aggregate_value(world, ms * 1e-3)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded normal / uniform)",
        "config": {"workload": WORKLOAD, "l2": "flushed between timed steps (256 MiB memset, outside the events)",
                   "parallelism": f"replicas x{world}"},
        "hbm_gbs": round(world * TOTAL_BYTES / (ms * 1e-3) / 1e9, 1),
        "parts_ms": {PARTS[i][0]: round(means[i], 4) for i in range(len(PARTS))},
        "roofline": {"bound": "hbm", "kernel": dname, "achieved": round(achieved, 1), "peak": peak,
                     "peak_source": f"{peak_src} hbm_gbs", "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": traffic, "algorithmic_bytes": dom_bytes},
        "e2e": {"value": round(aggregate_value(world, e2e_s), 2), "unit": "GFLOP/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_s * 1e3, 3)},
        "gpu_launches": 4 * args.steps,
        "clocks": clk,
    }
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        per = cpu_run(steps=3, warmup=1, threads=threads)
        t = statistics.median(per)
        line["cpu_baseline"] = {"value": round(TOTAL_FLOPS / t / 1e9, 3), "unit": "GFLOP/s", "cores": threads,
                                "kind": "port",
                                "sample": "the full workload, 3 timed steps after 1 warm-up; 1-D batches over all "
                                          "host threads, CFft2D on one thread"}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------- other configurations
# Optional workloads (--workload): the other benchmark configurations (large
# batches, uneven batches, the learned cost model, f64 latency), measured the
# same way; the default workload above is the headline line.

def smooth_numbers(lo, hi, primes=(2, 3, 5)):
    out = {1}
    for p in primes:
        grow = set(out)
        for v in out:
            x = v
            while x * p <= hi:
                x *= p
                grow.add(x)
        out = grow
    return np.array(sorted(v for v in out if v >= lo))


def primes_upto(n):
    s = np.ones(n + 1, bool)
    s[:2] = False
    for i in range(2, int(n ** 0.5) + 1):
        if s[i]:
            s[i * i::i] = False
    return np.nonzero(s)[0]


def mdct_def(x, n):
    """MDCT of one frame by its definition with the sine window, FP64
    (chfft's Mdct1D forward): the checker of the MDCT jobs."""
    w = np.sin(np.pi * (np.arange(n) + 0.5) / n)
    k, m = np.arange(n), np.arange(n // 2)
    return (w * x) @ np.cos(np.pi / (2 * n) * np.outer(1 + n // 2 + 2 * k, 1 + 2 * m))


def uneven_specs(count=10000, seed=4):
    """10,000 jobs, lengths log-uniform in [16, 65536]; C2C 60 % (a quarter of
    them prime, so ~15 % of all jobs), RFft1D 20 %, DCT-II 10 % (even
    {2,3,5}-smooth lengths), MDCT 10 % (frame 2048, sine window)."""
    rng = np.random.default_rng(seed)
    sm = smooth_numbers(16, 65536)
    even = sm[sm % 2 == 0]
    pr = primes_upto(65536)
    pr = pr[pr >= 16]
    specs = []
    for _ in range(count):
        u = rng.random()
        kind = "cfft1d" if u < 0.6 else "rfft1d" if u < 0.8 else "dct1d" if u < 0.9 else "mdct1d"
        x = math.exp(rng.uniform(math.log(16), math.log(65536)))
        if kind == "mdct1d":
            n = 2048
        elif kind == "cfft1d" and rng.random() < 0.25:
            n = int(pr[np.argmin(np.abs(pr - x))])
        elif kind == "cfft1d":
            n = int(sm[np.argmin(np.abs(sm - x))])
        else:
            n = int(even[np.argmin(np.abs(even - x))])
        specs.append((kind, n, "forward", 0))
    return specs


def _smooth7(n):
    for p in (2, 3, 5, 7):
        while n % p == 0:
            n //= p
    return n == 1


def uneven_subset(specs, name):
    """One class of the uneven workload (profiling): 'small' = one-CTA jobs
    (complex core <= 8192), 'big_c2c' / 'big_prime' = four-step C2C smooth /
    prime, 'big_real' = four-step real kinds, 'all' = everything."""
    if name == "all":
        return specs

    def core(k, n):
        return n if k == "cfft1d" else n // 2 if k in ("rfft1d", "dct1d") else n // 4

    keep = {
        "small": lambda k, n: core(k, n) <= 8192,
        "big_c2c": lambda k, n: k == "cfft1d" and core(k, n) > 8192 and _smooth7(n),
        "big_prime": lambda k, n: k == "cfft1d" and core(k, n) > 8192 and not _smooth7(n),
        "big_real": lambda k, n: k != "cfft1d" and core(k, n) > 8192,
    }[name]
    return [s for s in specs if keep(s[0], s[1])]


def spec_flops(kind, n):
    return (5.0 if kind == "cfft1d" else 2.5) * n * math.log2(n)


def spec_bytes(kind, n):
    return {"cfft1d": 16 * n, "rfft1d": 4 * n + 8 * (n // 2 + 1), "dct1d": 8 * n, "mdct1d": 6 * n}[kind]


def time_events(fn, steps, warmup, flush, stream):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    evs = []
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        evs.append((a, b))
    torch.cuda.synchronize()
    return statistics.mean(a.elapsed_time(b) for a, b in evs)


def oracle_job(spec, x):
    import oracle

    kind, n, method, _ = spec
    if kind == "cfft1d":
        return oracle.cfft1d(x, method, timing=True)[1]
    if kind == "rfft1d":
        return oracle.rfft1d(x, method, timing=True)[1]
    if kind == "dct1d":
        return oracle.dct1d(x, 2, False, method, timing=True)[1]
    return oracle.mdct1d(x, n, "sine", method, timing=True)[1]


def run_uneven(args):
    import concurrent.futures as cf

    import torch

    import chfft_gb300 as cg

    specs = uneven_subset(uneven_specs(), args.uneven_subset)
    b = cg.Batch(specs)
    rng = np.random.default_rng(5)
    host_in = torch.empty(b.in_bytes, dtype=torch.uint8).pin_memory()
    raw = rng.uniform(-1, 1, b.in_bytes // 4).astype(np.float32)
    host_in.numpy()[:] = raw.view(np.uint8)
    host_out = torch.empty(b.out_bytes, dtype=torch.uint8).pin_memory()
    d_in = host_in.cuda()
    d_out = torch.empty(b.out_bytes, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    # Tile widths per class of four-step items, timed on this batch
    # (chfft_batch_autotune), before the checked and timed launches.
    tiles_default = list(b.info().class_tile)
    tune_ms = b.autotune(d_in.data_ptr(), d_out.data_ptr(), sptr, reps=3) if not args.no_batch_tune else None
    run = lambda: b.execute(d_in.data_ptr(), d_out.data_ptr(), sptr, graph=True)  # noqa: E731
    run()
    b.wait(sptr)
    # spot-check 200 jobs against FP64 numpy / scipy
    out = d_out.cpu().numpy()
    import scipy.fft

    chk = np.random.default_rng(6).choice(len(specs), min(200, len(specs)), replace=False)
    worst = 0.0
    for i in chk:
        kind, n, method, _ = specs[i]
        io, oo = b.offsets[i]
        bi, bo = cg.job_bytes(kind, n)
        xin = host_in.numpy()[io:io + bi]
        x = xin.view(np.complex64).astype(np.complex128) if kind == "cfft1d" else xin.view(np.float32).astype(np.float64)
        y = out[oo:oo + bo].view(np.complex64 if kind in ("cfft1d", "rfft1d") else np.float32)
        if kind == "cfft1d":
            ref = np.fft.fft(x)
        elif kind == "rfft1d":
            ref = np.fft.rfft(x)
        elif kind == "dct1d":
            ref = scipy.fft.dct(x, type=2) / 2  # chfft's DCT-II is half of scipy's type 2
        else:
            ref = mdct_def(x, n)
        worst = max(worst, float(np.linalg.norm(y - ref) / np.linalg.norm(ref)))
    if worst > 5e-6:
        raise SystemExit(f"uneven batch: worst rel-L2 {worst:.2e}")
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    clocks = ClockSampler(0).start()
    ms = time_events(run, args.steps, args.warmup, flush, stream)

    def e2e():
        d_in.copy_(host_in, non_blocking=True)
        run()
        host_out.copy_(d_out, non_blocking=True)
        stream.synchronize()

    for _ in range(args.warmup):
        e2e()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e()
    e2e_s = (time.perf_counter() - t0) / args.steps
    clk = clocks.stop()
    flops = sum(spec_flops(k, n) for k, n, _, _ in specs)
    nbytes = sum(spec_bytes(k, n) for k, n, _, _ in specs)
    info = b.info()
    line = {
        "metric": METRIC, "value": round(flops / (ms * 1e-3) / 1e9, 2), "unit": "GFLOP/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded uniform[-1,1))",
        "config": {"workload": "uneven batch: 10000 jobs, lengths log-uniform [16, 65536], 60% C2C (15% of all prime), "
                               "20% RFft1D, 10% DCT-II, 10% MDCT 2048 sine; one work-queue launch in a CUDA graph",
                   "subset": args.uneven_subset,
                   "l2": "flushed between timed steps", "tasks": info.tasks, "ctas": info.ctas,
                   "four_step_lengths": info.four_step_lengths, "one_cta_lengths": info.one_cta_lengths,
                   "class_tiles": {"default": tiles_default, "autotuned": list(info.class_tile),
                                   "autotune_best_ms": tune_ms}},
        "hbm_gbs": round(nbytes / (ms * 1e-3) / 1e9, 1),
        "roofline": {"bound": "hbm", "kernel": "k_batch", "achieved": round(nbytes / (ms * 1e-3) / 1e9, 1),
                     "peak": 6767.1, "unit": "GB/s", "frac": round(nbytes / (ms * 1e-3) / 1e9 / 6767.1, 4),
                     "traffic": None, "algorithmic_bytes": nbytes},
        "e2e": {"value": round(flops / e2e_s / 1e9, 2), "unit": "GFLOP/s", "h2d_bytes_per_step": b.in_bytes,
                "d2h_bytes_per_step": b.out_bytes, "ms_per_step": round(e2e_s * 1e3, 3)},
        "gpu_launches": args.steps, "max_rel_l2_checked": worst, "clocks": clk,
    }
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sample = [int(i) for i in np.random.default_rng(7).choice(len(specs), 1000, replace=False)]

        def one(i):
            kind, n, _, _ = specs[i]
            io, _ = b.offsets[i]
            bi, _ = cg.job_bytes(kind, n)
            xin = host_in.numpy()[io:io + bi]
            x = xin.view(np.complex64) if kind == "cfft1d" else xin.view(np.float32)
            return oracle_job(specs[i], x.copy())

        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(threads) as ex:
            list(ex.map(one, sample))
        wall = time.perf_counter() - t0
        sflops = sum(spec_flops(specs[i][0], specs[i][1]) for i in sample)
        line["cpu_baseline"] = {"value": round(sflops / wall / 1e9, 3), "unit": "GFLOP/s", "cores": threads,
                                "kind": "port", "sample": "1000 of the 10000 jobs, one oracle call per job over all "
                                                           "host threads"}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------- default: precision configuration
PREC_WORKLOAD = ("cfft1d f32 64 x N=2^20 (pipelined four-step) + cfft1d f32 16384 x N=4096, forward; "
                 "complex N(0,1), 1% of entries x1e3")
PREC_PARTS = [("c2c_2^20x64", 1 << 20, 64), ("c2c_4096x16384", 4096, 16384)]
PREC_SMALL = [("c2c_2^20x16", 1 << 20, 16), ("c2c_4096x4096", 4096, 4096)]


def prec_input(n, batch, seed):
    """Complex N(0,1), 1% of the entries (seeded Bernoulli) scaled x1e3."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((batch, n), dtype=np.float32) + 1j * rng.standard_normal((batch, n), dtype=np.float32)
    x[rng.random((batch, n)) < 0.01] *= 1e3
    return x.astype(np.complex64)


def prec_flops(parts):
    return sum(5.0 * n * math.log2(n) * b for _, n, b in parts)


def prec_bytes(parts):
    return sum(16.0 * n * b for _, n, b in parts)


def rel_rows(x, y, rows):
    """Worst relative L2 error of rows of y against numpy's FP64 FFT of x."""
    worst = 0.0
    for r in rows:
        ref = np.fft.fft(x[r].astype(np.complex128))
        worst = max(worst, float(np.linalg.norm(y[r].astype(np.complex128) - ref) / np.linalg.norm(ref)))
    return worst


def prec_cpu(parts, reps, threads):
    """The oracle on a bounded sample of each part (2 transforms of 2^20, 256
    of 4096), all host threads; GFLOP/s of the sample."""
    import oracle

    sample = [(n, min(b, 2 if n > 65536 else 256)) for _, n, b in parts]
    xs = [prec_input(n, b, 40 + k) for k, (n, b) in enumerate(sample)]
    flops = sum(5.0 * n * math.log2(n) * b for n, b in sample)
    per = []
    for it in range(reps + 1):
        t = 0.0
        for x in xs:
            _, secs = oracle.cfft1d(x, "forward", nthreads=threads, timing=True)
            t += secs
        if it:
            per.append(t)
    t = statistics.median(per)
    desc = " + ".join(f"{b} x N={n}" for n, b in sample)
    return flops / t / 1e9, t, desc


def run_precision_reference(args, rank, world):
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    parts = PREC_SMALL if args.small else PREC_PARTS
    v, t, desc = prec_cpu(parts, max(1, min(args.steps, 5)), threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "GFLOP/s", "n_gpus": world,
        "steps": max(1, min(args.steps, 5)), "warmup": 1, "ms_per_step": round(t * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic N(0,1) complex with 1% of entries x1e3 (seeded)",
        "config": {"workload": PREC_WORKLOAD, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": round(v, 3), "unit": "GFLOP/s", "cores": threads, "kind": "port",
                         "sample": f"{desc} per step (bounded sample of the workload), one oracle call per part "
                                   "over all host threads"},
        "e2e": {"value": round(v, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_precision(args, rank, world, local_rank):
    import torch

    import chfft_gb300 as cg
    from chfft_gb300 import tuning

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    parts = PREC_SMALL if args.small else PREC_PARTS
    plans, d_in, d_out, h_in, h_out, fp32_err = [], [], [], [], [], []
    for k, (name, n, batch) in enumerate(parts):
        x = prec_input(n, batch, 4 + k)
        p = cg.CFft1D.with_len(n, np.float32)
        plans.append(p)
        hi = torch.from_numpy(x.view(np.float32)).pin_memory()
        h_in.append(hi)
        h_out.append(torch.empty_like(hi).pin_memory())
        d_in.append(hi.to(dev))
        d_out.append(torch.empty_like(d_in[-1]))
        p.execute_device("forward", d_in[-1].data_ptr(), d_out[-1].data_ptr(), batch, sptr)
        p.wait(sptr)
        y = d_out[-1].cpu().numpy().view(np.complex64)
        fp32_err.append(rel_rows(x, y, (0, batch // 2, batch - 1)))
        del x, y
    if max(fp32_err) > 1e-6:
        raise SystemExit(f"precision workload: FP32 rel-L2 {max(fp32_err):.2e} > 1e-6; refusing to time a wrong result")

    def step(evs=None):
        for i, (p, (_, _, batch)) in enumerate(zip(plans, parts)):
            if evs is not None:
                evs[i].record(stream)
            p.execute_device("forward", d_in[i].data_ptr(), d_out[i].data_ptr(), batch, sptr)
        if evs is not None:
            evs[len(plans)].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank).start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(len(plans) + 1)] for _ in range(args.steps)]
    for k in range(args.steps):
        step(ev[k])
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    for p in plans:
        p.wait(sptr)  # a timed-out device wait would have left the output incomplete
    part_ms = [[ev[k][i].elapsed_time(ev[k][i + 1]) for k in range(args.steps)] for i in range(len(plans))]
    step_ms = [sum(part_ms[i][k] for i in range(len(plans))) for k in range(args.steps)]
    ms = statistics.mean(step_ms)
    means = [statistics.mean(pm) for pm in part_ms]

    # end to end through the C ABI from pinned host memory
    def e2e_step():
        for i, (p, (_, _, batch)) in enumerate(zip(plans, parts)):
            rc = cg.lib().chfft_execute_batch(p.handle, cg.METHODS["forward"], h_in[i].data_ptr(),
                                              h_out[i].data_ptr(), batch)
            if rc != 0:
                raise SystemExit(f"chfft_execute_batch failed: {cg.lib().chfft_last_error().decode()}")

    e2e_steps = max(2, min(args.steps, 10))
    for _ in range(2):
        e2e_step()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    clk = clocks.stop()
    ms, e2e_s = reduce_max([ms, e2e_s], world, device=dev)

    # The tensor-core form on the same plans and inputs (rank 0 only; not timed
    # inside the step).
    tc = {}
    forms = {}
    if rank == 0:
        for i, (name, n, batch) in enumerate(parts):
            row = {"fp32": {"ms": round(means[i], 4), "rel_l2_vs_fp64": fp32_err[i]}}
            xs = h_in[i].numpy().view(np.complex64)
            for prec, label in ((1, "tc_fp16x2"), (2, "tc_bf16x2"), (3, "tc_bf16x3")):
                cfg = tuning.default_config()
                cfg.tc_precision = prec
                tuning.set_config(plans[i], cfg)
                fn = lambda: plans[i].execute_device("forward", d_in[i].data_ptr(), d_out[i].data_ptr(), batch, sptr)  # noqa: E731
                try:
                    fn()
                    plans[i].wait(sptr)
                except Exception as e:  # noqa: BLE001
                    row[label] = {"unavailable": str(e)}
                    continue
                err = rel_rows(xs, d_out[i].cpu().numpy().view(np.complex64), (0, batch - 1))
                t = time_events(fn, max(3, args.steps // 2), 2, None, stream)
                row[label] = {"ms": round(t, 4), "rel_l2_vs_fp64": err, "speedup_vs_fp32": round(means[i] / t, 3)}
            tuning.set_config(plans[i], tuning.default_config())
            tc[name] = row
            # four-step forms: the pipelined launch (default) against two launches
            if plans[i].info().algorithm == 2:
                fn = lambda: plans[i].execute_device("forward", d_in[i].data_ptr(), d_out[i].data_ptr(), batch, sptr)  # noqa: E731
                os.environ["CHFFT_PIPE"] = "0"
                try:
                    forms[name] = {"pipelined_ms": round(means[i], 4),
                                   "two_launch_ms": round(time_events(fn, max(3, args.steps // 2), 2, None, stream), 4)}
                finally:
                    os.environ.pop("CHFFT_PIPE", None)
    if rank != 0:
        return 0
    # roofline: the longest single launch (part 0 is one pipelined launch)
    dom = int(np.argmax(means))
    dname, dn, db = parts[dom]
    dom_bytes = 16.0 * dn * db
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured"
    if not peak:
        peak, peak_src = 6800.0, "fallback"
    achieved = dom_bytes / (means[dom] * 1e-3) / 1e9
    traffic = profiled_traffic().get(dname)
    flops = prec_flops(parts)
    nbytes = prec_bytes(parts)
    kernel = {0: "k_pipe<1024,1024> (both four-step passes, one launch)", 1: "k_c2c N=4096"}.get(dom, dname)
    line = {
        "metric": METRIC, "value": round(world * flops / (ms * 1e-3) / 1e9, 2), "unit": "GFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic N(0,1) complex with 1% of entries x1e3 (seeded)",
        "config": {"workload": PREC_WORKLOAD, "l2": "inputs larger than L2 (512 MiB per part), no flush",
                   "parallelism": f"replicas x{world}", "path": "plain FP32 kernels (value); tensor cores in tc_vs_fp32"},
        "hbm_gbs": round(world * nbytes / (ms * 1e-3) / 1e9, 1),
        "parts_ms": {parts[i][0]: round(means[i], 4) for i in range(len(parts))},
        "parts_frac_of_hbm": {parts[i][0]: round(16.0 * parts[i][1] * parts[i][2] / (means[i] * 1e-3) / 1e9 / peak, 4)
                              for i in range(len(parts))},
        "max_rel_l2_vs_fp64": max(fp32_err),
        "roofline": {"bound": "hbm", "kernel": kernel, "part": dname, "achieved": round(achieved, 1), "peak": peak,
                     "peak_source": f"{peak_src} hbm_gbs", "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": traffic, "traffic_note": "DRAM read + write bytes per launch (ncu, profiles/)",
                     "algorithmic_bytes": dom_bytes},
        "tc_vs_fp32": tc,
        "four_step_forms": forms,
        "e2e": {"value": round(world * flops / e2e_s / 1e9, 2), "unit": "GFLOP/s", "h2d_bytes_per_step": int(nbytes / 2),
                "d2h_bytes_per_step": int(nbytes / 2), "ms_per_step": round(e2e_s * 1e3, 3)},
        "gpu_launches": len(parts) * args.steps,
        "clocks": clk,
    }
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, t, desc = prec_cpu(parts, 2, threads)
        line["cpu_baseline"] = {"value": round(v, 3), "unit": "GFLOP/s", "cores": threads, "kind": "port",
                                "sample": f"{desc} (bounded sample), median of 2 after 1 warm-up, all host threads"}
    print(json.dumps(line), flush=True)
    return 0


def run_f64(args):
    """CFft1D<f64> forward + backward of one N = 1024 transform (latency):
    device time on device pointers, end-to-end time through chfft_execute on
    host arrays, relative L2 against numpy's FP64 FFT (<= 1e-12); the oracle
    is the timed CPU baseline."""
    import torch

    import chfft_gb300 as cg
    import oracle

    n = 1024
    rng = np.random.default_rng(1)
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex128)
    plan = cg.CFft1D.with_len(n, np.float64)
    ref_f = np.fft.fft(x)
    ref_b = np.fft.ifft(ref_f)  # chfft's backward scales by 1/N, as numpy's ifft
    y = plan.forward(x)
    z = plan.backward(y)
    err_f = float(np.linalg.norm(y - ref_f) / np.linalg.norm(ref_f))
    err_b = float(np.linalg.norm(z - ref_b) / np.linalg.norm(ref_b))
    if max(err_f, err_b) > 1e-12:
        raise SystemExit(f"f64 N=1024: rel-L2 {max(err_f, err_b):.2e} > 1e-12")
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    d_x = torch.from_numpy(x.view(np.float64)).to(dev)
    d_y = torch.empty_like(d_x)
    d_z = torch.empty_like(d_x)

    def step():
        plan.execute_device("forward", d_x.data_ptr(), d_y.data_ptr(), 1, sp)
        plan.execute_device("backward", d_y.data_ptr(), d_z.data_ptr(), 1, sp)

    reps = max(args.steps, 200)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    evs = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        evs.append((a, b))
    torch.cuda.synchronize()
    issue_us = statistics.median(a.elapsed_time(b) for a, b in evs) * 1e3
    # The same two launches captured once into a CUDA graph and replayed:
    # the device time without the per-call host work between the launches.
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        plan.execute_device("forward", d_x.data_ptr(), d_y.data_ptr(), 1, torch.cuda.current_stream().cuda_stream)
        plan.execute_device("backward", d_y.data_ptr(), d_z.data_ptr(), 1, torch.cuda.current_stream().cuda_stream)
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()
    gev = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        graph.replay()
        b.record(stream)
        gev.append((a, b))
    torch.cuda.synchronize()
    dev_us = statistics.median(a.elapsed_time(b) for a, b in gev) * 1e3
    # Steady state: PAIRS forward + backward pairs captured back to back in
    # one graph, the replay's event time over PAIRS (the event and graph
    # launch overheads amortised; each kernel's own launch latency counted).
    pairs = 50
    graph_n = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph_n):
        sp2 = torch.cuda.current_stream().cuda_stream
        for _ in range(pairs):
            plan.execute_device("forward", d_x.data_ptr(), d_y.data_ptr(), 1, sp2)
            plan.execute_device("backward", d_y.data_ptr(), d_z.data_ptr(), 1, sp2)
    for _ in range(args.warmup):
        graph_n.replay()
    torch.cuda.synchronize()
    sev = []
    for _ in range(max(20, reps // 10)):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        graph_n.replay()
        b.record(stream)
        sev.append((a, b))
    torch.cuda.synchronize()
    steady_us = statistics.median(a.elapsed_time(b) for a, b in sev) * 1e3 / pairs
    zz = d_z.cpu().numpy().view(np.complex128)
    if float(np.linalg.norm(zz - ref_b) / np.linalg.norm(ref_b)) > 1e-12:
        raise SystemExit("f64 N=1024: graph replay result differs")
    e2e = []
    for k in range(args.warmup + reps):
        t0 = time.perf_counter()
        yy = plan.forward(x)
        plan.backward(yy)
        if k >= args.warmup:
            e2e.append(time.perf_counter() - t0)
    e2e_us = statistics.median(e2e) * 1e6
    cpu = []
    for k in range(5 + reps):
        _, t1 = oracle.cfft1d(x, "forward", timing=True)
        _, t2 = oracle.cfft1d(ref_f, "backward", timing=True)
        if k >= 5:
            cpu.append(t1 + t2)
    cpu_us = statistics.median(cpu) * 1e6
    flops = 2 * 5.0 * n * math.log2(n)
    line = {
        "metric": METRIC, "value": round(flops / (dev_us * 1e-6) / 1e9, 3), "unit": "GFLOP/s", "n_gpus": 1,
        "steps": reps, "warmup": args.warmup, "ms_per_step": round(dev_us / 1e3, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic uniform[-1,1) complex, seed 1",
        "config": {"workload": "cfft1d f64 N=1024, one transform, forward + backward (latency)",
                   "l2": "resident (one 16 KiB transform)",
                   "timing": "value: CUDA-event time of the two launches replayed as a CUDA graph; "
                             "device_steady: 50 pairs back to back in one graph, per pair"},
        "latency_us": {"device_graph": round(dev_us, 2), "device_steady": round(steady_us, 2),
                       "device_per_call": round(issue_us, 2),
                       "e2e_host_arrays": round(e2e_us, 2), "cpu_oracle_1_thread": round(cpu_us, 2)},
        "rel_l2_vs_fp64": {"forward": err_f, "backward": err_b},
        "e2e": {"value": round(flops / (e2e_us * 1e-6) / 1e9, 3), "unit": "GFLOP/s",
                "h2d_bytes_per_step": 2 * 16 * n, "d2h_bytes_per_step": 2 * 16 * n},
        "cpu_baseline": {"value": round(flops / (cpu_us * 1e-6) / 1e9, 3), "unit": "GFLOP/s", "cores": 1, "kind": "port",
                         "sample": "the same forward + backward of N=1024 f64 on one host thread"},
        "gpu_launches": 2 * reps,
        "cluster": {"ctas": plan.info().cluster_ctas, "n1": plan.info().cluster_n1, "n2": plan.info().cluster_n2},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_costmodel(args):
    """Learned plan cost model: exhaustive autotune timings of seeded lengths
    (log-uniform in [64, 2^22]) at batches 1 / 64 / 4096 (capped at 2^24
    elements per launch), a 3-layer MLP (hidden 64, FP32) trained on them on
    the GPU, then held-out lengths: regret of the model's picks and of the
    heuristic plan against the exhaustive best, and held-out throughput under
    each. The library kernels are timed (plan-time compilation off), so the
    thousands of configurations need no NVRTC compiles."""
    os.environ["CHFFT_JIT"] = "0"
    import chfft_gb300 as cg
    from chfft_gb300 import tuning

    n_train = int(os.environ.get("CHFFT_COSTMODEL_TRAIN", "2000"))
    n_test = int(os.environ.get("CHFFT_COSTMODEL_TEST", "500"))
    rng = np.random.default_rng(5)
    train_len = tuning.log_uniform_lengths(rng, n_train, 64, 1 << 22)
    test_len = tuning.log_uniform_lengths(rng, n_test, 64, 1 << 22, exclude=train_len)
    batches = [1, 64, 4096]
    mk = lambda n: cg.CFft1D.with_len(int(n), np.float32)  # noqa: E731
    t0 = time.perf_counter()
    prog = lambda i: (i % 100 == 0) and print(f"  {i} lengths, {time.perf_counter() - t0:.0f} s",  # noqa: E731
                                              file=sys.stderr, flush=True)
    tr = tuning.collect(mk, train_len, batches, max_elems=1 << 24, reps=3, progress=prog)
    te = tuning.collect(mk, test_len, batches, max_elems=1 << 24, reps=3, progress=prog)
    t_collect = time.perf_counter() - t0
    X, y = tuning.dataset(tr)
    model = tuning.CostModel(64, seed=0)
    t1 = time.perf_counter()
    loss = model.train(X, y, epochs=200, batch=256, lr=2e-3)
    t_train = time.perf_counter() - t1
    pick, heur = tuning.regret(te, model)
    flops = np.array([5.0 * s.length * math.log2(s.length) * s.batch for s in te])
    t_best = np.array([float(s.ms.min()) for s in te])
    t_pick = pick * t_best
    t_heur = heur * t_best
    gf = lambda t: round(float(flops.sum() / (t.sum() * 1e-3) / 1e9), 2)  # noqa: E731
    line = {
        "metric": METRIC, "value": gf(t_pick), "unit": "GFLOP/s", "n_gpus": 1, "steps": len(te),
        "warmup": 1, "ms_per_step": round(float(t_pick.sum()) / len(te), 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (device scratch bytes 0x3c); lengths log-uniform in [64, 2^22], seeded",
        "config": {"workload": f"learned plan cost model: {len(train_len)} training lengths x batch {{1, 64, 4096}} "
                               f"(<= 2^24 elements), {len(test_len)} held-out lengths; CFft1D f32 forward",
                   "model": f"MLP {tuning.FEATURES}-64-64-1 ReLU FP32, Adam, 200 epochs, trained by the library's CUDA kernels",
                   "timing": "median of 3 CUDA-event launches after 1 warm-up, per candidate",
                   "kernels": "library kernels (plan-time compilation off)"},
        "held_out": {
            "cases": len(te), "train_cases": len(tr), "train_rows": int(len(y)),
            "regret_model_geomean": round(float(np.exp(np.mean(np.log(pick)))), 4),
            "regret_heuristic_geomean": round(float(np.exp(np.mean(np.log(heur)))), 4),
            "within_10pct_model": round(float(np.mean(pick <= 1.10)), 4),
            "within_10pct_heuristic": round(float(np.mean(heur <= 1.10)), 4),
            "gflops_model": gf(t_pick), "gflops_exhaustive": gf(t_best), "gflops_heuristic": gf(t_heur),
            "train_loss": round(float(loss), 5), "train_seconds": round(t_train, 2),
            "collect_seconds": round(t_collect, 1),
        },
    }
    print(json.dumps(line), flush=True)
    return 0


def run_latency(args):
    """Small batches in the cluster latency form against the one-CTA plans
    (CHFFT_CLUSTER=0 at plan creation): CUDA-event time per CUDA-graph
    replay of each case's launches, every forward result checked against
    numpy / scipy in FP64 (f64 <= 1e-12, f32 <= 5e-6 relative L2; chfft's
    DCT-II / DCT-III are half of scipy's types 2 / 3, its MDCT the
    windowed definition)."""
    import scipy.fft
    import torch

    import chfft_gb300 as cg

    def plan_with(ctor, cluster):
        old = os.environ.get("CHFFT_CLUSTER")
        if cluster:
            os.environ.pop("CHFFT_CLUSTER", None)
        else:
            os.environ["CHFFT_CLUSTER"] = "0"
        try:
            return ctor()
        finally:
            if old is None:
                os.environ.pop("CHFFT_CLUSTER", None)
            else:
                os.environ["CHFFT_CLUSTER"] = old

    # (name, kind, dtype, N, batch, methods run per replay, flops per transform and method)
    cases = [
        ("rfft1d_f64_1024_x1", "rfft1d", np.float64, 1024, 1, ("forward", "backward")),
        ("rfft1d_f32_16384_x1", "rfft1d", np.float32, 16384, 1, ("forward", "backward")),
        ("dct2_f64_16384_x1", "dct2", np.float64, 16384, 1, ("forward",)),
        ("dct3_f64_1024_x8", "dct3", np.float64, 1024, 8, ("forward",)),
        ("mdct_f64_1024_x1", "mdct1d", np.float64, 1024, 1, ("forward", "backward")),
        ("mdct_f32_8192_x8", "mdct1d", np.float32, 8192, 8, ("forward",)),
        ("cfft1d_f32_8192_x24", "cfft1d", np.float32, 8192, 24, ("forward",)),
    ]
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    reps = max(args.steps, 100)
    rows, tot_flops, tot_us, launches = {}, 0.0, 0.0, 0
    for name, kind, dt, n, batch, methods in cases:
        rdt = np.float64 if dt == np.float64 else np.float32
        cdt = np.complex128 if dt == np.float64 else np.complex64
        tdt = torch.float64 if dt == np.float64 else torch.float32
        tol = 1e-12 if dt == np.float64 else 5e-6
        rng = np.random.default_rng(n + batch)
        if kind == "rfft1d":
            ctor = lambda: cg.RFft1D(n, dt)  # noqa: E731
            x = rng.uniform(-1, 1, (batch, n)).astype(rdt)
            ref = np.fft.rfft(x.astype(np.float64), axis=-1)
            flops = 2.5 * n * math.log2(n)
        elif kind in ("dct2", "dct3"):
            t = 2 if kind == "dct2" else 3
            ctor = lambda: cg.Dct1D(cg.DctType(t), n, False, dt)  # noqa: E731
            x = rng.uniform(-1, 1, (batch, n)).astype(rdt)
            ref = scipy.fft.dct(x.astype(np.float64), type=t, axis=-1) / 2
            flops = 2.5 * n * math.log2(n)
        elif kind == "mdct1d":
            ctor = lambda: cg.Mdct1D.with_sine(n, dt)  # noqa: E731
            x = rng.uniform(-1, 1, (batch, n)).astype(rdt)
            ref = np.stack([mdct_def(x[i].astype(np.float64), n) for i in range(batch)])
            flops = 2.5 * n * math.log2(n)
        else:
            ctor = lambda: cg.CFft1D.with_len(n, dt)  # noqa: E731
            x = (rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))).astype(cdt)
            ref = np.fft.fft(x.astype(np.complex128), axis=-1)
            flops = 5.0 * n * math.log2(n)
        res = {}
        for form in ("cluster", "one_cta"):
            p = plan_with(ctor, form == "cluster")
            ctas = p.info().cluster_ctas
            if form == "cluster" and (ctas == 0 or batch > p.info().cluster_max_batch):
                raise SystemExit(f"{name}: the plan does not take the cluster form")
            if form == "one_cta" and ctas != 0:
                raise SystemExit(f"{name}: CHFFT_CLUSTER=0 left the cluster form on")
            y = p.execute_batch("forward", x)
            err = float(np.linalg.norm(np.asarray(y, np.complex128) - ref) / np.linalg.norm(ref))
            if err > tol:
                raise SystemExit(f"{name} ({form}): rel-L2 {err:.2e} against FP64 numpy / scipy > {tol}")
            # device buffers: the forward output feeds the inverse
            d_in = torch.from_numpy(np.ascontiguousarray(x).view(rdt)).to(dev)
            d_mid = torch.from_numpy(np.ascontiguousarray(y).view(rdt)).to(dev)
            d_out = torch.empty_like(d_in)

            def issue(sp):
                p.execute_device(methods[0], d_in.data_ptr(), d_mid.data_ptr(), batch, sp)
                if len(methods) > 1:
                    p.execute_device(methods[1], d_mid.data_ptr(), d_out.data_ptr(), batch, sp)

            issue(stream.cuda_stream)
            torch.cuda.synchronize()
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph):
                issue(torch.cuda.current_stream().cuda_stream)
            for _ in range(args.warmup):
                graph.replay()
            torch.cuda.synchronize()
            evs = []
            for _ in range(reps):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                graph.replay()
                b.record(stream)
                evs.append((a, b))
            torch.cuda.synchronize()
            res[form] = round(statistics.median(a.elapsed_time(b) for a, b in evs) * 1e3, 2)
            res[form + "_rel_l2"] = err
            if form == "cluster":
                res["cluster_ctas"] = ctas
                launches += reps * len(methods) * (1 if kind == "cfft1d" else 2 if kind == "rfft1d" else 3)
        res["speedup"] = round(res["one_cta"] / res["cluster"], 2)
        rows[name] = res
        tot_flops += flops * batch * len(methods)
        tot_us += res["cluster"]
    line = {
        "metric": METRIC, "value": round(tot_flops / (tot_us * 1e-6) / 1e9, 3), "unit": "GFLOP/s", "n_gpus": 1,
        "steps": reps, "warmup": args.warmup, "ms_per_step": round(tot_us / 1e3, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32", "data": "synthetic uniform[-1,1), seeded",
        "config": {"workload": "latency form: small batches of RFft1D, Dct1D, Mdct1D, CFft1D (cluster) against "
                               "the one-CTA plans; value: all cases' flops over the sum of their cluster times",
                   "l2": "resident (small batches)", "timing": "CUDA-event time per CUDA-graph replay, median"},
        "latency_us": rows,
        "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch-tune", action="store_true",
                    help="uneven workload: keep the default tile widths (skip chfft_batch_autotune)")
    ap.add_argument("--uneven-subset", default="all", choices=["all", "small", "big_c2c", "big_prime", "big_real"],
                    help="uneven workload: time one class of its jobs (profiling)")
    ap.add_argument("--small", action="store_true",
                    help="default workload only: the same kernels at 2^20 x 16 and 4096 x 4096 (profiling case)")
    ap.add_argument("--workload", choices=["precision", "batch", "uneven", "costmodel", "f64", "latency"],
                    default="precision",
                    help="precision: 64 x 2^20 + 16384 x 4096 with the tensor-core comparison (default); "
                         "batch / uneven / costmodel / f64: the other configurations; latency: the cluster "
                         "form of small batches against the one-CTA plans")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if args.workload == "precision":
            return run_precision_reference(args, rank, world)
        return run_reference(args, rank, world)
    if args.workload == "uneven":
        return run_uneven(args)
    if args.workload == "costmodel":
        return run_costmodel(args)
    if args.workload == "f64":
        return run_f64(args)
    if args.workload == "latency":
        return run_latency(args)
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    try:
        if args.workload == "precision":
            return run_precision(args, rank, world, local_rank)
        return run_gpu(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
