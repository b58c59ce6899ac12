"""Plan tuning: knobs, exhaustive autotuner and the learned cost model.

chfft has one plan per length, fixed by its factor order
(src/prime_factorization.rs:66-113) and Chirp-Z length rule
(src/cfft1d.rs:114-140). Here a plan's launch structure has knobs
(`PlanConfig`); `autotune` times every candidate on the GPU and keeps the
fastest; `CostModel` is a 3-layer MLP (CHFFT_FEATURES -> 64 -> 64 -> 1, FP32)
trained on the GPU by the library's own forward / backward kernels on the
autotuner's timings, and `propose` applies the candidate it predicts fastest,
without timing anything. Candidate 0 is always the built-in heuristic plan.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import METHODS, _check, lib

FEATURES = 48


class PlanConfig(ctypes.Structure):
    _fields_ = [
        ("k1", ctypes.c_int), ("seq_per_cta", ctypes.c_int), ("max_radix", ctypes.c_int), ("jit", ctypes.c_int),
        ("bluestein_len", ctypes.c_longlong), ("fs_n1", ctypes.c_int), ("tile_cols", ctypes.c_int),
        ("l2_chunk_mb", ctypes.c_int), ("tc_precision", ctypes.c_int), ("min_blocks_per_sm", ctypes.c_int),
        ("balanced", ctypes.c_int), ("l2_prefetch", ctypes.c_int),
        ("l2_evict_hints", ctypes.c_int), ("col_elems_per_thread", ctypes.c_int),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}

    def __repr__(self):
        return "PlanConfig(" + ", ".join(f"{k}={v}" for k, v in self.as_dict().items()) + ")"


_ready = False


def _lib():
    global _ready
    L = lib()
    if not _ready:
        vp, sz, i, f, pf = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_float, ctypes.POINTER(ctypes.c_float)
        pc = ctypes.POINTER(PlanConfig)
        pi = ctypes.POINTER(ctypes.c_int)
        sigs = {
            "chfft_plan_set_config": [vp, pc],
            "chfft_plan_get_config": [vp, pc],
            "chfft_plan_candidates": [vp, sz, i, pc, i, pi],
            "chfft_plan_features": [vp, sz, pc, pf],
            "chfft_autotune": [vp, i, sz, i, i, pc, pf, i, pi, pi],
            "chfft_plan_propose": [vp, sz, vp, i, pc],
            "chfft_mlp_create": [i, ctypes.c_uint, ctypes.POINTER(vp)],
            "chfft_mlp_destroy": [vp],
            "chfft_mlp_num_params": [vp],
            "chfft_mlp_get_params": [vp, pf],
            "chfft_mlp_set_params": [vp, pf],
            "chfft_mlp_set_moments": [vp, pf, pf, f, f],
            "chfft_mlp_get_moments": [vp, pf, pf, pf, pf],
            "chfft_mlp_loss_grad": [vp, pf, pf, i, pf, pf],
            "chfft_mlp_train": [vp, pf, pf, i, i, i, f, ctypes.c_uint, pf],
            "chfft_mlp_predict": [vp, pf, i, pf],
        }
        for name, args in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L.chfft_plan_config_default.argtypes = [pc]
        L.chfft_plan_config_default.restype = None
        _ready = True
    return L


def _fp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def default_config() -> PlanConfig:
    c = PlanConfig()
    _lib().chfft_plan_config_default(ctypes.byref(c))
    return c


def set_config(plan, cfg: PlanConfig):
    _check(_lib().chfft_plan_set_config(plan.handle, ctypes.byref(cfg)))


def get_config(plan) -> PlanConfig:
    c = PlanConfig()
    _check(_lib().chfft_plan_get_config(plan.handle, ctypes.byref(c)))
    return c


def candidates(plan, batch: int, tune_jit: bool = False) -> list[PlanConfig]:
    n = ctypes.c_int()
    _check(_lib().chfft_plan_candidates(plan.handle, batch, int(tune_jit), None, 0, ctypes.byref(n)))
    out = (PlanConfig * max(1, n.value))()
    _check(_lib().chfft_plan_candidates(plan.handle, batch, int(tune_jit), out, n.value, ctypes.byref(n)))
    return list(out[: n.value])


def features(plan, batch: int, cfg: PlanConfig) -> np.ndarray:
    f = np.zeros(FEATURES, np.float32)
    _check(_lib().chfft_plan_features(plan.handle, batch, ctypes.byref(cfg), _fp(f)))
    return f


@dataclass
class TuneResult:
    configs: list
    ms: np.ndarray   # median milliseconds per candidate
    best: int        # index of the fastest (the plan is left on it)

    @property
    def default_ms(self) -> float:
        return float(self.ms[0])

    @property
    def best_ms(self) -> float:
        return float(self.ms[self.best])


def autotune(plan, batch: int, method: str = "forward", reps: int = 3, tune_jit: bool = False) -> TuneResult:
    """Exhaustive autotune of `plan` for `batch` transforms (GPU timing)."""
    cap = 512
    cfgs = (PlanConfig * cap)()
    ms = np.zeros(cap, np.float32)
    n, best = ctypes.c_int(), ctypes.c_int()
    _check(_lib().chfft_autotune(plan.handle, METHODS[method], batch, reps, int(tune_jit), cfgs, _fp(ms), cap,
                                 ctypes.byref(n), ctypes.byref(best)))
    k = min(n.value, cap)
    return TuneResult(list(cfgs[:k]), ms[:k].copy(), best.value)


class CostModel:
    """The learned plan cost model: predicts log(ms) of a (plan, batch, config)."""

    def __init__(self, hidden: int = 64, seed: int = 0):
        self._h = ctypes.c_void_p()
        _check(_lib().chfft_mlp_create(hidden, seed, ctypes.byref(self._h)))
        self.hidden = hidden

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib().chfft_mlp_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    @property
    def num_params(self) -> int:
        return int(_lib().chfft_mlp_num_params(self._h))

    def params(self) -> np.ndarray:
        p = np.zeros(self.num_params, np.float32)
        _check(_lib().chfft_mlp_get_params(self._h, _fp(p)))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.num_params
        _check(_lib().chfft_mlp_set_params(self._h, _fp(p)))

    def moments(self):
        mu, sd = np.zeros(FEATURES, np.float32), np.zeros(FEATURES, np.float32)
        ym, ys = ctypes.c_float(), ctypes.c_float()
        _check(_lib().chfft_mlp_get_moments(self._h, _fp(mu), _fp(sd), ctypes.byref(ym), ctypes.byref(ys)))
        return mu, sd, ym.value, ys.value

    def set_moments(self, mu, sd, y_mean: float, y_sd: float):
        mu = np.ascontiguousarray(mu, np.float32)
        sd = np.ascontiguousarray(sd, np.float32)
        _check(_lib().chfft_mlp_set_moments(self._h, _fp(mu), _fp(sd), y_mean, y_sd))

    def loss_grad(self, X: np.ndarray, y: np.ndarray):
        """Loss and parameter gradient of the current model from the GPU kernels."""
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.zeros(self.num_params, np.float32)
        loss = ctypes.c_float()
        _check(_lib().chfft_mlp_loss_grad(self._h, _fp(X), _fp(y), len(y), ctypes.byref(loss), _fp(g)))
        return loss.value, g

    def train(self, X: np.ndarray, y: np.ndarray, epochs: int = 300, batch: int = 256, lr: float = 2e-3,
              seed: int = 0) -> float:
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        loss = ctypes.c_float()
        _check(_lib().chfft_mlp_train(self._h, _fp(X), _fp(y), len(y), epochs, batch, lr, seed, ctypes.byref(loss)))
        return loss.value

    def predict(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32)
        y = np.zeros(len(X), np.float32)
        _check(_lib().chfft_mlp_predict(self._h, _fp(X), len(X), _fp(y)))
        return y

    def save(self, path: str):
        mu, sd, ym, ys = self.moments()
        np.savez(path, params=self.params(), mean=mu, sd=sd, y_mean=ym, y_sd=ys, hidden=self.hidden)

    @classmethod
    def load(cls, path: str) -> "CostModel":
        z = np.load(path)
        m = cls(int(z["hidden"]))
        m.set_params(z["params"])
        m.set_moments(z["mean"], z["sd"], float(z["y_mean"]), float(z["y_sd"]))
        return m


def propose(plan, batch: int, model: CostModel, tune_jit: bool = False) -> PlanConfig:
    """Apply the candidate the cost model predicts fastest (nothing is timed)."""
    c = PlanConfig()
    _check(_lib().chfft_plan_propose(plan.handle, batch, model.handle, int(tune_jit), ctypes.byref(c)))
    return c


@dataclass
class Sample:
    length: int
    batch: int
    X: np.ndarray        # candidates x FEATURES
    ms: np.ndarray       # measured median ms per candidate
    best: int


def collect(make_plan, lengths, batches, max_elems: int = 1 << 24, reps: int = 3, tune_jit: bool = False,
            method: str = "forward", progress=None) -> list[Sample]:
    """Exhaustive timings of every candidate for each (length, batch): the
    cost model's training / evaluation data. Batches are capped so that
    batch * length <= max_elems."""
    out = []
    for i, n in enumerate(lengths):
        plan = make_plan(int(n))
        seen = set()
        for b in batches:
            b = int(max(1, min(b, max_elems // max(1, n))))
            if b in seen:
                continue
            seen.add(b)
            r = autotune(plan, b, method=method, reps=reps, tune_jit=tune_jit)
            X = np.stack([features(plan, b, c) for c in r.configs])
            out.append(Sample(int(n), b, X, r.ms, r.best))
        if progress:
            progress(i)
        del plan
    return out


def regret(samples: list[Sample], model: CostModel):
    """Per-sample time of the model's pick and of the heuristic plan, relative
    to the exhaustive best (1.0 = no regret)."""
    pick, heur = [], []
    for s in samples:
        p = model.predict(s.X)
        t_best = float(s.ms.min())
        pick.append(float(s.ms[int(np.argmin(p))]) / t_best)
        heur.append(float(s.ms[0]) / t_best)
    return np.array(pick), np.array(heur)


def dataset(samples: list[Sample]):
    X = np.concatenate([s.X for s in samples]).astype(np.float32)
    y = np.concatenate([np.log(np.maximum(s.ms, 1e-4)) for s in samples]).astype(np.float32)
    return X, y


def log_uniform_lengths(rng: np.random.Generator, count: int, lo: int, hi: int, exclude=()) -> np.ndarray:
    """`count` distinct integers, log-uniform in [lo, hi], none in `exclude`."""
    seen = set(int(v) for v in exclude)
    out = []
    while len(out) < count:
        v = int(math.exp(rng.uniform(math.log(lo), math.log(hi + 1))))
        v = min(max(v, lo), hi)
        if v not in seen:
            seen.add(v)
            out.append(v)
    return np.array(out, np.int64)
