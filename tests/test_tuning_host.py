"""CPU: host-side pieces of the tuning layer and the Rust binding's FFI list.

- `tuning.log_uniform_lengths`, `tuning.dataset` and `tuning.regret` on
  synthetic samples (no GPU): the protocol's bookkeeping;
- every `extern "C"` function the Rust crate (rust/chfft-gb300/src/ffi.rs)
  declares exists in include/chfft_gpu.h and is exported by the library.
"""
import ctypes
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
tuning = pytest.importorskip("chfft_gb300.tuning")


def test_log_uniform_lengths_distinct_in_range_and_excluding():
    rng = np.random.default_rng(1)
    a = tuning.log_uniform_lengths(rng, 300, 64, 1 << 22)
    assert len(a) == 300 and len(set(a.tolist())) == 300
    assert a.min() >= 64 and a.max() <= (1 << 22)
    b = tuning.log_uniform_lengths(rng, 100, 64, 1 << 22, exclude=a)
    assert not set(a.tolist()) & set(b.tolist())
    # Log-uniform: about half of the draws below the geometric midpoint.
    mid = math.sqrt(64 * (1 << 22))
    assert 0.35 < np.mean(a < mid) < 0.65


class _Model:
    """Predicts the column-0 feature: a stand-in with a known ranking."""

    def predict(self, X):
        return np.asarray(X)[:, 0]


def test_dataset_and_regret_bookkeeping():
    F = tuning.FEATURES
    s1 = tuning.Sample(100, 64, np.array([[3.0] + [0] * (F - 1), [1.0] + [0] * (F - 1), [2.0] + [0] * (F - 1)]),
                       np.array([0.3, 0.1, 0.2]), 1)
    s2 = tuning.Sample(200, 1, np.array([[1.0] + [0] * (F - 1), [2.0] + [0] * (F - 1)]), np.array([0.5, 0.4]), 1)
    X, y = tuning.dataset([s1, s2])
    assert X.shape == (5, F) and X.dtype == np.float32
    assert np.allclose(y, np.log([0.3, 0.1, 0.2, 0.5, 0.4]), atol=1e-6)
    pick, heur = tuning.regret([s1, s2], _Model())
    # s1: the model picks index 1 (the best); the heuristic (index 0) is 3x.
    # s2: the model picks index 0 (0.5 against the best 0.4).
    assert np.allclose(pick, [1.0, 1.25])
    assert np.allclose(heur, [3.0, 1.25])


def _rust_ffi_names():
    src = open(os.path.join(ROOT, "rust", "chfft-gb300", "src", "ffi.rs")).read()
    block = src[src.index('extern "C"'):]
    return re.findall(r"pub fn (chfft_\w+)\(", block)


def test_rust_ffi_matches_header_and_library():
    names = _rust_ffi_names()
    assert len(names) >= 12
    header = open(os.path.join(ROOT, "include", "chfft_gpu.h")).read()
    import chfft_gb300 as cg

    lib = cg.lib()
    for n in names:
        assert re.search(r"\b" + n + r"\s*\(", header), f"{n} not declared in include/chfft_gpu.h"
        assert hasattr(lib, n), f"{n} not exported"


def test_rust_constants_match_header():
    src = open(os.path.join(ROOT, "rust", "chfft-gb300", "src", "ffi.rs")).read()
    header = open(os.path.join(ROOT, "include", "chfft_gpu.h")).read()
    rust = dict(re.findall(r"pub const (\w+): c_int = (\d+);", src))
    c = {k: v for k, v in re.findall(r"CHFFT_(\w+) = (\d+)", header)}
    pairs = {"F32": "F32", "F64": "F64", "OK": "OK", "EINVAL_LEN": "EINVAL_LEN", "DCT_TWO": "DCT_TWO",
             "DCT_THREE": "DCT_THREE", "WINDOW_CUSTOM": "WINDOW_CUSTOM"}
    for method in ("FORWARD", "FORWARD0", "FORWARDU", "FORWARDN", "BACKWARD", "BACKWARD0", "BACKWARDU",
                   "BACKWARDN", "FORWARD0I", "BACKWARD0I", "FORWARDUI", "BACKWARDUI"):
        pairs[method] = method
    for r, h in pairs.items():
        assert rust[r] == c[h], (r, rust[r], c[h])
