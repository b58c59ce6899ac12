"""Generate tests/golden/golden.npz: seeded inputs and the CPU oracle's outputs.

The reference (a Rust crate) cannot be built here and ships no golden
vectors, so the fixtures record the oracle's outputs for small seeded inputs
of every plan type, dtype and method family. tests/test_golden.py checks the
oracle still reproduces them and the GPU path matches them.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")


def cases():
    rng = np.random.default_rng(20261203)
    for dt, cdt, tag in ((np.float64, np.complex128, "f64"), (np.float32, np.complex64, "f32")):
        for n in (8, 12, 97, 1000, 1009):
            rows = 2 if n < 100 else 1
            x = (rng.uniform(-1, 1, (rows, n)) + 1j * rng.uniform(-1, 1, (rows, n))).astype(cdt)
            for m in ("forward", "forwardu", "backward") if n < 100 else ("forward", "backward"):
                yield f"cfft1d/{tag}/{n}/{m}", x, oracle.cfft1d(x, m)
        x = (rng.uniform(-1, 1, (6, 10)) + 1j * rng.uniform(-1, 1, (6, 10))).astype(cdt)
        for m in ("forward", "backward"):
            yield f"cfft2d/{tag}/6x10/{m}", x, oracle.cfft2d(x, m)
        for n in (30, 64):
            x = rng.uniform(-1, 1, (2, n)).astype(dt)
            yield f"rfft1d/{tag}/{n}/forward", x, oracle.rfft1d(x, "forward")
            y = oracle.rfft1d(x, "forward")
            yield f"rfft1d/{tag}/{n}/backward", y, oracle.rfft1d(y, "backward")
            for t in (2, 3):
                for ortho in (False, True):
                    yield f"dct1d/{tag}/{n}/{t}/{int(ortho)}", x, oracle.dct1d(x, t, ortho, "forward")
        for n, w in ((64, "sine"), (44, "vorbis")):
            x = rng.uniform(-1, 1, (2, n)).astype(dt)
            y = oracle.mdct1d(x, n, w, "forward")
            yield f"mdct1d/{tag}/{n}/{w}/forward", x, y
            yield f"mdct1d/{tag}/{n}/{w}/backward", y, oracle.mdct1d(y, n, w, "backward")


def main():
    data = {}
    for key, x, y in cases():
        data[key + "|in"] = x
        data[key + "|out"] = y
    np.savez_compressed(OUT, **data)
    print(f"wrote {len(data) // 2} cases to {OUT}")


if __name__ == "__main__":
    main()
