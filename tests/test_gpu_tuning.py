"""GPU: plan knobs, the exhaustive autotuner and the learned cost model.

Every candidate configuration of a plan must compute the same transform
(checked against numpy.fft / the oracle within the parity tolerances); the
cost model's CUDA forward / backward kernels are checked against the CPU
oracle's float64 gradient (oracle/mlp.py); the autotuner's pick is never
slower than the heuristic plan it includes as candidate 0.
"""
import numpy as np
import pytest

import oracle
from oracle import mlp as omlp

cg = pytest.importorskip("chfft_gb300")
from chfft_gb300 import tuning  # noqa: E402

pytestmark = pytest.mark.gpu

F = tuning.FEATURES


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _check_c2c(plan, n, batch, dt, tol):
    rng = np.random.default_rng(n)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(
        np.complex64 if dt == np.float32 else np.complex128)
    y = plan.execute_batch("forward", x)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    assert rel(y, ref) <= tol


@pytest.mark.parametrize("n,batch,tune_jit", [(1000, 40, False), (1024, 33, False), (1009, 20, False),
                                              (4096, 9, False), (97, 50, False), (1 << 16, 3, False),
                                              (65521, 2, False), (1000, 40, True), (1 << 16, 3, True)])
def test_every_candidate_computes_the_transform(n, batch, tune_jit):
    plan = cg.CFft1D.with_len(n, np.float32)
    cands = tuning.candidates(plan, batch, tune_jit)
    assert len(cands) >= 1
    # Candidate 0 is the heuristic plan.
    assert cands[0].as_dict() == tuning.default_config().as_dict()
    for c in cands:
        tuning.set_config(plan, c)
        assert tuning.get_config(plan).as_dict() == c.as_dict()
        _check_c2c(plan, n, batch, np.float32, 5e-6)


@pytest.mark.parametrize("n", [1000, 1 << 20])
def test_every_candidate_f64(n):
    plan = cg.CFft1D.with_len(n, np.float64)
    batch = 6 if n < 4096 else 2
    for c in tuning.candidates(plan, batch, False):
        tuning.set_config(plan, c)
        _check_c2c(plan, n, batch, np.float64, 1e-12)


def test_candidates_2d_and_real_kinds():
    rng = np.random.default_rng(3)
    p2 = cg.CFft2D.with_len(48, 80, np.float32)
    x = (rng.random((48, 80)) + 1j * rng.random((48, 80))).astype(np.complex64)
    for c in tuning.candidates(p2, 1):
        tuning.set_config(p2, c)
        assert rel(p2.forward(x), np.fft.fft2(x.astype(np.complex128))) <= 5e-6
    pr = cg.RFft1D(4000, np.float32)
    xr = rng.random((7, 4000)).astype(np.float32)
    ref = np.fft.rfft(xr.astype(np.float64), axis=1)
    for c in tuning.candidates(pr, 7):
        tuning.set_config(pr, c)
        assert rel(pr.execute_batch("forward", xr), ref) <= 5e-6
    pd = cg.Dct1D(cg.DctType.Two, 512, False, np.float64)
    xd = rng.random((5, 512))
    exp = np.stack([oracle.dct1d(v, 2) for v in xd])
    for c in tuning.candidates(pd, 5):
        tuning.set_config(pd, c)
        assert rel(pd.execute_batch("forward", xd), exp) <= 1e-12


def test_autotune_picks_no_slower_than_heuristic():
    plan = cg.CFft1D.with_len(1000, np.float32)
    r = tuning.autotune(plan, 512, reps=5)
    assert len(r.configs) == len(r.ms) >= 2
    assert r.best_ms <= r.default_ms
    assert tuning.get_config(plan).as_dict() == r.configs[r.best].as_dict()
    _check_c2c(plan, 1000, 8, np.float32, 5e-6)


def test_features_shape_and_distinctness():
    plan = cg.CFft1D.with_len(1009, np.float32)
    cands = tuning.candidates(plan, 64)
    X = np.stack([tuning.features(plan, 64, c) for c in cands])
    assert X.shape == (len(cands), F)
    assert np.all(np.isfinite(X))
    # Distinct launch structures give distinct feature rows.
    assert len({tuple(r) for r in X}) == len(cands)


def _synthetic(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, F)).astype(np.float32) * rng.uniform(0.5, 3, F).astype(np.float32)
    y = (np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2] / 4 - 0.3 * np.abs(X[:, 3])).astype(np.float32)
    return X, y


@pytest.mark.parametrize("hidden,n", [(64, 300), (64, 64), (16, 130), (64, 1)])
def test_mlp_gradient_matches_cpu_oracle(hidden, n):
    X, y = _synthetic(max(n, 1), 7)
    m = tuning.CostModel(hidden, seed=11)
    mu = X.mean(0)
    sd = X.std(0) + 0.5
    m.set_moments(mu, sd, float(y.mean()), float(y.std() + 0.1))
    loss, g = m.loss_grad(X, y)
    Xs, ys = omlp.standardise(X, y, mu, sd, float(np.float32(y.mean())), float(np.float32(y.std() + 0.1)))
    lo, go = omlp.loss_grad(m.params(), Xs, ys, F, hidden)
    assert abs(loss - lo) <= 1e-4 * max(1.0, abs(lo))
    assert np.linalg.norm(g - go) <= 1e-4 * np.linalg.norm(go)


def test_mlp_training_and_prediction():
    X, y = _synthetic(4000, 5)
    m = tuning.CostModel(64, seed=3)
    m.set_moments(np.zeros(F), np.ones(F), 0.0, 1.0)
    before, _ = m.loss_grad(X, y)
    final = m.train(X, y, epochs=60, batch=128, lr=3e-3, seed=1)
    assert final < 0.2 * before
    # Prediction kernel = the oracle's forward pass on the trained parameters.
    mu, sd, ym, ys = m.moments()
    Xt, _ = _synthetic(200, 9)
    pred = m.predict(Xt)
    Xs = (Xt.astype(np.float64) - mu) / sd
    ref = omlp.forward(m.params(), Xs, F, 64) * ys + ym
    assert np.max(np.abs(pred - ref)) <= 1e-4 * max(1.0, np.max(np.abs(ref)))


def test_model_save_load_and_propose(tmp_path):
    X, y = _synthetic(500, 2)
    m = tuning.CostModel(64, seed=0)
    m.train(X, y, epochs=5, batch=64)
    path = str(tmp_path / "model.npz")
    m.save(path)
    m2 = tuning.CostModel.load(path)
    assert np.array_equal(m.params(), m2.params())
    assert np.allclose(m.predict(X[:20]), m2.predict(X[:20]))
    plan = cg.CFft1D.with_len(1000, np.float32)
    chosen = tuning.propose(plan, 64, m2)
    assert tuning.get_config(plan).as_dict() == chosen.as_dict()
    _check_c2c(plan, 1000, 8, np.float32, 5e-6)


def test_learned_plans_against_exhaustive_small(monkeypatch):
    """A small instance of the learned-plan protocol: timings of every
    candidate for seeded training lengths, a GPU-trained model, then held-out
    lengths: the model's picks must stay within 10% of the exhaustive best on
    (geometric) average and beat the heuristic plan (the method without the
    network). Library kernels only (no plan-time compiles)."""
    monkeypatch.setenv("CHFFT_JIT", "0")
    rng = np.random.default_rng(2024)
    train_len = tuning.log_uniform_lengths(rng, 200, 64, 1 << 18)
    test_len = tuning.log_uniform_lengths(rng, 48, 64, 1 << 18, exclude=train_len)
    mk = lambda n: cg.CFft1D.with_len(n, np.float32)  # noqa: E731
    tr = tuning.collect(mk, train_len, [1, 64, 4096], max_elems=1 << 21, reps=5)
    te = tuning.collect(mk, test_len, [1, 64, 4096], max_elems=1 << 21, reps=5)
    X, y = tuning.dataset(tr)
    m = tuning.CostModel(64, seed=0)
    m.train(X, y, epochs=200, batch=128, lr=2e-3)
    pick, heur = tuning.regret(te, m)
    g_pick = float(np.exp(np.mean(np.log(pick))))
    g_heur = float(np.exp(np.mean(np.log(heur))))
    print(f"held-out: model {g_pick:.3f}x of exhaustive, heuristic {g_heur:.3f}x ({len(te)} cases)")
    assert g_pick <= 1.10  # within 10% of exhaustive autotuning
    assert g_pick < g_heur  # the trained network beats the plan chosen without it
