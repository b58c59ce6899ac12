"""CPU: the index algebra and task orders the kernels rely on, restated in
numpy / Python and checked on small cases (the GPU tests check the kernels).

- three-pass four-step Bluestein of the uneven batch (k_batch.cu FS_A,
  FS_BB, FS_C): forward FFT with k = k1 + n1 k2, spectrum product, inverse
  FFT split as m = m2 + n2 m1 so its first pass runs over the same rows;
- the pipelined four-step launch's ticket order (k_pipe.cuh decode): every
  tile appears once, and every wait is on tickets taken earlier, for any
  batch, lead and ring the host allows (plan.cu BigCore::pipe_params).
"""
import numpy as np
import pytest


def chirp(n):
    j = np.arange(n)
    # exp(-i pi j^2 / n) with j^2 reduced mod 2n exactly in integers
    return np.exp(-1j * np.pi * ((j * j) % (2 * n)) / n)


def bluestein_three_pass(x, n1, n2):
    n = x.size
    M = n1 * n2
    c = chirp(n)
    # B^ = FFT_M(conj c, wrapped) / M
    b = np.zeros(M, complex)
    b[:n] = np.conj(c)
    b[M - n + 1:] = np.conj(c[1:])[::-1]
    bhat = np.fft.fft(b) / M
    a = np.zeros(M, complex)
    a[:n] = x * c
    # FS_A: column FFTs of length n1 over j1 (x[j1 n2 + j2]), twiddle w_M^(k1 j2)
    A = a.reshape(n1, n2)
    Y = np.fft.fft(A, axis=0) * np.exp(-2j * np.pi * np.outer(np.arange(n1), np.arange(n2)) / M)
    # FS_BB: per row k1: FFT over j2 -> Z[k1][k2] (X at k = k1 + n1 k2), spectrum, conj,
    # FFT over k2 -> G[k1][m2], twiddle w_M^(k1 m2), stored as [m2][k1]
    Z = np.fft.fft(Y, axis=1)
    k = np.arange(n1)[:, None] + n1 * np.arange(n2)[None, :]
    V = np.conj(Z * bhat[k])
    G = np.fft.fft(V, axis=1) * np.exp(-2j * np.pi * np.outer(np.arange(n1), np.arange(n2)) / M)
    W = G.T  # rows m2, n1 long
    # FS_C: FFT over k1 per row m2 -> F[m2 + n2 m1]; out = conj(F) c for m < n
    F = np.fft.fft(W, axis=1)
    m = np.arange(n2)[:, None] + n2 * np.arange(n1)[None, :]
    out = np.zeros(M, complex)
    out[m.ravel()] = F.ravel()
    return np.conj(out[:n]) * c


@pytest.mark.parametrize("n,n1,n2", [(17, 5, 8), (101, 16, 14), (1009, 45, 48), (10007, 140, 144)])
def test_three_pass_bluestein_matches_dft(n, n1, n2):
    assert n1 * n2 >= 2 * n - 1
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    got = bluestein_three_pass(x, n1, n2)
    ref = np.fft.fft(x)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12


def decode(t, count, ta, tb, lead):
    """Ticket t -> (is_a, transform, tile), as k_pipe.cuh decode() does."""
    per, pairs = ta + tb, count - lead
    if t < lead * ta:
        k = t // ta
        return True, k, t - k * ta
    if t - lead * ta < pairs * per:
        u = t - lead * ta
        j, r = divmod(u, per)
        return (True, j + lead, r) if r < ta else (False, j, r - ta)
    v = t - lead * ta - pairs * per
    k = pairs + v // tb
    return False, k, v - (k - pairs) * tb


@pytest.mark.parametrize("count", [1, 2, 3, 5, 9])
@pytest.mark.parametrize("ta,tb", [(1, 1), (3, 2), (4, 7)])
@pytest.mark.parametrize("lead,ring", [(1, 2), (2, 3), (2, 4), (3, 5), (4, 4)])
def test_pipe_ticket_order(count, ta, tb, lead, ring):
    # the host clamps as BigCore::pipe_params does
    lead = max(1, min(lead, count))
    ring = min(max(ring, lead + 1), count)
    pos = {}
    for t in range(count * (ta + tb)):
        is_a, k, tile = decode(t, count, ta, tb, lead)
        assert 0 <= k < count and 0 <= tile < (ta if is_a else tb)
        assert (is_a, k, tile) not in pos
        pos[(is_a, k, tile)] = t
    assert len(pos) == count * (ta + tb)
    for (is_a, k, _), t in pos.items():
        if is_a and k >= ring:  # waits for every B(k - ring) tile: its ring slot is free
            assert all(pos[(False, k - ring, x)] < t for x in range(tb))
        if not is_a:  # waits for every A(k) tile
            assert all(pos[(True, k, x)] < t for x in range(ta))


def rader(x):
    """Rader's algorithm as k_c2c_rader computes it: a_p = x[g^p], B^ = FFT_L(b) / L
    with b_m = w_N^(g^-m), the inverse as a conjugated forward FFT, x_0 + C_q
    scattered to g^-q, X_0 = x_0 + A_0."""
    n = x.size
    L = n - 1
    g = next(c for c in range(2, n) if all(L % q or pow(c, L // q, n) != 1 for q in (2, 3, 5, 7)))
    ginv = pow(g, L - 1, n)
    p_in = np.array([pow(g, i, n) for i in range(L)])
    p_out = np.array([pow(ginv, i, n) for i in range(L)])
    assert sorted(p_in) == list(range(1, n)) and sorted(p_out) == list(range(1, n)) and 0 not in p_out
    b = np.exp(-2j * np.pi * p_out / n) / L
    bhat = np.fft.fft(b)
    A = np.fft.fft(x[p_in])
    spec = np.conj(A * bhat)
    C = np.conj(np.fft.fft(spec))
    out = np.empty(n, complex)
    out[p_out] = x[0] + C
    out[0] = x[0] + A[0]
    return out


@pytest.mark.parametrize("n", [11, 13, 17, 29, 31, 97, 257, 1009, 7681, 12289])
def test_rader_matches_dft(n):
    L = n - 1
    while L % 2 == 0:
        L //= 2
    for q in (3, 5, 7):
        while L % q == 0:
            L //= q
    assert L == 1  # n - 1 is 7-smooth
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x)
    assert np.linalg.norm(rader(x) - ref) / np.linalg.norm(ref) < 1e-12


def batch_queue(chains, smalls, lag):
    """The uneven batch's queue order (csrc/batch.cu): chains[c] lists the
    task counts of an item's steps; a later step is queued once `lag`
    tickets followed its previous step, items start in order, one-CTA tasks
    fill the gaps and follow. Returns the queue as (chain, step, k) or
    ('s', k) entries."""
    out = []
    nxt = [0] * len(chains)
    end = [0] * len(chains)
    started = small_next = done = 0

    def emit(c):
        nonlocal done
        out.extend((c, nxt[c], k) for k in range(chains[c][nxt[c]]))
        end[c] = len(out)
        nxt[c] += 1
        if nxt[c] == len(chains[c]):
            done += 1

    while done < len(chains):
        due = next((c for c in range(started) if nxt[c] < len(chains[c]) and len(out) >= end[c] + lag), None)
        if due is not None:
            emit(due)
        elif started < len(chains):
            started += 1
            emit(started - 1)
        elif small_next < smalls:
            out.append(("s", small_next))
            small_next += 1
        else:
            emit(next(c for c in range(started) if nxt[c] < len(chains[c])))
    out.extend(("s", k) for k in range(small_next, smalls))
    return out


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("lag", [0, 16, 600])
def test_batch_queue_dependencies_precede(seed, lag):
    """Every task of a step follows every task of the step it waits for (so
    a waited-for task is held by a running CTA: deadlock-free), each task is
    queued once, and where enough work exists the lag separates the steps."""
    rng = np.random.default_rng(seed)
    chains = [list(rng.integers(1, 40, size=rng.integers(2, 4))) for _ in range(rng.integers(1, 200))]
    smalls = int(rng.integers(0, 500))
    q = batch_queue(chains, smalls, lag)
    assert len(q) == sum(map(sum, chains)) + smalls
    assert len(set(q)) == len(q)
    pos = {e: i for i, e in enumerate(q)}
    for c, steps in enumerate(chains):
        for s in range(1, len(steps)):
            first = min(pos[(c, s, k)] for k in range(steps[s]))
            last_prev = max(pos[(c, s - 1, k)] for k in range(steps[s - 1]))
            assert first > last_prev
