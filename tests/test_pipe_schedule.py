"""CPU checks of the pipelined four-step kernel's index arithmetic
(chfft_gb300/csrc/k_pipe.cuh), restated in numpy:

- the thread mapping of both passes (stage reads, exchange-buffer layout,
  radix-(N/32) then radix-32 butterflies, the tiles' twiddle tables, ring
  and output addresses) computes the DFT, for every supported (N1, N2),
  forward and backward;
- every exchange-buffer access stays inside the buffer, each pass writes
  every slot once, and a warp's 32 accesses of 8 bytes fall in at most two
  128-byte wavefronts (no bank conflicts);
- the shared-memory carve-up fits 227 KiB.
"""
import numpy as np
import pytest

TILE = 8192
CONS = 256
SHAPES = [(a, b) for a in (256, 512, 1024) for b in (256, 512, 1024)]


def xch_ld(n, w):
    q = 1 if w >= 16 else 16 // w
    ld = n + n // 32
    while ld % (2 * q) != q:
        ld += 1
    return ld


def pad(i):
    return i + (i >> 5)


def dft(v, axis=-1):
    """Forward DFT (y_k = sum x_n exp(-2 pi i n k / R)) along axis."""
    return np.fft.fft(v, axis=axis)


def w(n, e):
    return np.exp(-2j * np.pi * (np.asarray(e) % n) / n)


def tile_tables(n1, n2, q):
    """The pass-A tile q's tables as k_pipe_twiddles writes them:
    atab[r][t] = w_N^(c r0 r) (r < 32), wtab[j][t] = w_N^(c j) (j < r0)."""
    wa, r0, n = TILE // n1, n1 // 32, n1 * n2
    c = q * wa + np.arange(wa)[None, :]
    atab = w(n, c * r0 * np.arange(32)[:, None])
    wtab = w(n, c * np.arange(r0)[:, None])
    return atab, wtab


class Model:
    def __init__(self, n1, n2):
        self.n1, self.n2, self.n = n1, n2, n1 * n2
        self.wa, self.wb = TILE // n1, TILE // n2
        self.ta, self.tb = n2 // self.wa, n1 // self.wb
        self.lda, self.ldb = xch_ld(n1, self.wa), xch_ld(n2, self.wb)
        self.xch = max(self.wa * self.lda, self.wb * self.ldb)
        self.accesses = []  # (tag, warp addresses) for the bank check

    def note(self, tag, addr):
        self.accesses.append((tag, np.asarray(addr)))

    def tile_a(self, x, ring, tile, scale, back):
        n1, n2, W, R0 = self.n1, self.n2, self.wa, self.n1 // 32
        K0, LD = 32 // R0, self.lda
        c0 = tile * W
        stage = np.empty(TILE, np.complex128)
        rows = np.arange(n1)[:, None]
        cols = np.arange(W)[None, :]
        stage[(rows * W + cols).ravel()] = x[(rows * n2 + c0 + cols).ravel()]
        xch = np.full(self.xch, np.nan, np.complex128)
        tid = np.arange(CONS)
        written = np.zeros(self.xch, int)
        for kk in range(K0):
            bf = tid + kk * CONS
            t, j = bf % W, bf // W
            r = np.arange(R0)[:, None]
            src = (j[None, :] + 32 * r) * W + t[None, :]
            for rr in range(R0):
                self.note("A1 load", src[rr])
            v = stage[src]
            if back:
                v = np.conj(v)
            v = dft(v, axis=0)
            dst = t[None, :] * LD + pad(j[None, :] * R0 + r)
            for rr in range(R0):
                self.note("A1 store", dst[rr])
            assert dst.max() < self.xch
            xch[dst] = v
            np.add.at(written, dst.ravel(), 1)
        assert written.max() == 1 and written.sum() == n1 * W
        t, j = tid % W, tid // W
        r = np.arange(32)[:, None]
        src = t[None, :] * LD + pad(j[None, :] + R0 * r)
        for rr in range(32):
            self.note("A2 load", src[rr])
        u = xch[src]
        assert not np.isnan(u).any()
        u = u * w(n1, j[None, :] * r)
        u = dft(u, axis=0)
        atab, wtab = tile_tables(n1, n2, tile)
        wj = scale * wtab[j, t][None, :]
        tw = wj * atab[np.arange(32)[:, None], t[None, :]]
        c = c0 + t[None, :]
        k1 = j[None, :] + R0 * r
        ring[(k1 * n2 + c).ravel()] = (u * tw).ravel()

    def tile_b(self, ring, out, r0, back):
        n1, n2, W, R0 = self.n1, self.n2, self.wb, self.n2 // 32
        K0, LD = 32 // R0, self.ldb
        stage = ring[r0 * n2:(r0 + W) * n2]
        xch = np.full(self.xch, np.nan, np.complex128)
        tid = np.arange(CONS)
        for kk in range(K0):
            bf = tid + kk * CONS
            t, j = bf // 32, bf % 32
            r = np.arange(R0)[:, None]
            src = t[None, :] * n2 + j[None, :] + 32 * r
            for rr in range(R0):
                self.note("B1 load", src[rr])
            v = dft(stage[src], axis=0)
            dst = t[None, :] * LD + pad(j[None, :] * R0 + r)
            for rr in range(R0):
                self.note("B1 store", dst[rr])
            assert dst.max() < self.xch
            xch[dst] = v
        t, j = tid % W, tid // W
        r = np.arange(32)[:, None]
        src = t[None, :] * LD + pad(j[None, :] + R0 * r)
        for rr in range(32):
            self.note("B2 load", src[rr])
        u = xch[src]
        assert not np.isnan(u).any()
        u = dft(u * w(n2, j[None, :] * r), axis=0)
        if back:
            u = np.conj(u)
        out[(r0 + t[None, :] + n1 * (j[None, :] + R0 * r)).ravel()] = u.ravel()

    def run(self, x, scale=1.0, back=False):
        out = np.empty_like(x)
        for k in range(x.shape[0]):
            ring = np.full(self.n, np.nan, np.complex128)
            for tile in range(self.ta):
                self.tile_a(x[k], ring, tile, scale, back)
            assert not np.isnan(ring).any()
            for tile in range(self.tb):
                self.tile_b(ring, out[k], tile * self.wb, back)
        return out


@pytest.mark.parametrize("n1,n2", SHAPES)
def test_model_computes_the_fft(n1, n2):
    rng = np.random.default_rng(n1 + 7 * n2)
    n = n1 * n2
    x = rng.standard_normal((1, n)) + 1j * rng.standard_normal((1, n))
    m = Model(n1, n2)
    y = m.run(x)
    ref = np.fft.fft(x, axis=-1)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-12
    # backward with scale 1/N: conj(F(conj(x) / N)) = ifft(x)
    yb = m.run(x, scale=1.0 / n, back=True)
    assert np.linalg.norm(yb - np.fft.ifft(x, axis=-1)) / np.linalg.norm(x) < 1e-12


@pytest.mark.parametrize("n1,n2", SHAPES)
def test_shared_memory_accesses_are_conflict_free(n1, n2):
    m = Model(n1, n2)
    x = np.zeros((1, n1 * n2), np.complex128)
    ring = np.zeros(n1 * n2, np.complex128)
    m.tile_a(x[0], ring, 0, 1.0, False)
    m.tile_b(ring, np.zeros_like(ring), 0, False)
    for tag, addr in m.accesses:
        for wp in range(CONS // 32):
            lanes = addr[wp * 32:(wp + 1) * 32]
            distinct = np.unique(lanes)
            slots = np.bincount(distinct % 16, minlength=16)  # 8-byte words per 128-byte wavefront
            assert slots.max() <= 2, (tag, wp, slots.max())


@pytest.mark.parametrize("n1,n2", SHAPES)
def test_shared_memory_fits(n1, n2):
    wa, wb = TILE // n1, TILE // n2
    xch = max(wa * xch_ld(n1, wa), wb * xch_ld(n2, wb))
    rnd = lambda b: (b + 127) // 128 * 128  # noqa: E731
    stwb = 0 if n1 == n2 else rnd(31 * (n2 // 32) * 8)
    tabs = 2 * (32 * wa + (n1 // 32) * wa) * 8  # per stage: atab[32][wa], wtab[n1/32][wa]
    smem = 2 * TILE * 8 + rnd(xch * 8) + rnd(31 * (n1 // 32) * 8) + stwb + tabs + 64 + 1024
    assert smem <= 227 * 1024
    # tensor-map boxes: at most 256 rows, inner bytes a multiple of 16; the
    # tables' bulk copy is a multiple of 16 bytes
    assert wa <= 256 and (wa * 8) % 16 == 0 and min(n1, 256) <= 256
    assert (tabs // 2) % 16 == 0
