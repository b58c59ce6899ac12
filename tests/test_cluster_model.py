"""CPU model of the cluster latency form (chfft_gb300/csrc/k_cluster.cuh).

One transform of N = n1 x n2 over a cluster of C CTAs: CTA c stages columns
[c wa, (c+1) wa) (wa = n2 / C) of the input into buf0[t lda + i] and runs
the n1-point passes (one output per element, the next pass's twiddle
folded into each output); its last column pass multiplies by the
four-step twiddles (the scale folded in, [n2][k1] blocks) and stores
element (k1, n2) into row k1 mod wb of CTA k1 // wb (wb = n1 / C); after
the cluster barrier each CTA runs the n2-point passes of its rows and
stores X[k1 + n1 k2]. The model follows the kernel's index arithmetic
(pass indexing, per-pass twiddle tables, per-CTA offsets, each CTA's
table block) with numpy butterflies, and checks the shared-memory layout
stays inside the launch's dynamic shared memory. The real kinds' pre and
post launches around the cluster core (k_cluster.cu k_rfft_split /
k_rfft_merge, real_pre / real_post) are restated too, with numpy's FFT as
the core, against the oracle.
"""
import numpy as np
import pytest


def radix_code(n):
    """Pass radices of the cluster kernels: 4 while possible, then 2, 3, 5, 7."""
    rs = []
    while n % 4 == 0:
        rs.append(4)
        n //= 4
    for r in (2, 3, 5, 7):
        while n % r == 0:
            rs.append(r)
            n //= r
    assert n == 1
    return rs


def pass_table(n, radices, p):
    """Input twiddle of pass p at input position i (k_cluster.cu's
    k_pass_tables): r = i // (n / R), jm = (i mod (n / R)) mod Ns."""
    R = radices[p]
    ns = int(np.prod(radices[:p])) if p else 1
    nb = n // R
    i = np.arange(n)
    e = (i // nb) * ((i % nb) % ns) * (n // (ns * R))
    return np.exp(-2j * np.pi * e / n)


def dft_out(v, k, R):
    """Output k of a forward radix-R DFT (the kernel's dft_out)."""
    return sum(v[r] * np.exp(-2j * np.pi * ((r * k) % R) / R) for r in range(R))


def epass(load, store, n, tpb, R, ns):
    """One radix-R pass, one output per element e = t + tpb pos:
    pos = q ns R + k ns + jm reads butterfly j = q ns + jm's inputs."""
    nb = n // R
    for e in range(tpb * n):
        pos, t = e // tpb, e % tpb
        u = pos // ns
        jm = pos - u * ns
        q, k = u // R, u % R
        j = q * ns + jm
        v = [load(t, j + r * nb) for r in range(R)]
        store(t, pos, dft_out(v, k, R))


def cluster_model(x, n1, n2, C, back=False, scale=1.0):
    """Per CTA: stage columns into buf0[t lda + i]; column passes with the
    next pass's twiddle folded into each output and the four-step block
    (times the scale) into the last; rows: the first pass reads the owners'
    results, passes ping-pong the free buffer and the third, the last
    stores X[k1 + n1 k2]."""
    n = n1 * n2
    wa, wb = n2 // C, n1 // C
    lda, ldb = n1 | 1, n2 | 1
    tsz = max(wa * lda, wb * ldb)
    ra, rb = radix_code(n1), radix_code(n2)
    k = np.arange(n)
    blk = np.exp(-2j * np.pi * (((k // n1) * (k % n1)) % n) / n) * scale  # [n2][k1]
    cj = np.conj if back else (lambda z: z)
    bufs, results = [], []
    for c in range(C):  # columns
        b = [np.zeros(tsz, complex) for _ in range(3)]
        for e in range(n1 * wa):
            i, t = e // wa, e % wa
            b[0][t * lda + i] = cj(x[i * n2 + c * wa + t])
        src, dst, ns = 0, 1, 1
        sblk = blk[c * wa * n1:(c + 1) * wa * n1]
        for p, R in enumerate(ra):
            if p + 1 < len(ra):
                tw = pass_table(n1, ra, p + 1)
                st = lambda t, pos, v, dst=dst, tw=tw: b[dst].__setitem__(t * lda + pos, v * tw[pos])
            else:
                st = lambda t, pos, v, dst=dst: b[dst].__setitem__(t * lda + pos, v * sblk[t * n1 + pos])
            epass(lambda t, i, src=src: b[src][t * lda + i], st, n1, wa, R, ns)
            ns *= R
            src, dst = dst, src
        bufs.append(b)
        results.append(src)
    out = np.zeros(n, complex)
    for c in range(C):  # rows
        b = bufs[c]
        r0 = c * wb
        fa = results[c]
        g0, g1 = (1 if fa == 0 else 0), 2
        ns = 1
        for p, R in enumerate(rb):
            if p == 0:
                ld = lambda t, i: bufs[i // wa][results[i // wa]][(i % wa) * lda + r0 + t]
            else:
                ld = lambda t, i, src=g0: b[src][t * ldb + i]
            if p + 1 < len(rb):
                tw = pass_table(n2, rb, p + 1)
                dst = g0 if p == 0 else g1
                st = lambda t, pos, v, dst=dst, tw=tw: b[dst].__setitem__(t * ldb + pos, v * tw[pos])
            else:
                st = lambda t, pos, v: out.__setitem__(r0 + t + n1 * pos, cj(v))
            epass(ld, st, n2, wb, R, ns)
            if p > 0 and p + 1 < len(rb):
                g0, g1 = g1, g0
            ns *= R
        assert fa not in (g0, g1) or len(rb) == 1
    return out


@pytest.mark.parametrize("n1,n2,C", [(8, 8, 8), (32, 32, 8), (32, 32, 16), (16, 64, 8), (48, 48, 8), (64, 32, 16), (40, 56, 8)])
def test_cluster_model_matches_fft(n1, n2, C):
    rng = np.random.default_rng(n1 * 1000 + n2 + C)
    n = n1 * n2
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x)
    got = cluster_model(x, n1, n2, C)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12
    # backward: conj trick, the 1/n scale folded into the four-step block
    back = cluster_model(ref, n1, n2, C, back=True, scale=1.0 / n)
    assert np.linalg.norm(back - x) / np.linalg.norm(x) < 1e-12


@pytest.mark.parametrize("n1,n2,C", [(32, 32, 8), (128, 256, 16), (128, 128, 8), (16, 64, 8)])
def test_cluster_smem_layout_in_bounds(n1, n2, C):
    """Three buffers of max(wa lda, wb ldb) elements, the pass tables and
    the four-step block: every index a pass, the staging or the rows' first
    pass touches lies inside one buffer, and f64 fits a CTA's 227 KiB."""
    wa, wb = n2 // C, n1 // C
    lda, ldb = n1 | 1, n2 | 1
    tsz = max(wa * lda, wb * ldb)
    assert (wa - 1) * lda + n1 - 1 < tsz  # column sequences
    assert (wb - 1) * ldb + n2 - 1 < tsz  # row sequences
    assert (wa - 1) * lda + (C * wb - 1) < tsz  # rows' first pass reads (k1 < n1)
    tabs = (len(radix_code(n1)) - 1) * n1 + (len(radix_code(n2)) - 1) * n2 + wa * n1
    assert (3 * tsz + tabs) * 16 + 2 * 16 * 16 <= 227 * 1024


def test_radix_codes_fit_sixteen_passes():
    for n in (8, 16, 32, 48, 64, 216, 256, 1024, 4096, 3 ** 8, 2 ** 20):
        rs = radix_code(n)
        assert int(np.prod(rs)) == n and len(rs) <= 16


def test_cluster_table_blocks_partition():
    """Each CTA's block of the [n2][k1] four-step table holds exactly the
    twiddles of its columns."""
    n1, n2, C = 32, 32, 8
    n, wa = n1 * n2, n2 // C
    k = np.arange(n)
    tw = np.exp(-2j * np.pi * (((k // n1) * (k % n1)) % n) / n)
    for c in range(C):
        blk = tw[c * wa * n1:(c + 1) * wa * n1].reshape(wa, n1)
        col = np.arange(c * wa, (c + 1) * wa)[:, None]
        k1 = np.arange(n1)[None, :]
        assert np.allclose(blk, np.exp(-2j * np.pi * (col * k1) / n))


def test_fdiv_matches_floor_division():
    """q = (x m) >> 40, m = floor(2^40 / d) + 1 (k_cluster.cuh's FDiv) equals
    x // d for divisors below 2^19 and numerators below 2^21: every x that
    is one below a multiple of d (the hardest case) and random others."""
    rng = np.random.default_rng(0)
    ds = np.unique(np.concatenate([np.arange(1, 2049), rng.integers(1, 1 << 19, 4000), [(1 << 19) - 1]]))
    for d in ds.tolist():
        m = (1 << 40) // d + 1
        x = np.arange(d - 1, 1 << 21, d, dtype=np.uint64)  # k d - 1
        x = np.concatenate([x, rng.integers(0, 1 << 21, 64).astype(np.uint64)])
        q = (x * np.uint64(m)) >> np.uint64(40)
        assert np.array_equal(q, x // np.uint64(d)), d


def dft_part(v, k, h, R):
    """The kernel's dft_part: part h (0 real, 1 imaginary) of output k of a
    radix-R DFT from the parts alone, signs as the integer selects set them."""
    def comp(z, hh):
        return z.imag if hh else z.real

    def flip_if(x, cond):
        return -x if cond else x

    if R == 2:
        return comp(v[0], h) + flip_if(comp(v[1], h), k != 0)
    if R == 4:
        odd = (k & 1) != 0
        a = comp(v[0], h) + flip_if(comp(v[2], h), odd)
        hb = 1 - h if odd else h
        b = comp(v[1], hb) + flip_if(comp(v[3], hb), odd)
        return a + flip_if(b, (odd and h == 1) != ((k & 2) != 0))
    x = comp(v[0], h)
    for r in range(1, (R - 1) // 2 + 1):
        t = comp(v[r], h) + comp(v[R - r], h)
        d = comp(v[r], 1 - h) - comp(v[R - r], 1 - h)
        m = (r * k) % R
        c, sn = np.cos(2 * np.pi * m / R), np.sin(2 * np.pi * m / R)
        x = c * t + x
        x = flip_if(sn, h == 1) * d + x
    return x


@pytest.mark.parametrize("R", [2, 3, 4, 5, 7])
def test_dft_parts_match_complex_outputs(R):
    rng = np.random.default_rng(R)
    v = rng.standard_normal(R) + 1j * rng.standard_normal(R)
    for k in range(R):
        ref = dft_out(v, k, R)
        assert abs(dft_part(v, k, 0, R) - ref.real) < 1e-12
        assert abs(dft_part(v, k, 1, R) - ref.imag) < 1e-12


def test_twiddle_part_product():
    """Part h of x w from x_h, the partner's x_{1-h} and w: x_h w_re -+ x_{1-h} w_im."""
    rng = np.random.default_rng(5)
    x = complex(*rng.standard_normal(2))
    w = complex(*rng.standard_normal(2))
    parts = [x.real * w.real + (-(x.imag * w.imag)), x.imag * w.real + (x.real * w.imag)]
    assert abs(complex(*parts) - x * w) < 1e-12


# ---------------------------------------------------------------- real kinds
# The cluster form of Dct1D / Mdct1D (k_cluster.cu real_pre / real_post):
# a pre launch, the complex core on a cluster, a post launch. Restated here
# with numpy's FFT standing in for the core, the plan tables as k_tables.cu
# generates them, and checked against the oracle. DCT-III runs the core
# backward (conj . F . conj) on the unconjugated merge, where the one-CTA
# kernel runs it forward on the conjugated merge.

def _root(p, q):
    """exp(-2 pi i p / q)."""
    return np.exp(-2j * np.pi * (np.asarray(p) % q) / q)


def _tables_dct(n, dct_type):
    h = n // 2
    k = np.arange(h)
    w = _root(k, n)                      # (c, s) = (cos, -sin)
    c, s = w.real, w.imag
    coef = (0.5 * (1 - s) + 0.5j * c) if dct_type == 2 else (0.5 * (1 - s) - 0.5j * c)
    kk = np.arange(h + 1)
    om = np.conj(_root(kk, 4 * n)) if dct_type == 2 else _root(kk, 4 * n)
    return coef, om


def _dct2_cluster(x, scale, ortho):
    n = x.shape[-1]
    h = n // 2
    coef, om = _tables_dct(n, 2)

    def v(j):  # DctPackLoad::v
        return np.where(j < n // 2, x[np.minimum(2 * j, n - 1)], x[np.clip(2 * (n - 1 - j) + 1, 0, n - 1)])

    m = np.arange(h)
    re, im = v(2 * m), v(2 * m + 1)
    re = np.where(m == 0, re * ortho, re)
    z = np.fft.fft((re + 1j * im) * scale)   # the forward core
    out = np.empty(n)
    q2 = (n + 3) >> 2
    z0 = z[0]
    out[0] = z0.real + z0.imag
    out[h] = (z0.real - z0.imag) * om[h].real
    if n % 4 == 0:
        xq = z[q2] * om[q2]
        out[q2], out[n - q2] = xq.real, xq.imag
    for i in range(1, q2):
        zi, wc = z[i], np.conj(z[h - i])
        xx = coef[i] * (zi - wc)
        j = np.conj(zi - xx) * om[i]
        out[i], out[n - i] = j.real, j.imag
        kv = (wc + xx) * om[h - i]
        out[h - i], out[h + i] = kv.real, kv.imag
    return out


def _dct3_cluster(x, scale, ortho):
    n = x.shape[-1]
    h = n // 2
    coef, om = _tables_dct(n, 3)
    q = (n + 3) >> 2
    z = np.zeros(h, complex)
    zval, hval = x[0] * ortho, x[h] * om[h].real
    z[0] = (zval + hval) * scale + 1j * (zval - hval) * scale
    if n % 4 == 0:
        z[q] = (x[q] + 1j * x[n - q]) * om[q] * scale
    for i in range(1, q):
        j = np.conj((x[i] + 1j * x[n - i]) * om[i] * scale)
        kv = (x[h - i] + 1j * x[h + i]) * om[h - i] * scale
        xx = coef[i] * (j - kv)
        z[i] = j - xx
        z[h - i] = np.conj(kv + xx)
    u = np.fft.ifft(z) * h                   # the backward core, scale 1
    vv = np.conj(u)                          # k_post's conj_in: DctUnpackStore takes conj(u)
    out = np.empty(n)
    qh = h >> 1
    for m in range(h):                       # DctUnpackStore::store(t, m, vv[m]) writes conj(vv[m])
        re, im = vv[m].real, -vv[m].imag
        if m < qh:
            out[4 * m], out[4 * m + 2] = re, im
        elif (h & 1) and m == qh:
            out[2 * h - 2], out[2 * h - 1] = re, im
        else:
            i = h - 1 - m
            out[4 * i + 1], out[4 * i + 3] = im, re
    return out


def _mdct_geom(n):
    lenh = n >> 1
    lenq = lenh >> 1
    leno = lenq - (lenq >> 1)
    return lenh, lenq, leno, lenh + lenq, lenh + lenh + lenq


def _mdct_cluster(x, win, scale):
    n = x.shape[-1]
    q = n // 4
    tw = _root(8 * np.arange(q) + 1, 8 * n) * (2.0 / n) ** 0.25
    lenh, lenq, leno, len3q, len5q = _mdct_geom(n)
    z = np.empty(q, complex)
    for i in range(q):                       # MdctLoad
        k = 2 * i
        if i < leno:
            re = x[len3q - 1 - k] * win[len3q - 1 - k] + x[len3q + k] * win[len3q + k]
            im = x[lenq + k] * win[lenq + k] - x[lenq - 1 - k] * win[lenq - 1 - k]
        else:
            re = x[len3q - 1 - k] * win[len3q - 1 - k] - x[k - lenq] * win[k - lenq]
            im = x[lenq + k] * win[lenq + k] + x[len5q - 1 - k] * win[len5q - 1 - k]
        z[i] = (re + 1j * im) * tw[i]
    y = np.fft.fft(z)                        # the forward core
    out = np.empty(lenh)
    for i in range(q):                       # MdctStore
        r = y[i] * tw[i] * scale
        out[2 * i], out[lenh - 1 - 2 * i] = -r.real, r.imag
    return out


def _imdct_cluster(s, n, win, scale):
    q = n // 4
    tw = _root(8 * np.arange(q) + 1, 8 * n) * (2.0 / n) ** 0.25
    lenh, lenq, leno, len3q, len5q = _mdct_geom(n)
    z = np.array([(s[2 * i] + 1j * s[lenh - 1 - 2 * i]) * tw[i] * -2.0 for i in range(q)])  # ImdctLoad
    y = np.fft.fft(z)                        # the forward core
    out = np.empty(n)
    for i in range(q):                       # ImdctStore
        k = 2 * i
        r = y[i] * tw[i] * scale
        if i < leno:
            out[len3q - 1 - k] = r.real * win[len3q - 1 - k]
            out[len3q + k] = r.real * win[len3q + k]
            out[lenq + k] = -r.imag * win[lenq + k]
            out[lenq - 1 - k] = r.imag * win[lenq - 1 - k]
        else:
            out[len3q - 1 - k] = r.real * win[len3q - 1 - k]
            out[k - lenq] = -r.real * win[k - lenq]
            out[lenq + k] = -r.imag * win[lenq + k]
            out[len5q - 1 - k] = -r.imag * win[len5q - 1 - k]
    return out


@pytest.mark.parametrize("n", [16, 18, 40, 50, 128, 1152])
@pytest.mark.parametrize("ortho", [False, True])
def test_dct_cluster_form_model_matches_oracle(n, ortho):
    """N = 2 mod 4 (18, 50) runs the odd-half branches of the pre / post
    launches' formulas. The cluster path itself never takes them on the GPU
    (its split makes the core a multiple of 64); the one-CTA kernels, whose
    loops these restate, do."""
    import oracle
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, n)
    for method, sc in (("forward", 1.0), ("forwardu", np.sqrt(2.0 / n)), ("forwardn", 2.0 / n)):
        a2 = np.sqrt(0.5) if ortho else 1.0
        y2 = _dct2_cluster(x, sc, a2)
        r2 = oracle.dct1d(x, 2, ortho, method)
        assert np.linalg.norm(y2 - r2) / np.linalg.norm(r2) < 1e-12, ("II", method)
        a3 = np.sqrt(0.5) if ortho else 0.5
        y3 = _dct3_cluster(x, sc, a3)
        r3 = oracle.dct1d(x, 3, ortho, method)
        assert np.linalg.norm(y3 - r3) / np.linalg.norm(r3) < 1e-12, ("III", method)


@pytest.mark.parametrize("n", [16, 64, 2304])
def test_mdct_cluster_form_model_matches_oracle(n):
    import oracle
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, n)
    win = np.sin(np.pi * (np.arange(n) + 0.5) / n)
    for method, sc in (("forward", np.sqrt(n / 2.0)), ("forwardu", 1.0)):
        y = _mdct_cluster(x, win, sc)
        r = oracle.mdct1d(x, n, "sine", method)
        assert np.linalg.norm(y - r) / np.linalg.norm(r) < 1e-12, method
    s = rng.uniform(-1, 1, n // 2)
    for method, sc in (("backward", 1.0 / np.sqrt(n / 2.0)), ("backwardu", 1.0)):
        y = _imdct_cluster(s, n, win, sc)
        r = oracle.mdct1d(s, n, "sine", method)
        assert np.linalg.norm(y - r) / np.linalg.norm(r) < 1e-12, method


def _rfft_tables(n):
    h = n // 2
    w = _root(np.arange(h), n)
    c, s = w.real, w.imag
    return 0.5 * (1 - s) + 0.5j * c, 0.5 * (1 - s) - 0.5j * c   # RCOEF, RBCOEF


def _rfft_split_model(x, scale):
    """RFft1D forward in the cluster form: the half-length core on the
    real input read as complex pairs, then k_rfft_split."""
    n = x.shape[-1]
    h = n // 2
    coef, _ = _rfft_tables(n)
    z = np.fft.fft(x[0::2] + 1j * x[1::2])   # the forward core, scale 1
    q = (2 * h + 3) >> 2
    o = np.empty(h + 1, complex)
    o[0] = (z[0].real + z[0].imag) * scale
    o[h] = (z[0].real - z[0].imag) * scale
    if (2 * h) % 4 == 0:
        o[q] = np.conj(z[q]) * scale
    for i in range(1, q):
        xx = coef[i] * (z[i] - np.conj(z[h - i]))
        o[i] = (z[i] - xx) * scale
        o[h - i] = (z[h - i] + np.conj(xx)) * scale
    return o


def _rfft_merge_model(spec, n, s2):
    """RFft1D backward in the cluster form: k_rfft_merge (times 2 scale),
    then the core backward (conj . F . conj, scale 1); the complex result
    read as the N reals."""
    h = n // 2
    _, bcoef = _rfft_tables(n)
    q = (2 * h + 3) >> 2
    z = np.empty(h, complex)
    z[0] = (spec[0].real + spec[h].real) * 0.5 * s2 + 1j * (spec[0].real - spec[h].real) * 0.5 * s2
    if (2 * h) % 4 == 0:
        z[q] = np.conj(spec[q]) * s2
    for i in range(1, q):
        xx = bcoef[i] * (spec[i] - np.conj(spec[h - i]))
        z[i] = (spec[i] - xx) * s2
        z[h - i] = (spec[h - i] + np.conj(xx)) * s2
    u = np.fft.ifft(z) * h
    out = np.empty(n)
    out[0::2], out[1::2] = u.real, u.imag
    return out


@pytest.mark.parametrize("n", [16, 18, 128, 2304])
def test_rfft_cluster_form_model_matches_oracle(n):
    """The RFft1D cluster form's split (forward) and merge (backward) launches
    around the half-length core reproduce the oracle for every method scale
    (forward 1, 1/sqrt N, 1/N; backward 1/N, 1, 1/sqrt N; the merge takes
    twice the method's scale)."""
    import oracle
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, n)
    for method, sc in (("forward", 1.0), ("forwardu", 1 / np.sqrt(n)), ("forwardn", 1.0 / n)):
        ref = oracle.rfft1d(x, method)
        assert np.linalg.norm(_rfft_split_model(x, sc) - ref) / np.linalg.norm(ref) < 1e-12, method
    spec = np.fft.rfft(x)
    for method, sc in (("backward", 1.0 / n), ("backward0", 1.0), ("backwardu", 1 / np.sqrt(n))):
        ref = oracle.rfft1d(spec, method)
        assert np.linalg.norm(_rfft_merge_model(spec, n, 2 * sc) - ref) / np.linalg.norm(ref) < 1e-12, method
