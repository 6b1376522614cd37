"""CPU checks of the index arithmetic of the packed-pair F-stage (fstage_pair_kernel in
gcorr_gb300/csrc/fstage.cu), restated in numpy with the kernel's own index expressions:

* pass 0: thread iv takes samples n = iv + 256 r (r < 32) and forms the two lanes
  A = x[n] + x[n + M] and B = (x[n] - x[n + M]) W_N^(iv) W_32^r of the M = N/2-point sub-FFTs;
* three radix-16 Stockham passes over the padded pair buffer (one slot of padding per 16),
  with the pass twiddles read from the [r][k] tables make_twiddles builds;
* sub-FFT bin kk = iv + 256 r of lane A is channel 2 kk, of lane B channel 2 kk + 1; real data
  keeps r < 8 (channels below N/2).

The transform must equal numpy's FFT, and every buffer index must stay inside the buffer.

Also the compact baseline spans of the 33-64 antenna X-stage's staged epilogue
(xstage_tc_big2_kernel in gcorr_gb300/csrc/xstage_tc.cu).
"""
import numpy as np

N, M, NT, R, PAD = 8192, 4096, 256, 16, 16
NB = M // R          # butterflies per pass, one per thread
NB0 = N // 32        # pass-0 sample stride
PADM = M + M // PAD  # pair slots in shared memory


def _dft16(u):
    return np.fft.fft(u, axis=1)  # [thread][r][lane] -> DFT over r


def _pair_fft(x):
    WN = np.exp(-2j * np.pi * np.arange(N) / N)
    WM = np.exp(-2j * np.pi * np.arange(M) / M)
    tab1 = np.array([[WM[(16 * r * k) % M] for k in range(16)] for r in range(16)])    # [r][k]
    tab2 = np.array([[WM[(r * iv) % M] for iv in range(256)] for r in range(16)])     # [r][iv]
    iv = np.arange(NT)[:, None]
    r = np.arange(R)[None, :]
    buf = np.full((PADM, 2), np.nan + 0j)
    # pass 0
    x0, x1 = x[iv + NB0 * r], x[iv + NB0 * (r + R)]
    w = WN[iv] * np.exp(-2j * np.pi * r / 32)                       # W_N^iv W_32^r
    u = np.stack([x0 + x1, (x0 - x1) * w], axis=2)
    u = _dft16(u)
    idx0 = iv * (R + 1) + r
    assert idx0.max() < PADM
    buf[idx0] = u
    # pass 1: radix 16, span 16, in place
    ld = (iv + iv // PAD) + r * (NB + NB // PAD)
    assert ld.max() < PADM
    u = buf[ld]
    k = iv & (R - 1)
    u = u * tab1[r, k][:, :, None]
    u = _dft16(u)
    j = (iv - k) * R + k
    st = (j + j // PAD) + r * (R + R // PAD)
    assert st.max() < PADM and len(np.unique(st)) == NT * R
    buf[st] = u
    # pass 2: radix 16, span 256
    u = buf[ld]
    u = u * tab2[r, iv][:, :, None]
    u = _dft16(u)
    X = np.empty(N, complex)
    kk = iv + r * NB
    X[2 * kk] = u[:, :, 0]
    X[2 * kk + 1] = u[:, :, 1]
    return X


def test_pair_plan_8192_matches_numpy_fft():
    rng = np.random.default_rng(11)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    X = _pair_fft(x)
    ref = np.fft.fft(x)
    assert np.abs(X - ref).max() / np.abs(ref).max() < 1e-12


def test_pair_plan_real_band_is_the_first_eight_outputs():
    # channels below N/2 (a real band) come from r < 8 of the last pass, both lanes
    kk = np.arange(NT)[:, None] + np.arange(8)[None, :] * NB
    ch = np.concatenate([2 * kk.ravel(), 2 * kk.ravel() + 1])
    assert np.array_equal(np.sort(ch), np.arange(N // 2))


def test_pair_plan_twiddle_exponents_stay_in_the_tables():
    # make_twiddles stores W_M^(16 r k) for k < 16 and W_M^(r iv) for iv < 256, r < 16
    assert 16 * 15 * 15 < M and 15 * 255 < M
    # pass-0 twiddle W_N^(iv + 256 r) = W_N^iv W_32^r for every sample pair of every thread
    iv = np.arange(NT)[:, None]
    r = np.arange(R)[None, :]
    lhs = np.exp(-2j * np.pi * (iv + NB0 * r) / N)
    rhs = np.exp(-2j * np.pi * iv / N) * np.exp(-2j * np.pi * r / 32)
    assert np.abs(lhs - rhs).max() < 1e-12


def _baseline_index(j, k, nant):
    """Crosses in j-major order, then autos (gcorr_gb300/csrc/gxc_internal.h baseline_index)."""
    if j == k:
        return nant * (nant - 1) // 2 + j
    return j * nant - j * (j + 1) // 2 + (k - j - 1)


def _big2_span(nant, autos, ja, jb):
    """Big2Span of xstage_tc_big2_kernel: cross_start, ncr, nloc for antennas [ja, jb)."""
    m = nant - 1
    cross_start = ja * m - ja * (ja - 1) // 2
    ncr = jb * m - jb * (jb - 1) // 2 - cross_start
    return cross_start, ncr, ncr + (jb - ja if autos else 0)


def test_big2_baseline_spans_cover_every_baseline_once():
    """33..64 antennas: the top CTAs own the baselines (j, k), j < 32, the bottom CTA those with
    j >= 32.  Each stages its outputs at a compact index loc (cross baselines from cross_start,
    then its autos) and maps loc back to the baseline when adding into the accumulators.  Every
    baseline must be staged by exactly one kind, in range, and map back to itself."""
    for nant in range(33, 65):
        ncross = nant * (nant - 1) // 2
        for autos in (True, False):
            seen = {}
            for kind, (ja, jb) in (("top", (0, 32)), ("bottom", (32, nant))):
                cross_start, ncr, nloc = _big2_span(nant, autos, ja, jb)
                s_lo = 0 if kind == "top" else 64
                # the (j, k) the kernel's epilogue outputs: rows s1 >= s_lo, columns s2 >= s_lo (the
                # bottom CTA's D_bot) or all (the top CTA's D_top), j <= k
                for j in range(ja, jb):
                    for k in range(max(j, s_lo // 2), nant):
                        if j == k and not autos:
                            continue
                        bl = _baseline_index(j, k, nant)
                        loc = bl - cross_start if j < k else ncr + (j - ja)
                        assert 0 <= loc < nloc, (nant, autos, kind, j, k, loc, nloc)
                        back = cross_start + loc if loc < ncr else ncross + ja + (loc - ncr)
                        assert back == bl, (nant, kind, j, k)
                        assert bl not in seen, (nant, j, k, seen.get(bl), kind)
                        seen[bl] = kind
            nbl = ncross + (nant if autos else 0)
            assert sorted(seen) == list(range(nbl)), nant


def test_small_n_epilogue_stages_every_output_once():
    """1..32 antennas: the FP16 / FP8 X-stage's segment epilogue (xstage_tc_kernel), restated with
    the kernel's own index expressions.  Warp w reads TMEM lane quarter w % 4 of the groups
    G = w / 4, w / 4 + 2; lane row = 32 (w % 4) + lane is stream s1, part (re / im) of channel
    block my_gi; each 16-column piece gives a row 4 of its block's 8 streams.  Every output
    (baseline, product, channel of the CTA) must be staged exactly once, inside the staging area."""
    NG = 4
    for nant in range(1, 33):
        n = 2 * nant
        R = 16
        while R < 2 * n:
            R *= 2
        g = 128 // R
        CS = NG * g
        lcs = CS.bit_length() - 1
        for autos in (True, False):
            nbl = nant * (nant - 1) // 2 + (nant if autos else 0)
            nent = nbl * 4 * CS
            hits = np.zeros(nent, dtype=np.int64)
            for warp in range(8):
                wq = warp & 3
                for G in range(warp >> 2, NG, 2):
                    for lane in range(32):
                        row = 32 * wq + lane
                        my_gi = row // R
                        r = row - my_gi * R
                        s1, part1 = r >> 1, r & 1
                        gi0 = (32 * wq) // R
                        col0 = gi0 * R
                        clen = max(R, 32)
                        j, l = s1 >> 1, s1 & 1
                        cl = G * g + my_gi
                        for pc in range(0, clen, 16):
                            col = col0 + pc
                            if col < my_gi * R or col >= (my_gi + 1) * R or s1 >= n:
                                continue
                            s2b = (col - my_gi * R) >> 1
                            for qq in range(4):
                                s2 = s2b + qq + 4 * part1
                                if s2 >= n:
                                    continue
                                k, m = s2 >> 1, s2 & 1
                                if j > k or (j == k and not autos):
                                    continue
                                bl = _baseline_index(j, k, nant)
                                e = ((bl * 4 + 2 * l + m) << lcs) + cl
                                assert 0 <= e < nent, (nant, autos, e, nent)
                                hits[e] += 1
            assert (hits == 1).all(), (nant, autos, int((hits == 0).sum()), int((hits > 1).sum()))


def test_split_epilogue_stages_every_output_once():
    """1..32 antennas, FP32 data: the split X-stage's final staging (xstage_tc_split_kernel).
    Epilogue warp quarter qd, lane row = 32 qd + lane (stream s1, part of block my_gi); its sums
    acc[G][a][qq] are the streams s2 = 8a + qq + 4 part of its own block.  Every output must be
    staged exactly once at ((baseline * 4 + product) * CS + channel)."""
    NG = 2
    for nant in range(1, 33):
        n = 2 * nant
        R = 16
        while R < 2 * n:
            R *= 2
        GCH = 128 // R
        CS = NG * GCH
        PP = R // 16
        for autos in (True, False):
            nbl = nant * (nant - 1) // 2 + (nant if autos else 0)
            nent = nbl * 4 * CS
            hits = np.zeros(nent, dtype=np.int64)
            for qd in range(4):
                for lane in range(32):
                    row = 32 * qd + lane
                    my_gi = row // R
                    r = row - my_gi * R
                    s1, part1 = r >> 1, r & 1
                    if s1 >= n:
                        continue
                    j, l = s1 >> 1, s1 & 1
                    for G in range(NG):
                        cl = G * GCH + my_gi
                        for a in range(PP):
                            for qq in range(4):
                                s2 = 8 * a + qq + 4 * part1
                                if s2 >= n:
                                    continue
                                k, m = s2 >> 1, s2 & 1
                                if j > k or (j == k and not autos):
                                    continue
                                e = (_baseline_index(j, k, nant) * 4 + 2 * l + m) * CS + cl
                                assert 0 <= e < nent
                                hits[e] += 1
            assert (hits == 1).all(), (nant, autos, int((hits == 0).sum()), int((hits > 1).sum()))
