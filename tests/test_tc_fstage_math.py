"""CPU checks of the algebra of the tensor-core F-stage (fstage_tc_kernel in
gcorr_gb300/csrc/fstage_tc.cu), restated in numpy with the kernel's own factorisation:

* sample n = n2 + 128 n1 of a window has rotator tsub[n2] tstep[n1];
* step 1 uses the window's A1 = Re / Im of W64^(n1 k1) tstep[n1] against the real levels, so
  D1[n2][k1] = sum_n1 l[n2 + 128 n1] W64^(n1 k1) tstep[n1];
* the twiddle epilogue multiplies by W8192^(n2 k1) fsubt[k1] tsub[n2], advanced along k1 by
  one complex multiply per step (the factor is geometric in k1);
* step 2 is the DFT128 over n2 of the first 64 rows k2, and the output factor is fstept[k2].

Channel k = k1 + 64 k2 (k < 4096) must equal the 8192-point DFT of the rotated window times
the frac-delay phase fsubt[k1] fstept[k2]; and the two recurrences, run in FP32 as the kernel
runs them, must stay within a few parts in 1e6 of the directly evaluated factors.
"""
import numpy as np

N1, N2, N = 64, 128, 8192
NCHAN = N // 2


def _tables(rng):
    """tsub[128], tstep[64], fsubt[64], fstept[64] as the staging computes them:
    exp(-2 pi i (c0 + k c1)), exp(-2 pi i k cstep), exp(+2 pi i k cf), exp(+2 pi i 64 k cf)."""
    c0, c1, cf = rng.uniform(0, 1), rng.uniform(-1e-4, 1e-4), rng.uniform(-1e-5, 1e-5)
    cstep = N2 * c1
    k128, k64 = np.arange(N2), np.arange(N1)
    tsub = np.exp(-2j * np.pi * (c0 + k128 * c1))
    tstep = np.exp(-2j * np.pi * k64 * cstep)
    fsubt = np.exp(2j * np.pi * k64 * cf)
    fstept = np.exp(2j * np.pi * 64 * k64 * cf)
    return tsub, tstep, fsubt, fstept


def test_four_step_with_folded_rotator_equals_the_direct_dft():
    rng = np.random.default_rng(5)
    levels = np.array([-3.3359, -1.0, 1.0, 3.3359])
    lv = levels[rng.integers(0, 4, N)]
    tsub, tstep, fsubt, fstept = _tables(rng)
    n = np.arange(N)
    rot = tsub[n % N2] * tstep[n // N2]
    k = np.arange(NCHAN)
    direct = np.fft.fft(lv * rot)[:NCHAN] * fsubt[k % N1] * fstept[k // N1]

    W64 = np.exp(-2j * np.pi * np.arange(N1) / N1)
    k1, n1 = np.arange(N1)[:, None], np.arange(N1)[None, :]
    A1 = W64[(n1 * k1) % N1] * tstep[None, :]                 # [k1][n1]
    B1 = lv.reshape(N1, N2).T                                   # [n2][n1] = l[n2 + 128 n1]
    D1 = B1 @ A1.T                                              # [n2][k1]
    n2 = np.arange(N2)[:, None]
    tw = np.exp(-2j * np.pi * n2 * np.arange(N1)[None, :] / N)  # W8192^(n2 k1)
    Y = (D1 * tw * fsubt[None, :] * tsub[:, None]).T            # [k1][n2]
    k2 = np.arange(N1)[:, None]
    W128 = np.exp(-2j * np.pi * (np.arange(N2)[None, :] * k2 % N2) / N2)  # [k2][n2], k2 < 64
    X = (Y @ W128.T) * fstept[None, :]                          # [k1][k2]
    four_step = X.T.reshape(-1)                                 # k = k1 + 64 k2
    assert np.allclose(four_step, direct, rtol=0, atol=1e-9 * np.abs(direct).max())


def _c64(z):
    return np.complex64(z)


def test_fp32_recurrences_stay_close_to_the_direct_factors():
    """The A1 entries advance along n1 by tstep[1] W64^k1 (8 steps per thread), the twiddle
    factors along k1 by W8192^n2 fsubt[1] (32 steps per thread), both in FP32."""
    rng = np.random.default_rng(6)
    tsub, tstep, fsubt, fstept = _tables(rng)
    W64 = np.exp(-2j * np.pi * np.arange(N1) / N1)
    worst = 0.0
    for k1 in range(N1):
        for c in range(8):
            st = _c64(_c64(tstep[1]) * _c64(W64[k1]))
            a = _c64(_c64(tstep[8 * c]) * _c64(W64[(8 * c * k1) % N1]))
            for e in range(8):
                n1 = 8 * c + e
                exact = W64[(n1 * k1) % N1] * tstep[n1]
                worst = max(worst, abs(complex(a) - exact))
                a = _c64(a * st)
    assert worst < 3e-6, worst
    worst = 0.0
    for n2 in range(N2):
        for half in range(2):
            r = _c64(_c64(np.exp(-2j * np.pi * n2 / N)) * _c64(fsubt[1]))
            wk = _c64(_c64(_c64(np.exp(-2j * np.pi * 32 * half * n2 / N)) * _c64(fsubt[32 * half])) * _c64(tsub[n2]))
            for k1 in range(32 * half, 32 * half + 32):
                exact = np.exp(-2j * np.pi * n2 * k1 / N) * fsubt[k1] * tsub[n2]
                worst = max(worst, abs(complex(wk) - exact))
                wk = _c64(wk * r)
    assert worst < 1e-5, worst
