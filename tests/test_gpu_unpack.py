"""GPU decode of the packed input, bit for bit against the reference's unpack.

The F-stage kernels decode the packed window inside their first FFT pass.
``gxc_probe_unpack`` runs the same kernel templates with a probe write of every
decoded sample before the fringe rotation, so this test sees the values the
FFT starts from.  Each case compares them with the oracle's restatement of
``lut2bit`` / ``unpackReal2bit`` (fxkernel/src/fxkernel.cpp:15-28, :443-476),
itself pinned to the level table in tests/golden/lut2bit.npy, and with the
8-bit complex layout (int8 A.re, A.im, B.re, B.im per time sample): every
float's bits must match, for every kernel family (256..32768 points, FP32 and
FP16-buffer kernels, and the tensor-core F-stage of 8192-point 2-bit windows),
at odd and even window offsets, with all 256 byte values inside the decoded
windows.  Flagged windows must stay untouched.
"""
import ctypes as C

import numpy as np
import pytest

from gcorr_gb300 import FxKernel
from gcorr_gb300 import _lib as L
from oracle import oracle as O

pytestmark = pytest.mark.gpu

BW = 64e6
NANT, NFFT = 3, 4

# (FFT length, complex, precision, F-stage engine): one case per kernel family and input format.
# 8192-point 2-bit FP16 / FP8 runs the tensor-core F-stage by default (its own decode loop).
CASES = [
    (256, False, "fp32", "auto"), (2048, False, "fp32", "auto"), (4096, False, "fp16", "auto"),
    (8192, False, "fp32", "auto"), (8192, False, "fp8", "auto"), (8192, False, "fp16", "auto"),
    (8192, False, "fp16", "cuda_core"), (16384, False, "fp32", "auto"), (16384, False, "fp16", "auto"),
    (32768, False, "fp32", "auto"), (32768, False, "fp16", "auto"),
    (256, True, "fp32", "auto"), (1024, True, "fp32", "auto"), (8192, True, "fp32", "auto"),
    (16384, True, "fp32", "auto"), (16384, True, "fp16", "auto"), (32768, True, "fp32", "auto"),
    (32768, True, "fp8", "auto"),
]


def _delays(is_complex):
    """Negative delays of a few samples, a rate and an acceleration: window offsets of both
    parities that move from FFT to FFT, and a flagged last window for the drifting antennas."""
    ts = 1.0 / BW if is_complex else 1.0 / (2.0 * BW)
    poly = np.array([[0.0, 0.0, -1.0 * ts],
                     [0.0, 2.6 * ts, -2.0 * ts],
                     [1.0e-3 * ts, -1.3 * ts, -7.0 * ts]])
    return poly, np.zeros(NANT)


def _inputs(nbytes, seed):
    """Blocks of random permutations of 0..255: every 256-byte block holds every byte value."""
    rng = np.random.default_rng(seed)
    nblk = (nbytes + 255) // 256
    return [np.concatenate([rng.permutation(256) for _ in range(nblk)]).astype(np.uint8)[:nbytes]
            for _ in range(NANT)]


@pytest.mark.parametrize("F,is_complex,precision,fft_engine", CASES)
def test_gpu_unpack_bit_exact(F, is_complex, precision, fft_engine):
    import torch
    nchan = F if is_complex else F // 2
    nbit = 8 if is_complex else 2
    fx = FxKernel(NANT, nchan, NFFT, nbit, 8.4e9, BW, is_complex, precision=precision, device=0,
                  fft_engine=fft_engine)
    try:
        inputs = _inputs(fx.bytes_per_antenna, seed=F + int(is_complex))
        dev = [torch.from_numpy(x).cuda() for x in inputs]
        poly, fso = _delays(is_complex)
        fx.setInputData(dev)
        fx.setDelays(poly, fso)
        got = np.zeros((NANT, 2, NFFT, F), dtype=np.complex64)
        st = L.lib().gxc_probe_unpack(fx._h, C.c_void_p(got.ctypes.data))
        L.check(st, fx._h, "gxc_probe_unpack")
        flags = fx.valid_flags()
    finally:
        fx.close()

    cfg = O.make_config(NANT, nchan, NFFT, nbit, is_complex, 8.4e9, BW)
    seen = np.zeros(256, dtype=bool)
    parities = set()
    nvalid = 0
    for a in range(NANT):
        for t in range(NFFT):
            g = O.geometry(cfg, poly[a], fso[a], t)
            assert int(flags[a, t]) == int(g.valid), (a, t)
            if not g.valid:
                assert np.isnan(got[a, :, t].view(np.float32)).all(), "flagged window was written"
                continue
            nvalid += 1
            parities.add(g.offset & 1)
            p0, p1 = O.unpack(cfg, inputs[a], g.offset, F)
            for pol, ref in ((0, p0), (1, p1)):
                gv = got[a, pol, t]
                if not np.array_equal(gv.view(np.uint32), ref.astype(np.complex64).view(np.uint32)):
                    bad = np.nonzero(gv != ref)[0]
                    raise AssertionError(f"ant {a} pol {pol} FFT {t} offset {g.offset}: first mismatch at sample "
                                         f"{bad[0]}: {gv[bad[0]]} vs {ref[bad[0]]} ({len(bad)} samples differ)")
            if is_complex:
                seen[inputs[a][4 * g.offset:4 * (g.offset + F)]] = True
            else:
                seen[inputs[a][g.offset // 2:(g.offset + F + 1) // 2]] = True
    assert nvalid >= NANT * NFFT - 3
    assert parities == {0, 1}, "windows at both odd and even offsets"
    assert seen.all(), "every byte value decoded"
