"""GPU tests of the X-stage engines through gxc_xcorr.

Known-answer tests follow the reference's X-stage unit tests
(gcorr/test/unit.cc:73-159): complex data with small integer components
(uniform in [-5, 5]) so every product and sum is exact in FP32 (and in FP16),
compared for exact equality with a CPU triple loop (unit.cc:41-71: sum of
u*conj(v) over the FFTs, divided by nfft).  Same shapes as the reference:
(nant 3, fftwidth 512, nchan 256, nfft 4), (5, 1024, 1024, 100), (3, 1024, 512, 3000).
"""
import ctypes as C

import numpy as np
import pytest

import gcorr_gb300 as G
from gcorr_gb300 import _lib as L
from gcorr_gb300 import FxKernel, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

KAT_SHAPES = [(3, 512, 256, 4), (5, 1024, 1024, 100), (3, 1024, 512, 3000)]
# beyond the reference's shapes: 33..64 antennas (split-M tensor kernel)
BIG_KAT = (48, 256, 128, 70)


def cint_data(n, seed=12345):
    rng = np.random.default_rng(seed)
    return (rng.integers(-5, 6, n) + 1j * rng.integers(-5, 6, n)).astype(np.complex64)


def expected_crosscorraccum(data, nant, nfft, nchan, fftwidth, autos=False):
    """CPU triple loop of gcorr/test/unit.cc:41-71 (plus autos when asked)."""
    d = data.reshape(nant, 2, nfft, fftwidth)[..., :nchan].astype(np.complex128)
    out = []
    pairs = [(i, j) for i in range(nant - 1) for j in range(i + 1, nant)]
    if autos:
        pairs += [(i, i) for i in range(nant)]
    for i, j in pairs:
        for pi in range(2):
            for pj in range(2):
                out.append((d[i, pi] * np.conj(d[j, pj])).sum(axis=0) / nfft)
    return np.array(out, dtype=np.complex128).reshape(len(pairs), 4, nchan)


def xcorr(data, nant, nfft, nchan, fftwidth, precision, engine, autos=False):
    nbl = nant * (nant - 1) // 2 + (nant if autos else 0)
    out = np.zeros((nbl, 4, nchan), dtype=np.complex64)
    st = G.lib().gxc_xcorr(C.c_void_p(data.ctypes.data), nant, nfft, nchan, fftwidth, precision, engine,
                           int(autos), C.c_void_p(out.ctypes.data), None)
    assert st == L.GXC_OK, L.status_name(st)
    return out


# integers in [-5, 5] are exact in FP16 and in FP8 E4M3, so every engine must match exactly
ENGINES = [("fp32-cuda-core", L.GXC_PRECISION_FP32, L.GXC_XENGINE_CUDA_CORE),
           ("fp32-tensor-split", L.GXC_PRECISION_FP32, L.GXC_XENGINE_TENSOR),
           ("fp16-cuda-core", L.GXC_PRECISION_FP16, L.GXC_XENGINE_CUDA_CORE),
           ("fp16-tensor", L.GXC_PRECISION_FP16, L.GXC_XENGINE_TENSOR),
           ("fp8-cuda-core", L.GXC_PRECISION_FP8, L.GXC_XENGINE_CUDA_CORE),
           ("fp8-tensor", L.GXC_PRECISION_FP8, L.GXC_XENGINE_TENSOR)]


@pytest.mark.parametrize("shape", KAT_SHAPES)
@pytest.mark.parametrize("name,prec,eng", ENGINES)
def test_xstage_known_answer_exact(shape, name, prec, eng):
    nant, fftwidth, nchan, nfft = shape
    data = cint_data(2 * nant * fftwidth * nfft)
    exp = expected_crosscorraccum(data, nant, nfft, nchan, fftwidth).astype(np.complex64)
    got = xcorr(data, nant, nfft, nchan, fftwidth, prec, eng)
    assert np.array_equal(got, exp), (name, np.abs(got - exp).max())


@pytest.mark.parametrize("nant", [1, 2, 4, 7, 8, 16, 32, 33, 48, 64])
def test_tensor_vs_cuda_core_with_autos(nant):
    nchan, fftwidth, nfft = 128, 256, 300
    rng = np.random.default_rng(nant)
    n = 2 * nant * fftwidth * nfft
    data = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
    a = xcorr(data, nant, nfft, nchan, fftwidth, L.GXC_PRECISION_FP16, L.GXC_XENGINE_TENSOR, autos=True)
    b = xcorr(data, nant, nfft, nchan, fftwidth, L.GXC_PRECISION_FP16, L.GXC_XENGINE_CUDA_CORE, autos=True)
    ref = expected_crosscorraccum(data, nant, nfft, nchan, fftwidth, autos=True)
    assert O.rel_rms(a, b) < 1e-5
    assert O.rel_rms_per_product(a, ref).max() < 2e-3


def test_full_pipeline_tensor_fp16_vs_fp64():
    w = synth.Workload(nant=6, nchan=1024, nfft=100, bw_hz=64e6, rho=0.05, seed=61)
    d = synth.generate(w)
    inputs = [x.numpy() for x in d["inputs"]]
    ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), inputs, d["poly"], d["fso"])
    out = {}
    for eng in ("tensor", "cuda_core"):
        fx = FxKernel(w.nant, w.nchan, w.nfft, 2, w.lo_hz, w.bw_hz, False, precision="fp16", x_engine=eng,
                      fft_block=48)
        fx.setInputData(inputs)
        fx.setDelays(d["poly"], d["fso"])
        fx.process()
        out[eng] = fx.visibilities()
        assert np.array_equal(fx.baseline_counts(), rc)
        fx.close()
    assert O.rel_rms_per_product(out["tensor"], ref).max() < 1e-3
    assert O.rel_rms(out["tensor"], out["cuda_core"]) < 1e-5


def test_tensor_is_default_for_fp16():
    fx = FxKernel(4, 256, 8, 2, 8.4e9, 32e6, False, precision="fp16")
    d = synth.random_bytes(synth.Workload(nant=4, nchan=256, nfft=8, bw_hz=32e6))
    fx.setInputData([x.numpy() for x in d["inputs"]])
    fx.setDelays(d["poly"], d["fso"])
    fx.process()
    v = fx.visibilities()
    assert np.isfinite(v).all()
    fx.close()


@pytest.mark.parametrize("nant", [1, 3, 8, 16, 32])
def test_tensor_split_fp32_matches_cuda_core_fp32(nant):
    """FP32 data: the TF32 hi/lo split on tensor cores agrees with FP32 FMAs to FP32 accuracy."""
    nchan, fftwidth, nfft = 128, 256, 200
    rng = np.random.default_rng(100 + nant)
    n = 2 * nant * fftwidth * nfft
    data = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64) * np.float32(37.0)
    a = xcorr(data, nant, nfft, nchan, fftwidth, L.GXC_PRECISION_FP32, L.GXC_XENGINE_TENSOR, autos=True)
    b = xcorr(data, nant, nfft, nchan, fftwidth, L.GXC_PRECISION_FP32, L.GXC_XENGINE_CUDA_CORE, autos=True)
    ref = expected_crosscorraccum(data, nant, nfft, nchan, fftwidth, autos=True)
    assert O.rel_rms_per_product(a, ref).max() < 1e-5
    assert O.rel_rms_per_product(b, ref).max() < 1e-5


@pytest.mark.parametrize("name,prec,eng", [("fp32-cuda-core", L.GXC_PRECISION_FP32, L.GXC_XENGINE_CUDA_CORE),
                                           ("fp16-tensor", L.GXC_PRECISION_FP16, L.GXC_XENGINE_TENSOR),
                                           ("fp8-tensor", L.GXC_PRECISION_FP8, L.GXC_XENGINE_TENSOR)])
@pytest.mark.parametrize("autos", [True, False])
def test_xstage_known_answer_exact_many_antennas(name, prec, eng, autos):
    """48 antennas: the split-M tensor kernel (top and bottom CTAs, each staging its own span of
    baselines before the accumulator adds), with and without autos."""
    nant, fftwidth, nchan, nfft = BIG_KAT
    data = cint_data(2 * nant * fftwidth * nfft, seed=77)
    exp = expected_crosscorraccum(data, nant, nfft, nchan, fftwidth, autos=autos).astype(np.complex64)
    got = xcorr(data, nant, nfft, nchan, fftwidth, prec, eng, autos=autos)
    assert np.array_equal(got, exp), (name, np.abs(got - exp).max())


@pytest.mark.parametrize("nant", [1, 2, 5, 8, 16, 17, 32, 33, 64])
def test_fp8_tensor_vs_cuda_core(nant):
    """The same E4M3 data through kind::f8f6f4 MMAs and through FP32 FMAs."""
    nchan, fftwidth, nfft = 128, 256, 700  # several 128-FFT stages plus a partial one
    rng = np.random.default_rng(300 + nant)
    n = 2 * nant * fftwidth * nfft
    data = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64) * np.float32(3.0)
    a = xcorr(data, nant, nfft, nchan, fftwidth, L.GXC_PRECISION_FP8, L.GXC_XENGINE_TENSOR, autos=True)
    b = xcorr(data, nant, nfft, nchan, fftwidth, L.GXC_PRECISION_FP8, L.GXC_XENGINE_CUDA_CORE, autos=True)
    assert O.rel_rms(a, b) < 1e-5


@pytest.mark.parametrize("cplx", [False, True])
def test_full_pipeline_fp8_vs_fp64(cplx):
    """FP8 (E4M3) channelised data end to end: error against the FP64 oracle, measured.
    E4M3 keeps 3 mantissa bits (rounding error up to 2^-4 relative per component); with
    200 FFTs the cross products land near 2-3 % relative RMS and the autos near 0.3 %."""
    if cplx:
        w = synth.Workload(nant=6, nchan=512, nfft=200, nbit=8, is_complex=True, bw_hz=32e6, rho=0.05, seed=64)
    else:
        w = synth.Workload(nant=6, nchan=1024, nfft=200, bw_hz=64e6, rho=0.05, seed=63)
    d = synth.generate(w)
    inputs = [x.numpy() for x in d["inputs"]]
    ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), inputs, d["poly"], d["fso"])
    out = {}
    for eng in ("tensor", "cuda_core"):
        fx = FxKernel(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, precision="fp8",
                      x_engine=eng)
        fx.setInputData(inputs)
        fx.setDelays(d["poly"], d["fso"])
        fx.process()
        out[eng] = fx.visibilities()
        assert np.array_equal(fx.baseline_counts(), rc)
        fx.close()
    err = O.rel_rms_per_product(out["tensor"], ref)
    ncross = w.nant * (w.nant - 1) // 2
    assert err[:ncross].max() < 0.06, err[:ncross].max()
    assert err[ncross:][:, [1, 2]].max() < 0.06, err[ncross:].max()  # cross-hand autos behave like crosses
    assert err[ncross:][:, [0, 3]].max() < 0.01, err[ncross:].max()  # power spectra
    assert O.rel_rms(out["tensor"], out["cuda_core"]) < 1e-5
