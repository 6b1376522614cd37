"""The tensor-core F-stage (csrc/fstage_tc.cu): 8192-point windows of 2-bit real data, FP16 or
FP8 channelised output, the FFT as two DFT products on tcgen05 with FP16 operands.

Checked against the FP64 oracle (fxkernel/src/fxkernel.cpp:253-368 restated) at the FP16
tolerance of the other tests (the tensor-core FFT adds four FP16 roundings inside the FFT),
against the CUDA-core F-stage on the same input, with flagged edge FFTs and both rotators.
"""
import numpy as np
import pytest

from gcorr_gb300 import FxKernel, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP16_TOL = 1e-3
FP8_TOL = 0.12


def _run(w, inputs, poly, fso, **kw):
    fx = FxKernel(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, **kw)
    fx.setInputData(inputs)
    fx.setDelays(poly, fso)
    fx.process()
    v, c = fx.visibilities(), fx.baseline_counts()
    fx.close()
    return v, c


@pytest.mark.parametrize("precision", ["fp16", "fp8"])
@pytest.mark.parametrize("rotator", ["exact", "fxkernel"])
def test_tensor_fft_vs_fp64(precision, rotator):
    w = synth.Workload(nant=6, nchan=4096, nfft=20, bw_hz=256e6, rho=0.2, seed=61, offset_us=20.0)
    d = synth.generate(w)
    inputs = [x.numpy() for x in d["inputs"]]
    rot = O.ROT_EXACT if rotator == "exact" else O.ROT_FXKERNEL
    ref, rc = O.exact_process(O.config_from_workload(w, rot, True), inputs, d["poly"], d["fso"])
    assert (rc < w.nfft).any(), "some FFTs flagged"
    vis, counts = _run(w, inputs, d["poly"], d["fso"], precision=precision, rotator=rotator, fft_engine="tensor")
    assert np.array_equal(counts, rc)
    err = O.rel_rms_per_product(vis, ref)
    tol = FP16_TOL if precision == "fp16" else FP8_TOL
    assert err.max() < tol, (err.max(), float(np.median(err)))


@pytest.mark.parametrize("x_engine", ["tensor", "cuda_core"])
def test_tensor_fft_matches_cuda_core_fft(x_engine):
    """Same input through both F-stages at FP16, 16 antennas (the default workload's shape)."""
    w = synth.Workload(nant=16, nchan=4096, nfft=12, bw_hz=256e6, rho=0.05, seed=62)
    d = synth.generate(w)
    inputs = [x.numpy() for x in d["inputs"]]
    v_tc, c_tc = _run(w, inputs, d["poly"], d["fso"], precision="fp16", fft_engine="tensor", x_engine=x_engine)
    v_cc, c_cc = _run(w, inputs, d["poly"], d["fso"], precision="fp16", fft_engine="cuda_core", x_engine=x_engine)
    ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), inputs, d["poly"], d["fso"])
    assert np.array_equal(c_tc, rc) and np.array_equal(c_cc, rc)
    e_tc = O.rel_rms_per_product(v_tc, ref)
    e_cc = O.rel_rms_per_product(v_cc, ref)
    assert e_tc.max() < FP16_TOL and e_cc.max() < FP16_TOL, (e_tc.max(), e_cc.max())
    assert O.rel_rms_per_product(v_tc, v_cc).max() < FP16_TOL


def test_tensor_fft_blocks_and_device_inputs():
    """Several FFT blocks (fft_block < nfft), device-resident inputs, a tone in one channel."""
    import torch
    w = synth.Workload(nant=4, nchan=4096, nfft=40, bw_hz=256e6, rho=0.1, seed=63, tone_amp=0.3, tone_chan=777)
    d = synth.generate(w)
    inputs = [x.numpy() for x in d["inputs"]]
    dev = [torch.from_numpy(x).cuda() for x in inputs]
    ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), inputs, d["poly"], d["fso"])
    vis, counts = _run(w, dev, d["poly"], d["fso"], precision="fp16", fft_engine="tensor", fft_block=16)
    assert np.array_equal(counts, rc)
    assert O.rel_rms_per_product(vis, ref).max() < FP16_TOL
