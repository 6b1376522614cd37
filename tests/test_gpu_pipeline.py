"""GPU tests of streaming ingest (gxc_pipeline_*), long integration and linear->circular conversion."""
import numpy as np
import pytest
import torch

from gcorr_gb300 import FxKernel, synth
from gcorr_gb300.pipeline import Pipeline, lin2circ
from oracle import oracle as O

pytestmark = pytest.mark.gpu

W = synth.Workload(nant=5, nchan=512, nfft=60, bw_hz=32e6, seed=21)


def _subints(n, w=W):
    subs = []
    for k in range(n):
        d = synth.random_bytes(synth.Workload(**{**w.__dict__, "seed": w.seed + 17 * k}))
        d["inputs"] = [x.pin_memory() for x in d["inputs"]]
        subs.append(d)
    return subs


def _single(w, d, **kw):
    fx = FxKernel(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, **kw)
    fx.setInputData([x.numpy() for x in d["inputs"]])
    fx.setDelays(d["poly"], d["fso"])
    fx.process()
    v = fx.visibilities()
    fx.close()
    return v


@pytest.mark.parametrize("slots", [1, 2, 3])
def test_pipeline_matches_single_subints(slots):
    subs = _subints(5)
    p = Pipeline(W.nant, W.nchan, W.nfft, W.nbit, W.lo_hz, W.bw_hz, W.is_complex, slots=slots)
    outs = [torch.zeros((p.nbl, 4, W.nchan), dtype=torch.complex64).pin_memory() for _ in subs]
    seqs = [p.submit(d["inputs"], d["poly"], d["fso"], out=o) for d, o in zip(subs, outs)]
    assert seqs == list(range(len(subs)))
    p.wait(seqs[-1])
    total = np.zeros((p.nbl, 4, W.nchan), np.complex128)
    for d, o in zip(subs, outs):
        ref = _single(W, d)
        assert np.array_equal(o.numpy(), ref)
        total += ref
    integ, n = p.integration(reset=True)
    assert n == len(subs)
    assert O.rel_rms(integ, total) < 1e-6
    integ2, n2 = p.integration()
    assert n2 == 0 and not integ2.any()
    p.close()


def test_pipeline_chunked_input_matches_single():
    """8.6 MB per antenna and sub-integration: the pipeline loads it in eight time-ordered chunks
    and each of the nine F-stage blocks waits only for the chunk that holds its windows.  Delays of
    both signs, swept by up to four FFTs across the sub-integration: the visibilities must equal
    single process() calls bit for bit."""
    w = synth.Workload(nant=4, nchan=4096, nfft=2100, bw_hz=64e6, seed=33, offset_us=60.0)
    subs = _subints(3, w)
    for k, d in enumerate(subs):
        poly = np.array(d["poly"], dtype=np.float64)
        poly[:, 1] += np.array([4.0, -4.0, 2.0, -1.0]) * (k - 1 if k != 1 else 0.5) * w.fft_time / w.nfft
        d["poly"] = poly
    p = Pipeline(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, slots=2, integrate=False,
                 fft_block=256)
    outs = [torch.zeros((p.nbl, 4, w.nchan), dtype=torch.complex64).pin_memory() for _ in subs]
    for d, o in zip(subs, outs):
        p.submit(d["inputs"], d["poly"], d["fso"], out=o)
    p.sync()
    for d, o in zip(subs, outs):
        assert np.array_equal(o.numpy(), _single(w, d, fft_block=256))
    p.close()


def test_pipeline_device_output_and_8bit():
    w = synth.Workload(nant=3, nchan=256, nfft=40, nbit=8, is_complex=True, bw_hz=32e6, seed=4)
    subs = _subints(3, w)
    p = Pipeline(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, slots=2, integrate=False,
                 precision="fp16")
    outs = [torch.zeros((p.nbl, 4, w.nchan), dtype=torch.complex64, device="cuda") for _ in subs]
    for d, o in zip(subs, outs):
        p.submit(d["inputs"], d["poly"], d["fso"], out=o)
    p.sync()
    for d, o in zip(subs, outs):
        assert np.array_equal(o.cpu().numpy(), _single(w, d, precision="fp16"))
    p.close()


def _rand_gains(rng, nant, nchan):
    return (rng.normal(size=(nant, 2, nchan)) + 1j * rng.normal(size=(nant, 2, nchan))).astype(np.complex64)


@pytest.mark.parametrize("ideal", [True, False])
@pytest.mark.parametrize("autos", [True, False])
def test_lin2circ_kernel_vs_voltage_domain(ideal, autos):
    rng = np.random.default_rng(3)
    nant, nfft, nchan = 6, 9, 40
    x = (rng.normal(size=(nant, 2, nfft, nchan)) + 1j * rng.normal(size=(nant, 2, nfft, nchan)))
    g = None if ideal else _rand_gains(rng, nant, nchan)
    vis = O.correlate_voltages(x, autos=autos).astype(np.complex64)
    want = O.correlate_voltages(O.lin2circ_voltages(x, g), autos=autos)
    dv = torch.from_numpy(vis).cuda()
    dg = None if g is None else torch.from_numpy(g).cuda()
    lin2circ(dv, nant, nchan, autos, dg)
    torch.cuda.synchronize()
    got = dv.cpu().numpy()
    assert O.rel_rms_per_product(got, want).max() < 1e-6


def test_pipeline_lin2circ_and_integration():
    subs = _subints(2)
    rng = np.random.default_rng(8)
    g = _rand_gains(rng, W.nant, W.nchan)
    p = Pipeline(W.nant, W.nchan, W.nfft, W.nbit, W.lo_hz, W.bw_hz, W.is_complex)
    p.set_lin2circ(True, g)
    outs = [torch.zeros((p.nbl, 4, W.nchan), dtype=torch.complex64).pin_memory() for _ in subs]
    for d, o in zip(subs, outs):
        p.submit(d["inputs"], d["poly"], d["fso"], out=o)
    integ, n = p.integration()
    nbl = p.nbl
    total = np.zeros((nbl, 4, W.nchan), np.complex128)
    for d, o in zip(subs, outs):
        lin = torch.from_numpy(_single(W, d)).cuda()
        lin2circ(lin, W.nant, W.nchan, True, torch.from_numpy(g).cuda())
        torch.cuda.synchronize()
        assert np.array_equal(o.numpy(), lin.cpu().numpy())
        total += o.numpy()
    assert n == 2 and O.rel_rms(integ, total) < 1e-6
    p.close()
