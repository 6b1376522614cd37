"""GPU tests of the batch API (uneven jobs in one graph launch) and the autotuner."""
import numpy as np
import pytest
import torch

from gcorr_gb300 import FxKernel, synth
from gcorr_gb300.batch import Batch
from oracle import oracle as O

pytestmark = pytest.mark.gpu

JOBS = [synth.Workload(nant=3, nchan=256, nfft=40, bw_hz=32e6, seed=1),
        synth.Workload(nant=5, nchan=512, nfft=30, nbit=8, is_complex=True, bw_hz=32e6, seed=2),
        synth.Workload(nant=4, nchan=1024, nfft=24, bw_hz=64e6, seed=3),
        synth.Workload(nant=2, nchan=16384, nfft=4, bw_hz=64e6, seed=4)]


def _job(w, d, **kw):
    return dict(nant=w.nant, nchan=w.nchan, nfft=w.nfft, nbit=w.nbit, lo=w.lo_hz, bw=w.bw_hz,
                is_complex=w.is_complex, inputs=d["inputs"], poly=d["poly"], fso=d["fso"], **kw)


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_batch_matches_individual_runs(precision):
    data = [synth.random_bytes(w, device="cuda") for w in JOBS]
    b = Batch([_job(w, d, precision=precision) for w, d in zip(JOBS, data)])
    b.launch()
    b.launch()  # the graph replays from the same inputs
    for i, (w, d) in enumerate(zip(JOBS, data)):
        fx = FxKernel(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, precision=precision)
        fx.setInputData(d["inputs"])
        fx.setDelays(d["poly"], d["fso"])
        fx.process()
        ref = fx.visibilities()
        assert np.array_equal(b.baseline_counts(i), fx.baseline_counts())
        fx.close()
        assert O.rel_rms(b.visibilities(i), ref) < 1e-6, i
    assert b.launches > 0
    b.close()


def test_batch_vs_fp64_oracle():
    data = [synth.random_bytes(w, device="cuda") for w in JOBS[:3]]
    b = Batch([_job(w, d, precision="fp32") for w, d in zip(JOBS[:3], data)])
    b.launch()
    for i, (w, d) in enumerate(zip(JOBS[:3], data)):
        inputs = [x.cpu().numpy() for x in d["inputs"]]
        ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), inputs, d["poly"], d["fso"])
        assert np.array_equal(b.baseline_counts(i), rc)
        assert O.rel_rms_per_product(b.visibilities(i), ref).max() < 1e-5
    b.close()


def test_autotune_caches(tmp_path):
    from gcorr_gb300.autotune import tune
    w = JOBS[2]
    d = synth.random_bytes(w, device="cuda")
    path = str(tmp_path / "tune.json")
    r1 = tune(_job(w, d, precision="fp16"), blocks=(8, 24), path=path)
    assert r1["fft_block"] in (8, 24) and r1["x_engine"] in ("tensor", "cuda_core") and r1["tried"]
    assert r1["fft_engine"] == "cuda_core"  # 2048-point windows: the CUDA-core FFT is the only plan
    r2 = tune(_job(w, d, precision="fp16"), blocks=(8, 24), path=path)
    assert r2 == r1


def test_autotune_searches_f_plan_and_x_split(tmp_path):
    """An 8192-point FP16 shape: the tuner times both F-stage plans and, for the tensor X-stage,
    both FFT-range splits; a batch built from the tuned plan matches a single run of that plan."""
    from gcorr_gb300.autotune import tune
    w = synth.Workload(nant=4, nchan=4096, nfft=48, bw_hz=256e6, seed=9)
    d = synth.random_bytes(w, device="cuda")
    t = tune(_job(w, d, precision="fp16"), blocks=(16, 48), path=str(tmp_path / "tune.json"))
    assert {p["fft_engine"] for p in t["tried"]} == {"cuda_core", "tensor"}
    if t["x_engine"] == "tensor":
        assert {p["x_split"] for p in t["tried"]} >= {"off", "on"}
    plan = {k: t[k] for k in ("x_engine", "fft_block", "fft_engine", "x_split")}
    b = Batch([_job(w, d, precision="fp16", **plan)])
    b.launch()
    fx = FxKernel(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, precision="fp16", **plan)
    fx.setInputData(d["inputs"])
    fx.setDelays(d["poly"], d["fso"])
    fx.process()
    assert O.rel_rms(b.visibilities(0), fx.visibilities()) < 1e-6
    fx.close()
    b.close()


@pytest.mark.parametrize("precision", ["fp16", "fp8"])
def test_x_split_modes_agree(precision):
    """The FFT-range split only changes which CTA sums which FFTs (two accumulator planes added at
    finalisation).  Tensor memory accumulates with rounding toward zero, and the split halves each
    CTA's run of accumulations, so forced on and off differ by that bias (about 1e-6 relative over
    600 FFTs), far inside the FP16 / FP8 tolerances; counts agree exactly."""
    w = synth.Workload(nant=6, nchan=1024, nfft=600, bw_hz=64e6, seed=10)
    d = synth.random_bytes(w, device="cuda")
    out = {}
    for xs in ("off", "on", "auto"):
        fx = FxKernel(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, precision=precision,
                      x_engine="tensor", x_split=xs)
        fx.setInputData(d["inputs"])
        fx.setDelays(d["poly"], d["fso"])
        fx.process()
        out[xs] = (fx.visibilities(), fx.baseline_counts())
        fx.close()
    assert np.array_equal(out["on"][1], out["off"][1])
    assert O.rel_rms(out["on"][0], out["off"][0]) < 1e-5
    assert O.rel_rms(out["auto"][0], out["off"][0]) < 1e-5


def test_batch_on_pinned_host_inputs():
    """Host inputs: each job's host->device copy is captured into its graph branch."""
    data = [synth.random_bytes(w) for w in JOBS]
    host = [[x.pin_memory() for x in d["inputs"]] for d in data]
    dev = [[x.cuda() for x in d["inputs"]] for d in data]
    bh = Batch([dict(_job(w, d, precision="fp16"), inputs=hx) for w, d, hx in zip(JOBS, data, host)])
    bd = Batch([dict(_job(w, d, precision="fp16"), inputs=dx) for w, d, dx in zip(JOBS, data, dev)])
    bh.launch()
    bd.launch()
    for i in range(len(JOBS)):
        assert np.array_equal(bh.visibilities(i), bd.visibilities(i))
    # the graph re-reads the host buffers on every launch
    for hx in host:
        for x in hx:
            x.copy_(torch.randint(0, 256, x.shape, dtype=torch.uint8))
    bh.launch()
    assert not np.array_equal(bh.visibilities(0), bd.visibilities(0))
    bh.close()
    bd.close()
