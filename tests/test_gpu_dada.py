"""DADA streams into the correlator: one stream per antenna (header, then the engine's input
layout, as the reference's ingest writes its ring buffer, ingest/src/ingest.c:185-330), read a
sub-integration at a time into pinned buffers, configured from the header, correlated, and
compared bit for bit with the same bytes given to the engine directly."""
import numpy as np
import pytest

from gcorr_gb300 import FxKernel, dada, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_dada_streams_correlate_like_direct_input(tmp_path):
    import torch
    w = synth.Workload(nant=3, nchan=1024, nfft=40, bw_hz=64e6, lo_hz=8.4e9, rho=0.3, seed=95)
    d = synth.generate(w)
    inputs = [x.numpy() for x in d["inputs"]]
    fields = {"FREQ": (w.lo_hz + w.bw_hz / 2) / 1e6, "BW": w.bw_hz / 1e6, "NBIT": 2, "NPOL": 2, "NDIM": 1,
              "NCHAN": 1, "UTC_START": "2024-05-01-12:00:00"}
    paths = [str(tmp_path / f"ant{a}.dada") for a in range(w.nant)]
    for p, x in zip(paths, inputs):
        dada.write_stream(p, fields, np.concatenate([x, x[:1000]]))  # two sub-integrations' worth, the second short
    r = dada.DadaReader(paths, w.bytes_per_antenna)
    cfg = r.config(nant=w.nant, nchan=w.nchan, nfft=w.nfft)
    assert cfg.lo_hz == w.lo_hz and cfg.bw_hz == w.bw_hz and cfg.nbit == 2
    bufs = [torch.empty(w.bytes_per_antenna, dtype=torch.uint8).pin_memory() for _ in range(w.nant)]
    assert r.read(bufs)
    assert not r.read(bufs)  # the second sub-integration is incomplete: end of data
    r.close()

    def correlate(ins):
        fx = FxKernel(w.nant, w.nchan, w.nfft, 2, cfg.lo_hz, cfg.bw_hz, False)
        fx.setInputData(ins)
        fx.setDelays(d["poly"], d["fso"])
        fx.process()
        v, c = fx.visibilities(), fx.baseline_counts()
        fx.close()
        return v, c

    v_dada, c_dada = correlate(bufs)
    v_direct, c_direct = correlate(inputs)
    assert np.array_equal(v_dada, v_direct) and np.array_equal(c_dada, c_direct)
    ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), inputs, d["poly"], d["fso"])
    assert np.array_equal(c_dada, rc)
    assert O.rel_rms_per_product(v_dada, ref).max() < 1e-5
