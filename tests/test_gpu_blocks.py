"""FFT blocks: the chosen block size, and the short first block of host-input runs.

With host inputs the first F-stage waits for the copy of its block's samples, so a chosen
block size starts with a 4096-FFT block and doubles up to it; device inputs use equal
blocks.  The two runs differ only in where the blocks end (the order of the accumulator
additions)."""
import numpy as np
import pytest

from gcorr_gb300 import FxKernel, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_host_inputs_start_with_a_short_block():
    w = synth.Workload(nant=2, nchan=256, nfft=32768, bw_hz=64e6, seed=5)
    d = synth.random_bytes(w)
    out = {}
    for where in ("host", "device"):
        fx = FxKernel(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex)
        ins = [x.pin_memory() for x in d["inputs"]] if where == "host" else [x.cuda() for x in d["inputs"]]
        fx.setInputData(ins)
        fx.setDelays(d["poly"], d["fso"])
        fx.process()
        out[where] = (fx.visibilities(), fx.baseline_counts(), fx.fft_block, fx.num_blocks)
        fx.close()
    assert out["device"][2] == out["host"][2] == 16384
    assert out["device"][3] == 2  # 16384 + 16384
    assert out["host"][3] == 4    # 4096 + 8192 + 16384 + 4096
    assert np.array_equal(out["host"][1], out["device"][1])
    assert O.rel_rms(out["host"][0], out["device"][0]) < 1e-6


def test_explicit_block_is_kept_for_host_inputs():
    w = synth.Workload(nant=2, nchan=256, nfft=3000, bw_hz=64e6, seed=6)
    d = synth.random_bytes(w)
    fx = FxKernel(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, fft_block=1024)
    fx.setInputData([x.pin_memory() for x in d["inputs"]])
    fx.setDelays(d["poly"], d["fso"])
    fx.process()
    assert fx.fft_block == 1024 and fx.num_blocks == 3
    vis, counts = fx.visibilities(), fx.baseline_counts()
    fx.close()
    ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), [x.numpy() for x in d["inputs"]],
                              d["poly"], d["fso"])
    assert np.array_equal(counts, rc)
    assert O.rel_rms_per_product(vis, ref).max() < 1e-5
