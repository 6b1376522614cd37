"""GPU tests of the reference-compatible drivers: testfxkernel and bench_fxkernel run on
a .conf file and raw antenna files written here (fxkernel/src/testfxkernel.cpp,
fxkernel/src/bench_fxkernel.cpp), with vis.out checked against the engine and the
oracle, and lag S/N checked as util/lagsnr.py does."""
import os
import subprocess

import numpy as np
import pytest

from gcorr_gb300 import FxKernel, buildlib, conf, synth, visio
from gcorr_gb300.lagsnr import lag_snr_file
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _write_case(tmp_path, w):
    d = synth.generate(w)
    names = [f"A{a}" for a in range(w.nant)]
    files = [f"ant{a}.bin" for a in range(w.nant)]
    for f, x in zip(files, d["inputs"]):
        x.numpy().tofile(str(tmp_path / f))
    cpath = str(tmp_path / "case.conf")
    conf.write_conf(cpath, w.nant, w.nchan, w.nfft, w.lo_hz, w.bw_hz, names, files, d["poly"], d["fso"],
                    nbit=w.nbit, is_complex=w.is_complex)
    return cpath, d


def test_testfxkernel_vis_out(tmp_path):
    buildlib.build()
    w = synth.Workload(nant=4, nchan=1024, nfft=300, bw_hz=32e6, rho=0.3, seed=91)
    cpath, d = _write_case(tmp_path, w)
    r = subprocess.run([os.path.join(buildlib.BIN, "testfxkernel"), cpath], capture_output=True, text=True,
                       cwd=tmp_path, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Got NANT 4" in r.stdout and "Run time was" in r.stdout
    assert (tmp_path / "runtime.fxkernel.log").exists()
    nbl = w.nant * (w.nant - 1) // 2
    freq, vis = visio.load_visibilities(str(tmp_path / "vis.out"), nbl)
    # the same sub-integration through the Python API with the C++ class's defaults
    fx = FxKernel(w.nant, w.nchan, w.nfft, 2, w.lo_hz, w.bw_hz, False, rotator="fxkernel", autos=False)
    fx.setInputData([x.numpy() for x in d["inputs"]])
    fx.setDelays(d["poly"], d["fso"])
    fx.process()
    v = fx.visibilities()
    fx.close()
    assert np.allclose(vis, v, rtol=1e-6, atol=1.1e-5)  # vis.out prints 5 decimals
    # fxkernel semantics: the FP32 port of the reference (oracle)
    ref, _ = O.port_process(O.config_from_workload(w, O.ROT_FXKERNEL, False), [x.numpy() for x in d["inputs"]],
                            d["poly"], d["fso"])
    assert O.rel_rms_per_product(vis, ref).max() < 1e-5
    # lag S/N: delays are compensated, so every parallel-hand product peaks at lag 0
    snr, arg = lag_snr_file(str(tmp_path / "vis.out"))
    par = np.array([4 * b + p for b in range(nbl) for p in (0, 3)])
    assert (snr[par] > 8).all() and (arg[par] == 0).all(), (snr[par], arg[par])


def test_bench_fxkernel_runs(tmp_path):
    buildlib.build()
    w = synth.Workload(nant=3, nchan=256, nfft=100, bw_hz=32e6, seed=5)
    cpath, _ = _write_case(tmp_path, w)
    r = subprocess.run([os.path.join(buildlib.BIN, "bench_fxkernel"), "-nloop", "2", "-nbuf", "2", "-threads", "2",
                        cpath], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Mbps" in r.stdout and "Run time was" in r.stdout


def test_testfxkernel_8bit_complex(tmp_path):
    buildlib.build()
    w = synth.Workload(nant=3, nchan=512, nfft=120, nbit=8, is_complex=True, bw_hz=32e6, rho=0.3, seed=92)
    cpath, d = _write_case(tmp_path, w)
    r = subprocess.run([os.path.join(buildlib.BIN, "testfxkernel"), cpath], capture_output=True, text=True,
                       cwd=tmp_path, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    _, vis = visio.load_visibilities(str(tmp_path / "vis.out"), 3)
    ref, _ = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, False), [x.numpy() for x in d["inputs"]],
                             d["poly"], d["fso"])
    assert O.rel_rms_per_product(vis, ref).max() < 1e-5
