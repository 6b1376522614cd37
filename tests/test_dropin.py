"""The drop-in boundary, proven with the reference's own drivers.

fxkernel/src/testfxkernel.cpp and fxkernel/src/bench_fxkernel.cpp are compiled
UNMODIFIED (oracle/Makefile stages them, with the reference's fxkernel.cpp,
into the git-ignored oracle/_ref/src/) against the drop-in include directory
include/fxkernel_dropin/ (fxkernel.h, common.h, vectordefs.h forwarding to the
engine's C++ headers) and linked with libgxcorr.so instead of fxkernel.cpp and
IPP.  The CPU test builds them; the GPU tests run them on a .conf and compare
testfxkernel's vis.out with the one the reference's own process() and
saveVisibilities() write for the same files.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from gcorr_gb300 import buildlib, conf, synth, visio
from oracle import oracle as O

STAGED = os.path.join(ROOT, "oracle", "_ref", "src")
DRIVERS = ("testfxkernel", "bench_fxkernel")

needs_staged = pytest.mark.skipif(not all(os.path.exists(os.path.join(STAGED, d + ".cpp")) for d in DRIVERS),
                                  reason="reference driver sources not staged (oracle/Makefile REFDIR=...)")


def _build_driver(name, outdir):
    """Copies the unmodified driver into outdir (so that its quoted includes find the drop-in
    headers, not the reference's) and compiles it against include/fxkernel_dropin."""
    buildlib.build()
    src = os.path.join(outdir, name + ".cpp")
    shutil.copyfile(os.path.join(STAGED, name + ".cpp"), src)
    exe = os.path.join(outdir, name)
    cxx = shutil.which("g++") or shutil.which("c++")
    cmd = [cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include", "fxkernel_dropin"), "-I",
           os.path.join(ROOT, "include"), src, "-o", exe, "-L", os.path.dirname(buildlib.LIB), "-lgxcorr",
           "-Wl,-rpath," + os.path.dirname(buildlib.LIB), "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


@needs_staged
def test_reference_drivers_compile_unmodified(tmp_path):
    for d in DRIVERS:
        assert os.path.exists(_build_driver(d, str(tmp_path)))
        with open(os.path.join(STAGED, d + ".cpp"), "rb") as a, open(str(tmp_path / (d + ".cpp")), "rb") as b:
            assert a.read() == b.read()


def _write_case(tmp_path, w):
    d = synth.generate(w)
    names = [f"A{a}" for a in range(w.nant)]
    files = [f"ant{a}.bin" for a in range(w.nant)]
    for f, x in zip(files, d["inputs"]):
        x.numpy().tofile(str(tmp_path / f))
    cpath = str(tmp_path / "case.conf")
    conf.write_conf(cpath, w.nant, w.nchan, w.nfft, w.lo_hz, w.bw_hz, names, files, d["poly"], d["fso"])
    return cpath, d


@needs_staged
@pytest.mark.gpu
def test_reference_testfxkernel_on_engine_matches_reference_vis_out(tmp_path):
    exe = _build_driver("testfxkernel", str(tmp_path))
    w = synth.Workload(nant=5, nchan=1024, nfft=200, bw_hz=64e6, rho=0.2, seed=93)
    cpath, d = _write_case(tmp_path, w)
    r = subprocess.run([exe, cpath], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Got NANT 5" in r.stdout and "Run time was" in r.stdout
    ref_path = str(tmp_path / "vis_reference.out")
    O.ref_save(w.nant, w.nchan, w.nfft, w.lo_hz, w.bw_hz, [x.numpy() for x in d["inputs"]], d["poly"], d["fso"],
               ref_path)
    ours = open(str(tmp_path / "vis.out")).read().split("\n")
    theirs = open(ref_path).read().split("\n")
    assert len(ours) == len(theirs)
    nbl = w.nant * (w.nant - 1) // 2
    f1, v1 = visio.load_visibilities(str(tmp_path / "vis.out"), nbl)
    f2, v2 = visio.load_visibilities(ref_path, nbl)
    assert np.array_equal(f1, f2)
    # the FP32 tolerance of the parity tests, per (baseline, product), on the printed values
    assert O.rel_rms_per_product(v1, v2).max() < 1e-5


@needs_staged
@pytest.mark.gpu
def test_reference_bench_fxkernel_runs_on_engine(tmp_path):
    exe = _build_driver("bench_fxkernel", str(tmp_path))
    w = synth.Workload(nant=4, nchan=256, nfft=100, bw_hz=32e6, seed=6)
    cpath, _ = _write_case(tmp_path, w)
    r = subprocess.run([exe, "-nloop", "2", "-nbuf", "2", "-threads", "2", cpath], capture_output=True, text=True,
                       cwd=tmp_path, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Mbps" in r.stdout and "Run time was" in r.stdout
