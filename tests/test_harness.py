"""CPU tests of the harness formats: .conf parsing (fxkernel/src/common.cpp:54-114),
raw-file reading (common.cpp:38-52), the vis.out writer (fxkernel/src/fxkernel.cpp:370-412),
the lag S/N tool (util/lagsnr.py:16-31) and the command-line drivers' argument handling."""
import os
import subprocess

import numpy as np
import pytest

from gcorr_gb300 import _lib as L
from gcorr_gb300 import buildlib, conf, visio
from gcorr_gb300.lagsnr import lag_snr, lag_snr_file

# the layout of the reference's example config (fxkernel/src/test.conf): 5 numbers after
# each file name (the 5th is ignored), keywords in mixed case, plus an unknown keyword
# that is skipped; the values here are arbitrary
CONF = """NBIT 2
npol 2
Complex 0
NCHAN 1024
LO 2250000000
BANDWIDTH 16000000
NUMFFTS 1500
COLOUR blue
NANT 2
Xa xa.dat 2.5e-19  -3.0e-15   45.5e-9 40e-9 7
Yb yb.dat -1.5e-19  6.0e-15   -20.25e-9 -25e-9 0
"""


def test_conf_reader(tmp_path):
    p = tmp_path / "t.conf"
    p.write_text(CONF)
    c = conf.read_conf(str(p))
    assert (c["nbit"], c["npol"], c["is_complex"], c["nchan"], c["nfft"], c["nant"]) == (2, 2, False, 1024, 1500, 2)
    assert c["lo"] == 2.25e9 and c["bw"] == 16e6
    assert c["names"] == ["Xa", "Yb"] and c["files"] == ["xa.dat", "yb.dat"]
    assert np.array_equal(c["poly"], [[2.5e-19, -3.0e-15, 45.5e-9], [-1.5e-19, 6.0e-15, -20.25e-9]])
    assert np.array_equal(c["fso"], [40e-9, -25e-9])


def test_conf_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    poly = rng.normal(size=(3, 3)) * 1e-6
    fso = rng.normal(size=3) * 1e-7
    p = str(tmp_path / "r.conf")
    conf.write_conf(p, 3, 256, 10, 8.4e9, 64e6, ["A", "B", "C"], ["a", "b", "c"], poly, fso, nbit=8,
                    is_complex=True)
    c = conf.read_conf(p)
    assert np.array_equal(c["poly"], poly) and np.array_equal(c["fso"], fso)
    assert c["nbit"] == 8 and c["is_complex"]


@pytest.mark.parametrize("text", ["NBIT 2\n\nNCHAN 4\n", "NANT 2\nA a 1 2 3 4\n", "NCHAN x\n", "NANT 1\nA a 1 2\n"])
def test_conf_errors(tmp_path, text):
    p = tmp_path / "bad.conf"
    p.write_text(text)
    with pytest.raises(L.GxcError):
        conf.read_conf(str(p))


def test_raw_reader(tmp_path):
    rng = np.random.default_rng(2)
    data = [rng.integers(0, 256, 250, dtype=np.uint8) for _ in range(3)]
    paths = []
    for i, d in enumerate(data):
        paths.append(str(tmp_path / f"a{i}.bin"))
        d.tofile(paths[-1])
    r = conf.RawReader(paths, 100)
    for k in range(2):
        out = r.read()
        for i in range(3):
            assert np.array_equal(out[i], data[i][100 * k:100 * (k + 1)])
    assert r.read() is None  # 50 bytes left: end of data, as readdata returns 2
    r.close()
    with pytest.raises(L.GxcError):
        conf.RawReader([paths[0], str(tmp_path / "missing.bin")], 10)


def test_vis_writer_matches_python_writer(tmp_path):
    rng = np.random.default_rng(3)
    vis = (rng.normal(size=(3, 4, 16)) + 1j * rng.normal(size=(3, 4, 16))).astype(np.complex64) * 50
    a, b = str(tmp_path / "c.out"), str(tmp_path / "py.out")
    conf.save_visibilities(a, vis, 64e6)
    visio.save_visibilities(b, vis, 64e6)
    ta, tb = np.loadtxt(a), np.loadtxt(b)
    assert ta.shape == tb.shape == (16, 2 + 3 * 4 * 4)
    assert np.allclose(ta, tb, rtol=3e-7, atol=1.1e-5)  # float32 amplitudes may differ by an ulp
    assert [ln.split()[:2] for ln in open(a)] == [ln.split()[:2] for ln in open(b)]
    freq, back = visio.load_visibilities(a, 3)
    assert np.allclose(back, vis, atol=1e-5)
    assert np.allclose(freq, (np.arange(16) + 0.5) / 16 * 64)


def test_lag_snr():
    nchan = 256
    rng = np.random.default_rng(4)
    noise = (rng.normal(size=(2, nchan)) + 1j * rng.normal(size=(2, nchan))) * 0.1
    vis = noise.copy()
    vis[0] += np.exp(-2j * np.pi * 5 * np.arange(nchan) / nchan)  # peaks at lag bin 5 of the inverse FFT
    snr, arg = lag_snr(vis)
    assert snr[0] > 2.5 * snr[1] and arg[0] == 5  # a single-lag peak caps S/N near sqrt(nchan)


def test_lag_snr_file(tmp_path):
    vis = np.zeros((1, 4, 64), np.complex64)
    vis[0, 0] = 1.0
    p = str(tmp_path / "v.out")
    visio.save_visibilities(p, vis, 32e6)
    snr, arg = lag_snr_file(p)
    assert snr.shape == (4,) and arg[0] == 0


def test_drivers_built_and_check_arguments(tmp_path):
    buildlib.build()
    for app in buildlib.APPS:
        exe = os.path.join(buildlib.BIN, app)
        assert os.access(exe, os.X_OK)
        r = subprocess.run([exe], capture_output=True, text=True, cwd=tmp_path, timeout=60)
        assert r.returncode == 1 and "Usage" in r.stdout
    bad = tmp_path / "bad.conf"
    bad.write_text("NBIT 2\n\n")
    r = subprocess.run([os.path.join(buildlib.BIN, "testfxkernel"), str(bad)], capture_output=True, text=True,
                       cwd=tmp_path, timeout=60)
    assert r.returncode == 1 and "could not parse" in r.stderr
