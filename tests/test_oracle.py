"""CPU tests of the oracle: pinned against the reference's own outputs.

The golden fixtures hold outputs of the reference FxKernel::process()
(fxkernel/src/fxkernel.cpp:253-368) compiled from its unmodified source; where
the reference sources are present the oracle is also checked live against it.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from gcorr_gb300 import synth
from oracle import oracle as O


def _cfg(d, rotator, autos):
    return O.make_config(int(d["nant"]), int(d["nchan"]), int(d["nfft"]), int(d["nbit"]), bool(d["is_complex"]),
                         float(d["lo_hz"]), float(d["bw_hz"]), rotator, autos)


def test_lut_matches_fixture():
    lut = np.load(os.path.join(GOLDEN, "lut2bit.npy"))
    for b in range(256):
        assert np.array_equal(O.lut2bit(b), lut[b])
    levels = np.array([-3.3359, -1.0, 1.0, 3.3359], dtype=np.float32)
    for b in range(256):
        for i in range(4):
            assert lut[b, i] == levels[(b >> (2 * i)) & 3]


@pytest.mark.parametrize("offset", [0, 1, 2, 3, 17, 1000, 1001])
def test_unpack_2bit_offsets(offset):
    """Odd and even offsets (fxkernel.cpp:452-475) reduce to sample offset+o."""
    rng = np.random.default_rng(offset)
    cfg = O.make_config(1, 256, 8)
    buf = rng.integers(0, 256, 4096, dtype=np.uint8)
    n = 512
    p0, p1 = O.unpack(cfg, buf, offset, n)
    lv = np.array([-3.3359, -1.0, 1.0, 3.3359], dtype=np.float32)
    m = offset + np.arange(n)
    byte = buf[m >> 1]
    h = (m & 1) * 2
    a = lv[(byte >> (2 * h)) & 3]
    b = lv[(byte >> (2 * (h + 1))) & 3]
    assert np.array_equal(p0.real, a) and np.array_equal(p1.real, b)
    assert not p0.imag.any() and not p1.imag.any()


def test_unpack_8bit_complex():
    cfg = O.make_config(1, 256, 8, nbit=8, is_complex=True)
    rng = np.random.default_rng(3)
    buf = rng.integers(0, 256, 8192, dtype=np.uint8)
    p0, p1 = O.unpack(cfg, buf, 5, 100)
    s = buf.view(np.int8).astype(np.float32)[20:20 + 400].reshape(100, 4)
    assert np.array_equal(p0, s[:, 0] + 1j * s[:, 1])
    assert np.array_equal(p1, s[:, 2] + 1j * s[:, 3])


def test_geometry_matches_fixture(golden_cases):
    for name, d in golden_cases.items():
        cfg = _cfg(d, O.ROT_EXACT, True)
        for a in range(int(d["nant"])):
            for i in range(int(d["nfft"])):
                g = O.geometry(cfg, d["poly"][a], float(d["fso"][a]), i)
                assert (g.offset if g.valid else 0, g.valid) == tuple(d["geom"][a, i]) or \
                    (not g.valid and d["geom"][a, i, 1] == 0), (name, a, i)


def test_port_matches_reference_fixture(golden_cases):
    """FP32 port in fxkernel-rotator mode reproduces the reference output."""
    for name, d in golden_cases.items():
        cfg = _cfg(d, O.ROT_FXKERNEL, False)
        vis, counts = O.port_process(cfg, list(d["inputs"]), d["poly"], d["fso"])
        assert O.rel_rms(vis, d["ref_vis"]) < 1e-6, name
        assert np.all(O.rel_rms_per_product(vis, d["ref_vis"]) < 1e-5), name


def test_fp64_oracle_compat_matches_reference_fixture(golden_cases):
    for name, d in golden_cases.items():
        cfg = _cfg(d, O.ROT_FXKERNEL, False)
        vis, _ = O.exact_process(cfg, list(d["inputs"]), d["poly"], d["fso"])
        assert O.rel_rms(vis, d["ref_vis"]) < 2e-6, name


def test_port_and_fp64_oracle_match_benchmark_shaped_fixtures(shape_cases):
    """The oracle pinned at the benchmark shapes: the reference's own process() output for 6
    antennas x nchan 1024 (2048-point FFTs, flagged edge FFTs) and 16 antennas x nchan 4096
    (8192-point FFTs), fxkernel rotator, crosses only."""
    from conftest import reference_checks
    assert set(shape_cases) == {"shape_c0_6ant_n1024", "shape_c1_16ant_n4096"}
    for name, d in shape_cases.items():
        cfg = _cfg(d, O.ROT_FXKERNEL, False)
        vis, counts = O.port_process(cfg, list(d["inputs"]), d["poly"], d["fso"], nthreads=4)
        assert np.array_equal(counts, d["counts"]), name
        r = reference_checks(vis, d)
        assert r["per_product"] < 1e-5 and r.get("sum", 0.0) < 1e-6 and r.get("power", 0.0) < 1e-5, (name, r)
        ve, ce = O.exact_process(cfg, list(d["inputs"]), d["poly"], d["fso"])
        assert np.array_equal(ce, d["counts"]), name
        r = reference_checks(ve, d)
        assert r["per_product"] < 1e-5 and r.get("sum", 0.0) < 1e-6 and r.get("power", 0.0) < 1e-5, (name, r)
        for a in range(int(d["nant"])):
            for i in range(int(d["nfft"])):
                g = O.geometry(cfg, d["poly"][a], float(d["fso"][a]), i)
                assert g.valid == d["geom"][a, i, 1] and (not g.valid or g.offset == d["geom"][a, i, 0]), (name, a, i)


def test_exact_fixture_reproducible(golden_cases):
    for name, d in golden_cases.items():
        cfg = _cfg(d, O.ROT_EXACT, True)
        vis, counts = O.exact_process(cfg, list(d["inputs"]), d["poly"], d["fso"])
        assert np.array_equal(counts, d["exact_counts"]), name
        assert O.rel_rms(vis, d["exact_vis"]) < 1e-12, name


def test_port_exact_vs_fp64():
    w = synth.Workload(nant=3, nchan=128, nfft=30, bw_hz=32e6, seed=21)
    d = synth.random_bytes(w)
    cfg = O.config_from_workload(w, O.ROT_EXACT, True)
    vp, cp = O.port_process(cfg, d["inputs"], d["poly"], d["fso"], nthreads=2)
    ve, ce = O.exact_process(cfg, d["inputs"], d["poly"], d["fso"])
    assert np.array_equal(cp, ce)
    assert O.rel_rms(vp, ve) < 1e-6


def test_rotator_quirk_is_real():
    """The reference's half-rate step table (fxkernel.cpp:112 vs :553-558) differs from
    the exact linear rotator for real data when the delay rate is large."""
    w = synth.Workload(nant=2, nchan=256, nfft=16, bw_hz=64e6, lo_hz=8.4e9, seed=5, rate_us_per_s=300.0)
    d = synth.random_bytes(w)
    ve, _ = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, False), d["inputs"], d["poly"], d["fso"])
    vc, _ = O.exact_process(O.config_from_workload(w, O.ROT_FXKERNEL, False), d["inputs"], d["poly"], d["fso"])
    assert O.rel_rms(vc, ve) > 1e-3


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not present on this host")
@pytest.mark.parametrize("seed", [31, 32])
def test_port_vs_live_reference(seed):
    w = synth.Workload(nant=4, nchan=64, nfft=40, bw_hz=16e6, seed=seed, offset_us=5.0)
    d = synth.random_bytes(w)
    ref = O.ref_process(w.nant, w.nchan, w.nfft, w.lo_hz, w.bw_hz, d["inputs"], d["poly"], d["fso"])
    vis, _ = O.port_process(O.config_from_workload(w, O.ROT_FXKERNEL, False), d["inputs"], d["poly"], d["fso"])
    assert O.rel_rms(vis, ref) < 1e-6


def test_generator_coherence():
    """Seeded generator: fringe-stopped crosses recover rho x 2-bit efficiency (~0.88) with flat phase."""
    w = synth.Workload(nant=3, nchan=64, nfft=200, bw_hz=16e6, lo_hz=8.4e9, rho=0.5, seed=7)
    d = synth.generate(w)
    cfg = O.config_from_workload(w, O.ROT_EXACT, True)
    v, _ = O.exact_process(cfg, d["inputs"], d["poly"], d["fso"])
    nx = 3
    for b, (j, k) in enumerate([(0, 1), (0, 2), (1, 2)]):
        coh = v[b, 0, 4:-4] / np.sqrt(v[nx + j, 0, 4:-4].real * v[nx + k, 0, 4:-4].real)
        m = coh.mean()
        assert 0.38 < abs(m) < 0.50
        assert abs(np.angle(m)) < 0.1
        assert abs(v[b, 1, 4:-4].mean()) / np.sqrt(v[nx + j, 0, 4:-4].real.mean() * v[nx + k, 3, 4:-4].real.mean()) < 0.05
