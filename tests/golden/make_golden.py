"""Generates the golden fixtures in this directory.

Runs the reference's own FxKernel::process() (fxkernel/src/fxkernel.cpp:253-368,
compiled unmodified against the IPP-compatible shim into oracle/_ref/libfxref.so)
and the FP64 restatement (oracle/fxoracle.c) on small seeded inputs, and stores
inputs, delay models and outputs as .npz files.  The GPU tests compare against
these files on hosts where the reference sources are absent.

Usage (where the reference library oracle/_ref/libfxref.so has been built, see oracle/Makefile):
    python tests/golden/make_golden.py [case names]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gcorr_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

# name -> (workload, input kind)
CASES = {
    # 4 antennas, nchan 256 (square), physics input with a strong correlation
    "c4_n256_synth": (synth.Workload(nant=4, nchan=256, nfft=48, bw_hz=32e6, lo_hz=8.4e9, rho=0.3, seed=11), "synth"),
    # 3 antennas, nchan 1024 (square), uniform random bytes, 20 us delays -> flagged edge FFTs
    "c3_n1024_random": (synth.Workload(nant=3, nchan=1024, nfft=24, bw_hz=64e6, lo_hz=8.4e9, seed=12,
                                       offset_us=20.0), "random"),
    # 5 antennas, nchan 256, fractional LO, negative and positive delays, odd offsets
    "c5_n256_fraclo": (synth.Workload(nant=5, nchan=256, nfft=40, bw_hz=16e6, lo_hz=1650000000.37, rho=0.1,
                                      seed=13, offset_us=3.0, rate_us_per_s=30.0), "synth"),
}


def make(name: str, w: synth.Workload, kind: str):
    d = synth.generate(w) if kind == "synth" else synth.random_bytes(w)
    inputs = np.stack([x.numpy() for x in d["inputs"]])
    poly, fso = d["poly"], d["fso"]
    ref_vis = O.ref_process(w.nant, w.nchan, w.nfft, w.lo_hz, w.bw_hz, list(inputs), poly, fso)
    cfg_x = O.config_from_workload(w, rotator=O.ROT_EXACT, autos=True)
    exact_vis, counts = O.exact_process(cfg_x, list(inputs), poly, fso)
    cfg_c = O.config_from_workload(w, rotator=O.ROT_FXKERNEL, autos=False)
    port_vis, _ = O.port_process(cfg_c, list(inputs), poly, fso)
    geom = np.array([[(g.offset, g.valid) for g in (O.geometry(cfg_x, poly[a], fso[a], i) for i in range(w.nfft))]
                     for a in range(w.nant)], dtype=np.int32)
    err = O.rel_rms(port_vis, ref_vis)
    assert err < 1e-5, (name, err)
    np.savez_compressed(
        os.path.join(HERE, f"{name}.npz"),
        nant=w.nant, nchan=w.nchan, nfft=w.nfft, nbit=w.nbit, is_complex=int(w.is_complex), lo_hz=w.lo_hz,
        bw_hz=w.bw_hz, inputs=inputs, poly=poly, fso=fso, ref_vis=ref_vis, exact_vis=exact_vis,
        exact_counts=counts, geom=geom)
    print(f"{name}: port-vs-reference rel RMS {err:.2e}, flagged FFTs {int((geom[..., 1] == 0).sum())}")


# Benchmark-shaped cases.  Inputs are stored whole; the reference output is stored whole for the
# 6-antenna case and, for 16 antennas at nchan 4096 (15.7 MB of crosses), on every CH_STEP-th
# channel of every baseline plus each (baseline, product)'s sum and power over all channels.
CH_STEP = 16
SHAPE_CASES = {
    # 6 antennas, nchan 1024 (2048-point FFT), 8.4 GHz, 64 MHz: the CPU-runnable benchmark's shape,
    # +-20 us delays flag the edge FFTs
    "shape_c0_6ant_n1024": synth.Workload(nant=6, nchan=1024, nfft=160, bw_hz=64e6, lo_hz=8.4e9, rho=0.05, seed=21),
    # 16 antennas, nchan 4096 = 64^2 (8192-point FFT), 256 MHz: the default benchmark's shape
    "shape_c1_16ant_n4096": synth.Workload(nant=16, nchan=4096, nfft=16, bw_hz=256e6, lo_hz=8.4e9, rho=0.05,
                                           seed=22),
}


def make_shape(name: str, w: synth.Workload):
    d = synth.generate(w)
    inputs = np.stack([x.numpy() for x in d["inputs"]])
    poly, fso = d["poly"], d["fso"]
    ref_vis = O.ref_process(w.nant, w.nchan, w.nfft, w.lo_hz, w.bw_hz, list(inputs), poly, fso)
    cfg_c = O.config_from_workload(w, rotator=O.ROT_FXKERNEL, autos=False)
    port_vis, counts = O.port_process(cfg_c, list(inputs), poly, fso)
    err = O.rel_rms(port_vis, ref_vis)
    assert err < 1e-5, (name, err)
    geom = np.array([[(g.offset, g.valid) for g in (O.geometry(cfg_c, poly[a], fso[a], i) for i in range(w.nfft))]
                     for a in range(w.nant)], dtype=np.int32)
    extra = {}
    if w.nchan > 1024:
        extra = dict(ref_vis_sub=ref_vis[:, :, ::CH_STEP].copy(), ch_step=CH_STEP,
                     ref_sum=ref_vis.astype(np.complex128).sum(axis=-1),
                     ref_pow=(np.abs(ref_vis.astype(np.complex128)) ** 2).sum(axis=-1))
    else:
        extra = dict(ref_vis=ref_vis)
    np.savez_compressed(
        os.path.join(HERE, f"{name}.npz"),
        nant=w.nant, nchan=w.nchan, nfft=w.nfft, nbit=w.nbit, is_complex=int(w.is_complex), lo_hz=w.lo_hz,
        bw_hz=w.bw_hz, inputs=inputs, poly=poly, fso=fso, counts=counts, geom=geom, **extra)
    print(f"{name}: port-vs-reference rel RMS {err:.2e}, flagged FFTs {int((geom[..., 1] == 0).sum())}")


def main():
    if not O.ref_available():
        O.build()
    if not O.ref_available():
        raise SystemExit("the reference library could not be built here")
    only = sys.argv[1:]
    for name, (w, kind) in CASES.items():
        if not only or name in only:
            make(name, w, kind)
    for name, w in SHAPE_CASES.items():
        if not only or name in only:
            make_shape(name, w)
    # 2-bit level table: the reference LUT restated (fxkernel.cpp:15-28), all 256 bytes
    lut = np.stack([O.lut2bit(b) for b in range(256)])
    np.save(os.path.join(HERE, "lut2bit.npy"), lut)


if __name__ == "__main__":
    main()
