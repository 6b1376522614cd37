"""GPU parity tests: the libgxcorr CUDA path against the oracle and the
reference's own outputs, through the FxKernel-compatible API over the C ABI.

Tolerances: FP32 end to end <= 1e-5 relative RMS per (baseline, product);
FP16 channelised data <= 1e-3 relative RMS; counts and flags bit-exact.
"""
import numpy as np
import pytest

from gcorr_gb300 import FxKernel, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5
FP16_TOL = 1e-3


def _run(w_or_d, inputs, poly, fso, **kw):
    d = w_or_d
    fx = FxKernel(int(d["nant"]), int(d["nchan"]), int(d["nfft"]), int(d["nbit"]), float(d["lo_hz"]),
                  float(d["bw_hz"]), bool(d["is_complex"]), **kw)
    fx.setInputData([x if hasattr(x, "data_ptr") else np.ascontiguousarray(x) for x in inputs])
    fx.setDelays(poly, fso)
    fx.process()
    vis, counts = fx.visibilities(), fx.baseline_counts()
    flags = fx.valid_flags()
    fx.close()
    return vis, counts, flags


def _wd(w: synth.Workload):
    return dict(nant=w.nant, nchan=w.nchan, nfft=w.nfft, nbit=w.nbit, is_complex=int(w.is_complex), lo_hz=w.lo_hz,
                bw_hz=w.bw_hz)


@pytest.mark.parametrize("engine", ["tensor", "cuda_core"])
def test_golden_fxkernel_mode_matches_reference(golden_cases, engine):
    """fxkernel rotator, crosses only: the reference's own process() output."""
    for name, d in golden_cases.items():
        vis, counts, flags = _run(d, d["inputs"], d["poly"], d["fso"], rotator="fxkernel", autos=False,
                                  x_engine=engine)
        ref = d["ref_vis"]
        assert vis.shape == ref.shape
        err = O.rel_rms_per_product(vis, ref)
        assert err.max() < FP32_TOL, (name, err.max())
        nx = int(d["nant"]) * (int(d["nant"]) - 1) // 2
        assert np.array_equal(counts, d["exact_counts"][:nx]), name
        assert np.array_equal(flags, d["geom"][..., 1].astype(np.uint8)), name


@pytest.mark.parametrize("engine", ["tensor", "cuda_core"])
def test_benchmark_shapes_match_reference(shape_cases, engine):
    """fxkernel rotator, crosses only, at the benchmark shapes: the reference's own process()
    output for 6 antennas x nchan 1024 (2048-point FFTs) and 16 antennas x nchan 4096
    (8192-point FFTs, the packed-pair F-stage), with flagged edge FFTs."""
    from conftest import reference_checks
    assert len(shape_cases) == 2
    for name, d in shape_cases.items():
        vis, counts, flags = _run(d, d["inputs"], d["poly"], d["fso"], rotator="fxkernel", autos=False,
                                  x_engine=engine)
        r = reference_checks(vis, d)
        assert r["per_product"] < FP32_TOL and r.get("sum", 0.0) < FP32_TOL and r.get("power", 0.0) < FP32_TOL, \
            (name, r)
        assert np.array_equal(counts, d["counts"]), name
        assert np.array_equal(flags, d["geom"][..., 1].astype(np.uint8)), name


@pytest.mark.parametrize("engine", ["tensor", "cuda_core"])
def test_benchmark_shapes_exact_mode_vs_fp64(shape_cases, engine):
    for name, d in shape_cases.items():
        cfg = O.make_config(int(d["nant"]), int(d["nchan"]), int(d["nfft"]), 2, False, float(d["lo_hz"]),
                            float(d["bw_hz"]), O.ROT_EXACT, True)
        ref, rc = O.exact_process(cfg, list(d["inputs"]), d["poly"], d["fso"])
        vis, counts, _ = _run(d, d["inputs"], d["poly"], d["fso"], rotator="exact", autos=True, x_engine=engine)
        assert np.array_equal(counts, rc), name
        err = O.rel_rms_per_product(vis, ref)
        assert err.max() < FP32_TOL, (name, err.max())


# FP8 (E4M3, 3 mantissa bits) is reported with its measured error; this bound only catches breakage.
FP8_TOL = 0.12


@pytest.mark.parametrize("nant,nchan,nfft,is_complex,precision", [
    (32, 8192, 8, False, "fp16"), (32, 8192, 8, False, "fp8"),
    (64, 32768, 4, True, "fp16"), (64, 32768, 4, True, "fp8"),
    (32, 16384, 4, True, "fp16")])
def test_reduced_precision_large_arrays_vs_fp64(nant, nchan, nfft, is_complex, precision):
    """FP16 and FP8 channelised data on the tensor-core X-stage at 32 and 64 antennas with
    16384- and 32768-point windows (the FP16-buffer F-stage), against the FP64 oracle."""
    w = synth.Workload(nant=nant, nchan=nchan, nfft=nfft, nbit=8 if is_complex else 2, is_complex=is_complex,
                       bw_hz=128e6, rho=0.05, seed=nant * 7 + nfft, offset_us=2.0)
    d = synth.generate(w)
    inputs = [x.numpy() for x in d["inputs"]]
    ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), inputs, d["poly"], d["fso"])
    vis, counts, _ = _run(_wd(w), inputs, d["poly"], d["fso"], precision=precision, x_engine="tensor")
    assert np.array_equal(counts, rc)
    err = O.rel_rms_per_product(vis, ref)
    nx = nant * (nant - 1) // 2
    tol = FP16_TOL if precision == "fp16" else FP8_TOL
    assert err.max() < tol, (err.max(), float(np.median(err)))
    assert err[nx:, [0, 3]].max() < tol / 2, err[nx:, [0, 3]].max()  # power spectra (autos AA, BB)


@pytest.mark.parametrize("engine", ["tensor", "cuda_core"])
def test_golden_exact_mode_matches_fp64_oracle(golden_cases, engine):
    for name, d in golden_cases.items():
        vis, counts, _ = _run(d, d["inputs"], d["poly"], d["fso"], rotator="exact", autos=True, x_engine=engine)
        err = O.rel_rms_per_product(vis, d["exact_vis"])
        assert err.max() < FP32_TOL, (name, err.max())
        assert np.array_equal(counts, d["exact_counts"]), name


@pytest.mark.parametrize("nchan,is_complex", [(128, False), (256, False), (512, False), (1024, False),
                                              (2048, False), (4096, False), (8192, False), (16384, False),
                                              (256, True), (1024, True), (4096, True), (8192, True),
                                              (16384, True), (32768, True)])
def test_fft_sizes_vs_fp64(nchan, is_complex):
    nfft = 4 if nchan * (1 if is_complex else 2) >= 32768 else 6 if nchan * (1 if is_complex else 2) >= 8192 else 12
    w = synth.Workload(nant=2, nchan=nchan, nfft=nfft, nbit=8 if is_complex else 2, is_complex=is_complex,
                       bw_hz=64e6, seed=nchan + is_complex, offset_us=0.5)
    d = synth.random_bytes(w)
    inputs = [x.numpy() for x in d["inputs"]]
    cfg = O.config_from_workload(w, O.ROT_EXACT, True)
    ref, rc = O.exact_process(cfg, inputs, d["poly"], d["fso"])
    vis, counts, _ = _run(_wd(w), inputs, d["poly"], d["fso"])
    assert np.array_equal(counts, rc)
    assert O.rel_rms_per_product(vis, ref).max() < FP32_TOL


@pytest.mark.parametrize("nant", [1, 2, 3, 5, 8])
def test_antenna_counts_vs_fp64(nant):
    w = synth.Workload(nant=nant, nchan=256, nfft=20, bw_hz=32e6, seed=100 + nant, offset_us=10.0)
    d = synth.random_bytes(w)
    inputs = [x.numpy() for x in d["inputs"]]
    ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), inputs, d["poly"], d["fso"])
    vis, counts, _ = _run(_wd(w), inputs, d["poly"], d["fso"])
    assert np.array_equal(counts, rc)
    assert O.rel_rms_per_product(vis, ref).max() < FP32_TOL


def test_fxkernel_rotator_8192_point_vs_port():
    """The fxkernel-compatible rotator (its stride/substride table split and step quirk) through
    the 8192-point packed-pair F-stage (2-bit real, nchan 4096 = 64^2; complex 8192 is not square):
    crosses within the FP32 tolerance of the FP32 port of fxkernel's process(), counts bit-exact."""
    w = synth.Workload(nant=3, nchan=4096, nfft=10, bw_hz=64e6, rho=0.3, seed=55, offset_us=5.0)
    d = synth.generate(w)
    inputs = [x.numpy() for x in d["inputs"]]
    ref, rc = O.port_process(O.config_from_workload(w, O.ROT_FXKERNEL, False), inputs, d["poly"], d["fso"])
    vis, counts, _ = _run(_wd(w), inputs, d["poly"], d["fso"], rotator="fxkernel", autos=False)
    assert np.array_equal(counts, rc)
    assert O.rel_rms_per_product(vis, ref).max() < FP32_TOL


def test_8bit_complex_physics_vs_fp64():
    w = synth.Workload(nant=3, nchan=512, nfft=24, nbit=8, is_complex=True, bw_hz=32e6, rho=0.3, seed=77)
    d = synth.generate(w)
    inputs = [x.numpy() for x in d["inputs"]]
    ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), inputs, d["poly"], d["fso"])
    vis, counts, _ = _run(_wd(w), inputs, d["poly"], d["fso"])
    assert np.array_equal(counts, rc)
    assert O.rel_rms_per_product(vis, ref).max() < FP32_TOL


def test_fp16_channelised_vs_fp64():
    w = synth.Workload(nant=4, nchan=1024, nfft=40, bw_hz=64e6, rho=0.2, seed=88)
    d = synth.generate(w)
    inputs = [x.numpy() for x in d["inputs"]]
    ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), inputs, d["poly"], d["fso"])
    vis, counts, _ = _run(_wd(w), inputs, d["poly"], d["fso"], precision="fp16", x_engine="cuda_core")
    assert np.array_equal(counts, rc)
    err = O.rel_rms_per_product(vis, ref)
    assert err.max() < FP16_TOL, err.max()


@pytest.mark.parametrize("fft_len", [8192, 16384, 32768])
@pytest.mark.parametrize("is_complex", [True, False])
@pytest.mark.parametrize("precision", ["fp16", "fp8"])
def test_large_fft_reduced_precision_vs_fp64(fft_len, is_complex, precision):
    """8192-point windows go through the tensor-core F-stage (2-bit real) or the packed-pair one
    (8-bit complex); 16384- and 32768-point windows with FP16 or FP8 channelised data through the
    F-stage whose intermediate spectrum is held in FP16 shared memory (two extra 2^-11 roundings).
    FP16 must stay within the FP16 tolerance of the FP64 oracle.  FP8: crosses within 6 % (the
    E4M3 bound of the other FP8 tests); the power spectra's E4M3 rounding error only averages
    over the 8 FFTs here (1 % holds for 200 FFTs; about 2.3 % is expected for 8), bound 3.5 %."""
    nchan = fft_len if is_complex else fft_len // 2
    w = synth.Workload(nant=3, nchan=nchan, nfft=8, nbit=8 if is_complex else 2, is_complex=is_complex,
                       bw_hz=64e6, rho=0.3, seed=321 + int(is_complex))
    d = synth.generate(w)
    inputs = [x.numpy() for x in d["inputs"]]
    ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), inputs, d["poly"], d["fso"])
    vis, counts, _ = _run(_wd(w), inputs, d["poly"], d["fso"], precision=precision, x_engine="cuda_core")
    assert np.array_equal(counts, rc)
    err = O.rel_rms_per_product(vis, ref)
    if precision == "fp16":
        assert err.max() < FP16_TOL, err.max()
    else:
        ncross = w.nant * (w.nant - 1) // 2
        assert err[:ncross].max() < 0.06, err[:ncross].max()
        assert err[ncross:][:, [0, 3]].max() < 0.035, err[ncross:].max()


def test_device_inputs_and_blocks_match_host_inputs():
    import torch
    w = synth.Workload(nant=3, nchan=512, nfft=50, bw_hz=32e6, seed=5, offset_us=8.0)
    d = synth.random_bytes(w)
    host = [x.numpy() for x in d["inputs"]]
    v_host, c_host, _ = _run(_wd(w), host, d["poly"], d["fso"])
    dev = [x.cuda() for x in d["inputs"]]
    v_dev, c_dev, _ = _run(_wd(w), dev, d["poly"], d["fso"], fft_block=7)  # ragged last block
    assert np.array_equal(c_host, c_dev)
    assert O.rel_rms(v_dev, v_host) < 1e-6
    torch.cuda.synchronize()


def test_host_input_chunks_match_device_input():
    """Host inputs of 8.6 MB per antenna load on the handle's copy stream in eight time-ordered
    chunks, each F-stage block (256 FFTs) waiting only for its chunk; delays of both signs.
    The visibilities must equal those of the same data in device memory bit for bit."""
    import torch
    w = synth.Workload(nant=4, nchan=4096, nfft=2100, bw_hz=64e6, seed=61, offset_us=60.0)
    d = synth.random_bytes(w)
    poly = np.array(d["poly"], dtype=np.float64)
    poly[:, 1] += np.array([3.0, -3.0, 1.0, -0.5]) * w.fft_time / w.nfft
    host = [x.pin_memory() for x in d["inputs"]]
    v_host, c_host, _ = _run(_wd(w), host, poly, d["fso"], fft_block=256)
    dev = [x.cuda() for x in d["inputs"]]
    v_dev, c_dev, _ = _run(_wd(w), dev, poly, d["fso"], fft_block=256)
    assert np.array_equal(c_host, c_dev)
    assert np.array_equal(v_host, v_dev)
    torch.cuda.synchronize()


def test_accumulate_adds():
    w = synth.Workload(nant=2, nchan=256, nfft=10, bw_hz=32e6, seed=9)
    d = synth.random_bytes(w)
    fx = FxKernel(w.nant, w.nchan, w.nfft, 2, w.lo_hz, w.bw_hz, False)
    fx.setInputData([x.numpy() for x in d["inputs"]])
    fx.setDelays(d["poly"], d["fso"])
    fx.process()
    acc = np.zeros((fx.nbaselines, 4, w.nchan), dtype=np.complex64)
    fx.accumulate(acc)
    fx.accumulate(acc)
    v = fx.visibilities()
    assert np.allclose(acc, 2 * v, rtol=1e-6, atol=1e-6)
    fx.close()


def test_call_order_errors():
    from gcorr_gb300 import GxcError
    fx = FxKernel(2, 256, 4, 2, 8.4e9, 32e6, False)
    with pytest.raises(GxcError):
        fx.process()
    fx.close()


def test_misaligned_device_input_is_rejected_before_any_launch():
    import torch
    from gcorr_gb300 import GxcError
    w = synth.Workload(nant=2, nchan=256, nfft=4, bw_hz=32e6, seed=3)
    fx = FxKernel(w.nant, w.nchan, w.nfft, 2, w.lo_hz, w.bw_hz, False)
    big = torch.zeros(w.bytes_per_antenna + 64, dtype=torch.uint8, device="cuda")
    with pytest.raises(GxcError):
        fx.setInputData([big[1:1 + w.bytes_per_antenna], big[1:1 + w.bytes_per_antenna]])
    fx.close()


@pytest.mark.parametrize("precision,engine,tol", [("fp32", "cuda_core", FP32_TOL), ("fp32", "tensor", FP32_TOL),
                                                  ("fp16", "tensor", FP16_TOL),
                                                  ("fp16", "cuda_core", FP16_TOL)])
def test_long_integration_accuracy_vs_fp64(precision, engine, tol):
    """8192 FFTs accumulated in one block: the accumulation error must stay inside
    the tolerance of the precision (per baseline and product, autos included)."""
    w = synth.Workload(nant=4, nchan=256, nfft=8192, bw_hz=32e6, rho=0.05, seed=5)
    d = synth.generate(w)
    inputs = [x.numpy() for x in d["inputs"]]
    ref, rc = O.exact_process(O.config_from_workload(w, O.ROT_EXACT, True), inputs, d["poly"], d["fso"])
    vis, counts, _ = _run(_wd(w), inputs, d["poly"], d["fso"], precision=precision, x_engine=engine,
                          fft_block=w.nfft)
    assert np.array_equal(counts, rc)
    assert O.rel_rms_per_product(vis, ref).max() < tol
