"""CPU tests of the C ABI: the library loads, exports every declared symbol and
validates configurations the way fxkernel does (fxkernel/src/fxkernel.cpp:46-63),
with status codes instead of exit()."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT, gpu_available
import gcorr_gb300 as G
from gcorr_gb300 import _lib as L
from gcorr_gb300 import synth
from oracle import oracle as O


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gxc_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(L.LIB_PATH)
    names = _declared("gxc.h")
    assert names, "no declarations parsed"
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(names) == sorted(L.EXPORTS)
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True).stdout
    for n in names:
        assert re.search(rf"\bT {n}\b", out), n


def test_header_constants_match_bindings():
    txt = open(os.path.join(ROOT, "include", "gxc.h")).read()
    m = re.search(r"#define GXC_XCORR_NOALLOC_SCRATCH_BYTES \((\d+)u << (\d+)\)", txt)
    assert m, "scratch size define"
    assert int(m.group(1)) << int(m.group(2)) == L.GXC_XCORR_NOALLOC_SCRATCH_BYTES


def _status(**kw):
    cfg = G.make_config(**kw)
    return L.lib().gxc_validate_config(C.byref(cfg))


def test_validation_codes():
    assert _status(nant=4, nchan=1024, nfft=10) == L.GXC_OK
    assert _status(nant=4, nchan=1000, nfft=10) == L.GXC_ERR_INVALID_ARGUMENT       # FFT not a power of two
    assert _status(nant=4, nchan=1024, nfft=10, nbit=4) == L.GXC_ERR_INVALID_ARGUMENT
    assert _status(nant=0, nchan=1024, nfft=10) == L.GXC_ERR_INVALID_ARGUMENT
    assert _status(nant=4, nchan=1024, nfft=0) == L.GXC_ERR_INVALID_ARGUMENT
    assert _status(nant=4, nchan=1024, nfft=10, bw=0.0) == L.GXC_ERR_INVALID_ARGUMENT
    # the fxkernel rotator needs a square nchan, like the reference constructor
    assert _status(nant=4, nchan=2048, nfft=10, rotator="fxkernel") == L.GXC_ERR_INVALID_ARGUMENT
    assert _status(nant=4, nchan=2048, nfft=10, rotator="exact") == L.GXC_OK
    # formats outside 2-bit real / 8-bit complex
    assert _status(nant=4, nchan=1024, nfft=10, nbit=8, is_complex=False) == L.GXC_ERR_UNSUPPORTED
    assert _status(nant=4, nchan=1024, nfft=10, nbit=2, is_complex=True) == L.GXC_ERR_UNSUPPORTED
    assert _status(nant=4, nchan=1024, nfft=10, nbit=8, is_complex=True) == L.GXC_OK
    assert _status(nant=4, nchan=64, nfft=10) == L.GXC_ERR_UNSUPPORTED              # FFT below 256
    # the tensor-core FFT: 8192-point windows of 2-bit real data with FP16 / FP8 output only
    assert _status(nant=4, nchan=4096, nfft=10, precision="fp16", fft_engine="tensor") == L.GXC_OK
    assert _status(nant=4, nchan=4096, nfft=10, precision="fp8", fft_engine="tensor") == L.GXC_OK
    assert _status(nant=4, nchan=4096, nfft=10, precision="fp32", fft_engine="tensor") == L.GXC_ERR_UNSUPPORTED
    assert _status(nant=4, nchan=2048, nfft=10, precision="fp16", fft_engine="tensor") == L.GXC_ERR_UNSUPPORTED
    assert _status(nant=4, nchan=4096, nfft=10, precision="fp16", fft_engine=7) == L.GXC_ERR_INVALID_ARGUMENT
    assert _status(nant=4, nchan=4096, nfft=10, x_split="on") == L.GXC_OK
    assert _status(nant=4, nchan=4096, nfft=10, x_split=5) == L.GXC_ERR_INVALID_ARGUMENT
    assert _status(nant=4, nchan=4096, nfft=10, precision="fp8", fp8_scaling="handle") == L.GXC_OK
    assert _status(nant=4, nchan=4096, nfft=10, precision="fp8", fp8_scaling=3) == L.GXC_ERR_INVALID_ARGUMENT


def test_input_bytes_match_reference_formula():
    for kw in [dict(nant=6, nchan=1024, nfft=15625), dict(nant=3, nchan=256, nfft=7)]:
        cfg = G.make_config(**kw)
        got = L.lib().gxc_input_bytes_per_antenna(C.byref(cfg))
        # fxkernel/src/common.cpp:82 for 2-bit real: nchan*2*(nfft+1)*nbit/8*npol
        assert got == kw["nchan"] * 2 * (kw["nfft"] + 1) * 2 // 8 * 2
        assert got == O.lib().fxo_bytes_per_antenna(C.byref(O.make_config(kw["nant"], kw["nchan"], kw["nfft"])))
    cfg = G.make_config(nant=2, nchan=512, nfft=9, nbit=8, is_complex=True)
    assert L.lib().gxc_input_bytes_per_antenna(C.byref(cfg)) == 4 * 512 * 10
    w = synth.Workload(nant=2, nchan=512, nfft=9, nbit=8, is_complex=True)
    assert w.bytes_per_antenna == 4 * 512 * 10


def test_num_baselines():
    assert L.lib().gxc_num_baselines(C.byref(G.make_config(nant=6, nchan=1024, nfft=1, autos=True))) == 21
    assert L.lib().gxc_num_baselines(C.byref(G.make_config(nant=6, nchan=1024, nfft=1, autos=False))) == 15


def test_status_strings():
    for s in range(7):
        assert L.lib().gxc_status_string(s)


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_create_without_gpu_fails_loudly():
    with pytest.raises((L.GxcError, ValueError)):
        G.FxKernel(4, 256, 8, 2, 8.4e9, 32e6, False)


def test_visibility_text_roundtrip(tmp_path):
    import numpy as np
    from gcorr_gb300.visio import load_visibilities, save_visibilities
    rng = np.random.default_rng(0)
    v = (rng.normal(size=(3, 4, 16)) + 1j * rng.normal(size=(3, 4, 16))).astype(np.complex64)
    p = tmp_path / "vis.out"
    save_visibilities(str(p), v, 64e6)
    f, back = load_visibilities(str(p), 3)
    assert np.allclose(back, v, atol=1e-5)
    assert np.allclose(f, (np.arange(16) + 0.5) / 16 * 64.0)


def _end_bytes_at(offset, F, is_complex):
    end = 4 * (offset + F) if is_complex else (offset + F + 1) // 2
    return (end + 15) // 16 * 16


def _window_end_bytes(ocfg, poly3, fso, fft, F, is_complex):
    """Last byte (exclusive) of the 16-byte staged window of one FFT, from the oracle's geometry
    (fxkernel.cpp:288-309); 0 when the FFT is flagged."""
    g = O.geometry(ocfg, poly3, fso, fft)
    return _end_bytes_at(g.offset, F, is_complex) if g.valid else 0


@pytest.mark.parametrize("is_complex", [False, True])
@pytest.mark.parametrize("case", ["synth", "fast", "vertex", "flagged"])
def test_input_bytes_for_ffts_bounds_every_window(is_complex, case):
    """gxc_input_bytes_for_ffts (the streaming pipeline's per-block input bound) covers every
    window the FFTs of the block read, and exceeds the tightest bound by little more than the
    delay change over the block."""
    import numpy as np
    nchan, nfft, T = (512, 96, 12)
    nbit = 8 if is_complex else 2
    w = synth.Workload(nant=4, nchan=nchan, nfft=nfft, nbit=nbit, is_complex=is_complex, bw_hz=32e6, seed=7,
                       offset_us=40.0)
    poly, fso = synth.delay_model(w)
    poly = np.array(poly, dtype=np.float64)
    F = nchan if is_complex else 2 * nchan
    Ts = 1.0 / 32e6 if is_complex else 1.0 / 64e6
    fft_s = F * Ts
    if case == "fast":      # delays sweeping several FFTs over the sub-integration, both signs
        poly[:, 1] = np.array([3.0, -3.0, 1.5, -0.7]) * fft_s / 8
    elif case == "vertex":  # a delay minimum inside the sub-integration
        poly[:, 0] = 4.0 * fft_s / nfft ** 2
        poly[:, 1] = -2.0 * poly[:, 0] * (nfft * np.array([0.3, 0.5, 0.55, 0.8]))
    elif case == "flagged":  # windows pushed off both ends of the buffer
        poly[:, 2] = np.array([-1.5, 1.5, 0.0, 0.2]) * nfft * fft_s
    cfg = G.make_config(nant=4, nchan=nchan, nfft=nfft, nbit=nbit, is_complex=is_complex, bw=32e6)
    ocfg = O.make_config(4, nchan, nfft, nbit, is_complex, 8.4e9, 32e6)
    fsoa = np.ascontiguousarray(fso, dtype=np.float64)
    P = C.POINTER(C.c_double)
    total = L.lib().gxc_input_bytes_per_antenna(C.byref(cfg))
    for t0 in range(0, nfft, T):
        nt = min(T, nfft - t0)
        got = L.lib().gxc_input_bytes_for_ffts(C.byref(cfg), poly.ctypes.data_as(P), fsoa.ctypes.data_as(P), t0, nt)
        need = max(_window_end_bytes(ocfg, poly[a], fso[a], t, F, is_complex)
                   for a in range(4) for t in range(t0, t0 + nt))
        assert need <= got <= total, (t0, need, got)
        # looseness: the delay change across the block (in bytes) plus the rounding margins
        nd = [[round((np.polyval(poly[a], t + 0.5) - fso[a]) / Ts) for t in range(t0, t0 + nt)] for a in range(4)]
        spread = max(max(v) - min(v) for v in nd)
        per_sample = 4 if is_complex else 0.5
        # a bound clamped at the last valid window (maxoffset) may exceed windows flagged off the end
        clamp = _end_bytes_at((nfft - 1) * F, F, is_complex) + 16
        if need > 0 and got < clamp:
            assert got - need <= (spread + 8) * per_sample + 48, (t0, need, got, spread)
    assert L.lib().gxc_input_bytes_for_ffts(C.byref(cfg), poly.ctypes.data_as(P), fsoa.ctypes.data_as(P), 0, 0) == 0
    assert L.lib().gxc_input_bytes_for_ffts(C.byref(cfg), poly.ctypes.data_as(P), fsoa.ctypes.data_as(P),
                                            nfft - 1, 2) == 0
