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
