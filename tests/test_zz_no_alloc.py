"""gxc_xcorr_noalloc: the X-stage for callers that cannot allocate device memory.

Callers such as a real-time ingest thread or a host callback may not call
cudaMalloc (it can block and synchronise the device), so this entry point
keeps its scratch in a fixed device array of the library.  The test calls it
twice in a row through the C ABI, on device buffers, and checks each result
against gxc_xcorr (which allocates its own scratch): exactly on small-integer
data, and within the FP32 tolerance of the other tests on Gaussian data.
The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import gcorr_gb300 as G
from gcorr_gb300 import _lib as L

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5


def _rel_rms(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.sqrt(np.sum(np.abs(a - b) ** 2) / max(np.sum(np.abs(b) ** 2), 1e-300)))


def _reference_call(data, nant, nfft, nchan, fftwidth, autos):
    nbl = nant * (nant - 1) // 2 + (nant if autos else 0)
    out = np.zeros((nbl, 4, nchan), dtype=np.complex64)
    st = G.lib().gxc_xcorr(C.c_void_p(data.ctypes.data), nant, nfft, nchan, fftwidth, L.GXC_PRECISION_FP32,
                           L.GXC_XENGINE_CUDA_CORE, int(autos), C.c_void_p(out.ctypes.data), None)
    assert st == L.GXC_OK, L.status_name(st)
    return out


def _noalloc_call(data, nant, nfft, nchan, fftwidth, autos):
    import torch
    nbl = nant * (nant - 1) // 2 + (nant if autos else 0)
    d_in = torch.from_numpy(data.view(np.float32)).cuda()
    d_out = torch.full((nbl * 4 * nchan * 2,), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = G.lib().gxc_xcorr_noalloc(C.c_void_p(d_in.data_ptr()), nant, nfft, nchan, fftwidth, L.GXC_PRECISION_FP32,
                                   int(autos), C.c_void_p(d_out.data_ptr()), C.c_void_p(stream))
    assert st == L.GXC_OK, L.status_name(st)
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(np.complex64).reshape(nbl, 4, nchan)


def test_noalloc_matches_allocating_entry_point_twice():
    rng = np.random.default_rng(7)
    # call 1: small-integer data (exact sums), crosses only
    nant, fftwidth, nchan, nfft = 5, 1024, 1024, 100
    n = 2 * nant * fftwidth * nfft
    ints = (rng.integers(-5, 6, n) + 1j * rng.integers(-5, 6, n)).astype(np.complex64)
    a1 = _noalloc_call(ints, nant, nfft, nchan, fftwidth, autos=False)
    assert np.array_equal(a1, _reference_call(ints, nant, nfft, nchan, fftwidth, autos=False))
    # call 2: Gaussian data, autos on, a different shape over the same scratch
    nant, fftwidth, nchan, nfft = 6, 512, 256, 300
    n = 2 * nant * fftwidth * nfft
    gauss = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
    a2 = _noalloc_call(gauss, nant, nfft, nchan, fftwidth, autos=True)
    ref2 = _reference_call(gauss, nant, nfft, nchan, fftwidth, autos=True)
    assert np.isfinite(a2).all()
    assert _rel_rms(a2, ref2) < FP32_TOL


def test_noalloc_rejects_oversize_and_host_buffers():
    import torch
    # accumulators alone exceed the fixed scratch: 64 antennas x 8192 channels
    nant, nchan, nfft, fftwidth = 64, 8192, 1, 8192
    d_in = torch.zeros(2 * nant * nfft * fftwidth * 2, dtype=torch.float32, device="cuda")
    d_out = torch.zeros(16, dtype=torch.float32, device="cuda")
    st = G.lib().gxc_xcorr_noalloc(C.c_void_p(d_in.data_ptr()), nant, nfft, nchan, fftwidth, L.GXC_PRECISION_FP32,
                                   1, C.c_void_p(d_out.data_ptr()), None)
    assert st == L.GXC_ERR_INVALID_ARGUMENT
    host = np.zeros(2 * 2 * 4 * 256 * 2, dtype=np.float32)
    st = G.lib().gxc_xcorr_noalloc(C.c_void_p(host.ctypes.data), 2, 4, 256, 256, L.GXC_PRECISION_FP32, 1,
                                   C.c_void_p(d_out.data_ptr()), None)
    assert st == L.GXC_ERR_INVALID_ARGUMENT
