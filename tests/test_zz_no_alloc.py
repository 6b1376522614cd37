"""gxc_xcorr_noalloc: the X-stage for callers that cannot allocate device memory.

Callers such as a real-time ingest thread or a host callback may not call
cudaMalloc (it can block and synchronise the device), so this entry point
keeps its scratch in a fixed device array of the library.  The tests call it
through the C ABI on device buffers: twice in a row against gxc_xcorr (which
allocates its own scratch), exactly on small-integer data and within the FP32
tolerance of the other tests on Gaussian data; exactly against a CPU triple
loop; on a problem that needs several passes over the fixed scratch, in FP32
and FP16; and with the device's free memory compared before and after a call.
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


def _reference_call(data, nant, nfft, nchan, fftwidth, autos, precision=L.GXC_PRECISION_FP32):
    nbl = nant * (nant - 1) // 2 + (nant if autos else 0)
    out = np.zeros((nbl, 4, nchan), dtype=np.complex64)
    st = G.lib().gxc_xcorr(C.c_void_p(data.ctypes.data), nant, nfft, nchan, fftwidth, precision,
                           L.GXC_XENGINE_CUDA_CORE, int(autos), C.c_void_p(out.ctypes.data), None)
    assert st == L.GXC_OK, L.status_name(st)
    return out


def _noalloc_call(data, nant, nfft, nchan, fftwidth, autos, precision=L.GXC_PRECISION_FP32):
    import torch
    nbl = nant * (nant - 1) // 2 + (nant if autos else 0)
    d_in = torch.from_numpy(data.view(np.float32)).cuda()
    d_out = torch.full((nbl * 4 * nchan * 2,), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = G.lib().gxc_xcorr_noalloc(C.c_void_p(d_in.data_ptr()), nant, nfft, nchan, fftwidth, precision,
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


def _cpu_triple_loop(data, nant, nfft, nchan, fftwidth, autos):
    """Exact visibilities of small-integer spectra: integer sums over the FFTs of
    X[j][l] * conj(X[k][m]) (products AA, AB, BA, BB; crosses in fxkernel order, then autos),
    then one float32 division by nfft, as the library's final step does."""
    x = data.reshape(nant, 2, nfft, fftwidth)[..., :nchan]
    xr = np.rint(x.real).astype(np.int64)
    xi = np.rint(x.imag).astype(np.int64)
    assert np.array_equal(xr + 1j * xi, x)
    pairs = [(j, k) for j in range(nant) for k in range(j + 1, nant)] + ([(j, j) for j in range(nant)] if autos else [])
    out = np.zeros((len(pairs), 4, nchan), dtype=np.complex64)
    for b, (j, k) in enumerate(pairs):
        for p, (l, m) in enumerate(((0, 0), (0, 1), (1, 0), (1, 1))):
            re = (xr[j, l] * xr[k, m] + xi[j, l] * xi[k, m]).sum(axis=0)
            im = (xi[j, l] * xr[k, m] - xr[j, l] * xi[k, m]).sum(axis=0)
            out[b, p] = (re.astype(np.float32) / np.float32(nfft)) + 1j * (im.astype(np.float32) / np.float32(nfft))
    return out


def _noalloc_blocks(nant, nchan, nfft, autos, esz):
    """FFTs per pass and number of passes of gxc_xcorr_noalloc (its scratch layout)."""
    a256 = lambda x: (x + 255) // 256 * 256  # noqa: E731
    nat = (nant + 1) // 2
    nbl = nant * (nant - 1) // 2 + (nant if autos else 0)
    off_chan = a256(8 * nat * (nat + 1) // 2) + 2 * a256(8 * nbl * 4 * nchan)
    T = min(nfft, (L.GXC_XCORR_NOALLOC_SCRATCH_BYTES - off_chan) // (2 * nant * nchan * esz))
    return T, -(-nfft // T)


def test_noalloc_exact_against_cpu_triple_loop():
    rng = np.random.default_rng(11)
    nant, fftwidth, nchan, nfft = 4, 256, 240, 37
    n = 2 * nant * fftwidth * nfft
    ints = (rng.integers(-5, 6, n) + 1j * rng.integers(-5, 6, n)).astype(np.complex64)
    got = _noalloc_call(ints, nant, nfft, nchan, fftwidth, autos=True)
    assert np.array_equal(got, _cpu_triple_loop(ints, nant, nfft, nchan, fftwidth, autos=True))


def test_noalloc_several_passes_and_fp16():
    """A problem whose channelised data needs three passes over the fixed scratch, the last one
    shorter (FFT offset t0 > 0, the pass stride in the relayout), in FP32 and in FP16, each
    against gxc_xcorr (which allocates its scratch) on the same data."""
    rng = np.random.default_rng(12)
    nant, fftwidth, nchan, nfft = 8, 1024, 1024, 300
    T, nb = _noalloc_blocks(nant, nchan, nfft, True, 8)
    assert nb == 3 and nfft % T != 0, (T, nb)
    n = 2 * nant * fftwidth * nfft
    ints = (rng.integers(-5, 6, n) + 1j * rng.integers(-5, 6, n)).astype(np.complex64)
    got = _noalloc_call(ints, nant, nfft, nchan, fftwidth, autos=True)
    assert np.array_equal(got, _cpu_triple_loop(ints, nant, nfft, nchan, fftwidth, autos=True))
    gauss = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
    for prec in (L.GXC_PRECISION_FP32, L.GXC_PRECISION_FP16):
        got = _noalloc_call(gauss, nant, nfft, nchan, fftwidth, autos=True, precision=prec)
        ref = _reference_call(gauss, nant, nfft, nchan, fftwidth, autos=True, precision=prec)
        assert np.isfinite(got).all()
        assert _rel_rms(got, ref) < FP32_TOL, prec


def test_noalloc_leaves_device_memory_unchanged():
    """Device memory in use (cudaMemGetInfo) is the same before and after a call: nothing is
    allocated.  The first call on the device may load the library's device code, so one call
    runs before the measurement."""
    import torch
    rng = np.random.default_rng(13)
    nant, fftwidth, nchan, nfft = 6, 512, 512, 64
    nbl = nant * (nant - 1) // 2 + nant
    data = (rng.normal(size=2 * nant * fftwidth * nfft) + 1j * rng.normal(size=2 * nant * fftwidth * nfft))
    d_in = torch.from_numpy(data.astype(np.complex64).view(np.float32)).cuda()
    d_out = torch.zeros(nbl * 4 * nchan * 2, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        st = G.lib().gxc_xcorr_noalloc(C.c_void_p(d_in.data_ptr()), nant, nfft, nchan, fftwidth,
                                       L.GXC_PRECISION_FP32, 1, C.c_void_p(d_out.data_ptr()), C.c_void_p(stream))
        assert st == L.GXC_OK, L.status_name(st)
        torch.cuda.synchronize()

    call()
    reserved = torch.cuda.memory_reserved()
    free0, _ = torch.cuda.mem_get_info()
    call()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert torch.cuda.memory_reserved() == reserved


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
