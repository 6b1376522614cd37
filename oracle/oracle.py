"""ctypes bindings for the CPU checkers (TEST INFRASTRUCTURE ONLY).

* ``liboracle.so`` — the C restatement in fxoracle.c: the FP32 port of
  FxKernel::process() (fxkernel/src/fxkernel.cpp:253-368) and the FP64 oracle.
* ``_ref/libfxref.so`` — the reference's own fxkernel.cpp compiled unmodified
  against the IPP-compatible shim (only where oracle/Makefile found the
  reference sources); ``_ref/libfxref_f32.so`` the same with the shim's
  float-internal FFT, timed as the CPU baseline.

Only tests/, the smoke entry point and bench.py's CPU-baseline / reference arm
use this module; the GPU engine never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libfxref.so")
REF_F32_SO = os.path.join(HERE, "_ref", "libfxref_f32.so")

ROT_EXACT = 0
ROT_FXKERNEL = 1


class FxoConfig(C.Structure):
    _fields_ = [("nant", C.c_int), ("nchan", C.c_int), ("nfft", C.c_int), ("nbit", C.c_int),
                ("is_complex", C.c_int), ("lo_hz", C.c_double), ("bw_hz", C.c_double),
                ("rotator", C.c_int), ("autos", C.c_int)]


class FxoGeom(C.Structure):
    _fields_ = [("offset", C.c_int), ("valid", C.c_int), ("frac", C.c_double),
                ("a", C.c_double), ("b", C.c_double)]


def build(force: bool = False) -> None:
    """Compile liboracle.so (and _ref/libfxref.so where the reference exists)."""
    if force or not os.path.exists(ORACLE_SO) or \
            os.path.getmtime(ORACLE_SO) < os.path.getmtime(os.path.join(HERE, "fxoracle.c")):
        subprocess.run(["make", "-s", "-C", HERE, os.path.join(HERE, "liboracle.so")], check=True)
    if not os.path.exists(REF_SO):
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


_lib = None
_ref = None
_ref32 = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = C.CDLL(ORACLE_SO)
        P = C.POINTER
        L.fxo_geometry.argtypes = [P(FxoConfig), P(C.c_double), C.c_double, C.c_int, P(FxoGeom)]
        L.fxo_unpack.argtypes = [P(FxoConfig), C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        L.fxo_lut2bit.argtypes = [C.c_uint8, P(C.c_float)]
        for fn in (L.fxo_port_process,):
            fn.argtypes = [P(FxoConfig), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
            fn.restype = C.c_int
        L.fxo_port_process_range.argtypes = [P(FxoConfig), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                             C.c_int, C.c_void_p, C.c_void_p]
        L.fxo_exact_process.argtypes = [P(FxoConfig), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.fxo_exact_process_masked.argtypes = [P(FxoConfig), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_void_p]
        L.fxo_port_channelise.argtypes = [P(FxoConfig), C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_void_p]
        L.fxo_exact_channelise.argtypes = [P(FxoConfig), C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_void_p]
        L.fxo_bytes_per_antenna.argtypes = [P(FxoConfig)]
        L.fxo_bytes_per_antenna.restype = C.c_size_t
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_SO)
        R.fxref_process.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        R.fxref_process.restype = C.c_int
        R.fxref_save.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p]
        _ref = R
    return _ref


def ref_bench_available() -> bool:
    return os.path.exists(REF_F32_SO)


def ref_bench(nant, nchan, lo_hz, bw_hz, inputs, poly, fso, fft0: int, nfft: int, nthreads: int) -> float:
    """Seconds the reference's own process() (float-FFT shim build) takes for FFTs [fft0, fft0+nfft)
    of a 2-bit real sub-integration, one FxKernel per thread over contiguous FFT slices, as
    fxkernel/src/bench_fxkernel.cpp:93-139 replicates it."""
    global _ref32
    if _ref32 is None:
        R = C.CDLL(REF_F32_SO)
        R.fxref_bench.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
        R.fxref_bench.restype = C.c_double
        _ref32 = R
    arrs, ptrs = _inputs_array(inputs)
    poly, fso = _f64(poly), _f64(fso)
    dt = _ref32.fxref_bench(int(nant), int(nchan), 2, float(lo_hz), float(bw_hz), 0, ptrs, poly.ctypes.data,
                            fso.ctypes.data, int(fft0), int(nfft), int(nthreads))
    if dt < 0:
        raise ValueError(f"reference cannot run this case ({dt})")
    return dt


def make_config(nant, nchan, nfft, nbit=2, is_complex=False, lo_hz=8.4e9, bw_hz=64e6,
                rotator=ROT_EXACT, autos=True) -> FxoConfig:
    return FxoConfig(int(nant), int(nchan), int(nfft), int(nbit), int(bool(is_complex)), float(lo_hz),
                     float(bw_hz), int(rotator), int(bool(autos)))


def config_from_workload(w, rotator=ROT_EXACT, autos=True) -> FxoConfig:
    return make_config(w.nant, w.nchan, w.nfft, w.nbit, w.is_complex, w.lo_hz, w.bw_hz, rotator, autos)


def nbaselines(cfg: FxoConfig) -> int:
    return cfg.nant * (cfg.nant - 1) // 2 + (cfg.nant if cfg.autos else 0)


def _inputs_array(inputs):
    arrs = [np.ascontiguousarray(np.asarray(x, dtype=np.uint8)) for x in inputs]
    ptrs = (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    return arrs, ptrs


def _f64(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64))


def port_process(cfg: FxoConfig, inputs, poly, fso, nthreads: int = 1):
    """FP32 restatement of process(); returns (vis complex64 [nbl,4,nchan], counts int32 [nbl])."""
    arrs, ptrs = _inputs_array(inputs)
    poly, fso = _f64(poly), _f64(fso)
    nbl = nbaselines(cfg)
    vis = np.zeros((nbl, 4, cfg.nchan), dtype=np.complex64)
    counts = np.zeros(nbl, dtype=np.int32)
    rc = lib().fxo_port_process(C.byref(cfg), ptrs, poly.ctypes.data, fso.ctypes.data, int(nthreads),
                                vis.ctypes.data, counts.ctypes.data)
    if rc:
        raise ValueError(f"fxo_port_process failed ({rc})")
    return vis, counts


def port_process_range(cfg: FxoConfig, inputs, poly, fso, fft_begin: int, fft_end: int, normalise=False):
    arrs, ptrs = _inputs_array(inputs)
    poly, fso = _f64(poly), _f64(fso)
    nbl = nbaselines(cfg)
    vis = np.zeros((nbl, 4, cfg.nchan), dtype=np.complex64)
    counts = np.zeros(nbl, dtype=np.int32)
    rc = lib().fxo_port_process_range(C.byref(cfg), ptrs, poly.ctypes.data, fso.ctypes.data, int(fft_begin),
                                      int(fft_end), int(bool(normalise)), vis.ctypes.data, counts.ctypes.data)
    if rc:
        raise ValueError(f"fxo_port_process_range failed ({rc})")
    return vis, counts


def exact_process(cfg: FxoConfig, inputs, poly, fso, mask=None):
    """FP64 oracle; returns (vis complex128 [nbl,4,nchan], counts int32 [nbl]).
    mask: optional uint8 [nant, nfft], 0 flags that antenna's FFT on top of the geometry."""
    arrs, ptrs = _inputs_array(inputs)
    poly, fso = _f64(poly), _f64(fso)
    nbl = nbaselines(cfg)
    vis = np.zeros((nbl, 4, cfg.nchan), dtype=np.complex128)
    counts = np.zeros(nbl, dtype=np.int32)
    m = None if mask is None else np.ascontiguousarray(np.asarray(mask, dtype=np.uint8).reshape(cfg.nant, cfg.nfft))
    rc = lib().fxo_exact_process_masked(C.byref(cfg), ptrs, poly.ctypes.data, fso.ctypes.data,
                                        None if m is None else m.ctypes.data, vis.ctypes.data, counts.ctypes.data)
    if rc:
        raise ValueError(f"fxo_exact_process failed ({rc})")
    return vis, counts


def port_channelise(cfg: FxoConfig, inp, poly3, fso: float, fft: int):
    a = np.ascontiguousarray(np.asarray(inp, dtype=np.uint8))
    p = _f64(poly3)
    out = np.zeros((2, cfg.nchan), dtype=np.complex64)
    rc = lib().fxo_port_channelise(C.byref(cfg), a.ctypes.data, p.ctypes.data, float(fso), int(fft), out.ctypes.data)
    if rc:
        raise ValueError("fxo_port_channelise failed")
    return out


def exact_channelise(cfg: FxoConfig, inp, poly3, fso: float, fft: int):
    a = np.ascontiguousarray(np.asarray(inp, dtype=np.uint8))
    p = _f64(poly3)
    out = np.zeros((2, cfg.nchan), dtype=np.complex128)
    rc = lib().fxo_exact_channelise(C.byref(cfg), a.ctypes.data, p.ctypes.data, float(fso), int(fft), out.ctypes.data)
    if rc:
        raise ValueError("fxo_exact_channelise failed")
    return out


def geometry(cfg: FxoConfig, poly3, fso: float, fft: int):
    g = FxoGeom()
    p = _f64(poly3)
    lib().fxo_geometry(C.byref(cfg), p.ctypes.data_as(C.POINTER(C.c_double)), float(fso), int(fft), C.byref(g))
    return g


def lut2bit(byte: int):
    out = (C.c_float * 4)()
    lib().fxo_lut2bit(C.c_uint8(byte), out)
    return np.array(out[:], dtype=np.float32)


def unpack(cfg: FxoConfig, inp, offset: int, nsamp: int):
    a = np.ascontiguousarray(np.asarray(inp, dtype=np.uint8))
    p0 = np.zeros(nsamp, dtype=np.complex64)
    p1 = np.zeros(nsamp, dtype=np.complex64)
    lib().fxo_unpack(C.byref(cfg), a.ctypes.data, int(offset), int(nsamp), p0.ctypes.data, p1.ctypes.data)
    return p0, p1


def ref_process(nant, nchan, nfft, lo_hz, bw_hz, inputs, poly, fso):
    """The reference FxKernel::process() (2-bit real, square nchan); complex64 [nbl,4,nchan]."""
    arrs, ptrs = _inputs_array(inputs)
    poly, fso = _f64(poly), _f64(fso)
    nbl = nant * (nant - 1) // 2
    vis = np.zeros((nbl, 4, nchan), dtype=np.complex64)
    rc = ref().fxref_process(int(nant), int(nchan), int(nfft), 2, float(lo_hz), float(bw_hz), 0, ptrs,
                             poly.ctypes.data, fso.ctypes.data, vis.ctypes.data)
    if rc:
        raise ValueError(f"reference cannot run this case ({rc})")
    return vis


def ref_save(nant, nchan, nfft, lo_hz, bw_hz, inputs, poly, fso, path: str) -> None:
    """The reference's process() then saveVisibilities(path) (fxkernel/src/fxkernel.cpp:370-412)."""
    arrs, ptrs = _inputs_array(inputs)
    poly, fso = _f64(poly), _f64(fso)
    rc = ref().fxref_save(int(nant), int(nchan), int(nfft), 2, float(lo_hz), float(bw_hz), 0, ptrs,
                          poly.ctypes.data, fso.ctypes.data, path.encode())
    if rc:
        raise ValueError(f"reference cannot run this case ({rc})")


def rel_rms(a, b) -> float:
    """||a-b|| / ||b|| over all elements."""
    a = np.asarray(a).astype(np.complex128)
    b = np.asarray(b).astype(np.complex128)
    den = np.sqrt(np.sum(np.abs(b) ** 2))
    return float(np.sqrt(np.sum(np.abs(a - b) ** 2)) / (den if den > 0 else 1.0))


def rel_rms_per_product(a, b):
    """Relative RMS error per (baseline, product) over channels: array [nbl, 4]."""
    a = np.asarray(a).astype(np.complex128)
    b = np.asarray(b).astype(np.complex128)
    num = np.sqrt(np.sum(np.abs(a - b) ** 2, axis=-1))
    den = np.sqrt(np.sum(np.abs(b) ** 2, axis=-1))
    return num / np.where(den > 0, den, 1.0)


# ---------------------------------------------------------------- polarisation conversion (test oracle)
def lin2circ_voltages(x, gains=None):
    """Voltage-domain linear->circular conversion of channelised data x[nant][2][..][nchan]
    (complex), restating examples/chris/bench/gpubench.cu:145-160: per antenna and
    channel, P1' = g1*P1 - g2*P2, P2' = g1*P1 + g2*P2.  gains [nant][2][nchan]
    (g1, g2); None = ideal feeds g1 = 1/sqrt2, g2 = i/sqrt2."""
    x = np.asarray(x, dtype=np.complex128)
    nant, nchan = x.shape[0], x.shape[-1]
    if gains is None:
        g = np.empty((nant, 2, nchan), np.complex128)
        g[:, 0] = 1 / np.sqrt(2)
        g[:, 1] = 1j / np.sqrt(2)
    else:
        g = np.asarray(gains, dtype=np.complex128).reshape(nant, 2, nchan)
    shape = (nant,) + (1,) * (x.ndim - 3) + (nchan,)
    p1 = x[:, 0] * g[:, 0].reshape(shape)
    p2 = x[:, 1] * g[:, 1].reshape(shape)
    return np.stack([p1 - p2, p1 + p2], axis=1)


def correlate_voltages(x, autos=True):
    """Visibilities [nbl][4][nchan] of channelised voltages x[nant][2][nfft][nchan]:
    mean over FFTs of X_j,l * conj(X_k,m), crosses in fxkernel order
    (fxkernel/src/fxkernel.cpp:328-355) then autos."""
    x = np.asarray(x, dtype=np.complex128)
    nant = x.shape[0]
    pairs = [(j, k) for j in range(nant - 1) for k in range(j + 1, nant)]
    if autos:
        pairs += [(j, j) for j in range(nant)]
    out = np.empty((len(pairs), 4, x.shape[-1]), np.complex128)
    for b, (j, k) in enumerate(pairs):
        for l in range(2):
            for m in range(2):
                out[b, 2 * l + m] = (x[j, l] * np.conj(x[k, m])).mean(axis=0)
    return out
