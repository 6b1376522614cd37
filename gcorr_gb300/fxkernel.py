"""Python host mirror of the reference FxKernel API over the libgxcorr C ABI.

Same names, argument meaning and error behaviour as fxkernel/src/fxkernel.h:29-64
(``FxKernel(nant, nchan, nfft, nbit, lo, bw, is_complex)``, ``setInputData``,
``setDelays``, ``process``, ``accumulate``, ``saveVisibilities``), except that
invalid configurations raise ``ValueError`` instead of calling ``exit(1)``
(fxkernel/src/fxkernel.cpp:46-63).  All compute runs in libgxcorr.so on the GPU;
there is no CPU fallback: if the library or a GPU is missing, construction fails.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

from . import _lib as L

PRECISION = {"fp32": L.GXC_PRECISION_FP32, "fp16": L.GXC_PRECISION_FP16, "fp8": L.GXC_PRECISION_FP8}
ROTATOR = {"exact": L.GXC_ROTATOR_EXACT, "fxkernel": L.GXC_ROTATOR_FXKERNEL}
XENGINE = {"auto": L.GXC_XENGINE_AUTO, "cuda_core": L.GXC_XENGINE_CUDA_CORE, "tensor": L.GXC_XENGINE_TENSOR}
FFTENGINE = {"auto": L.GXC_FFT_AUTO, "cuda_core": L.GXC_FFT_CUDA_CORE, "tensor": L.GXC_FFT_TENSOR}
XSPLIT = {"auto": L.GXC_XSPLIT_AUTO, "off": L.GXC_XSPLIT_OFF, "on": L.GXC_XSPLIT_ON}
FP8SCALE = {"channel": L.GXC_FP8_SCALE_CHANNEL, "handle": L.GXC_FP8_SCALE_HANDLE}


def make_config(nant, nchan, nfft, nbit=2, lo=8.4e9, bw=64e6, is_complex=False, precision="fp32",
                rotator="exact", autos=True, x_engine="auto", fft_block=0, device=-1,
                fft_engine="auto", x_split="auto", fp8_scaling="channel") -> L.GxcConfig:
    cfg = L.GxcConfig()
    L.lib().gxc_config_init(C.byref(cfg))
    cfg.nant, cfg.nchan, cfg.nfft, cfg.nbit = int(nant), int(nchan), int(nfft), int(nbit)
    cfg.is_complex = int(bool(is_complex))
    cfg.lo_hz, cfg.bw_hz = float(lo), float(bw)
    cfg.precision = PRECISION[precision] if isinstance(precision, str) else int(precision)
    cfg.rotator = ROTATOR[rotator] if isinstance(rotator, str) else int(rotator)
    cfg.autos = int(bool(autos))
    cfg.x_engine = XENGINE[x_engine] if isinstance(x_engine, str) else int(x_engine)
    cfg.fft_block = int(fft_block)
    cfg.device = int(device)
    cfg.fft_engine = FFTENGINE[fft_engine] if isinstance(fft_engine, str) else int(fft_engine)
    cfg.x_split = XSPLIT[x_split] if isinstance(x_split, str) else int(x_split)
    cfg.fp8_scaling = FP8SCALE[fp8_scaling] if isinstance(fp8_scaling, str) else int(fp8_scaling)
    return cfg


def _ptr(x) -> int:
    """Address of a numpy array, torch tensor, or an integer address."""
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    if isinstance(x, np.ndarray):
        return int(x.ctypes.data)
    raise TypeError(f"cannot take the address of {type(x)}")


class FxKernel:
    """GPU FX correlator for one sub-integration at a time (FxKernel drop-in)."""

    def __init__(self, nant: int, nchan: int, nfft: int, nbit: int, lo: float, bw: float, is_complex: bool = False,
                 *, precision: str = "fp32", rotator: str = "exact", autos: bool = True, x_engine: str = "auto",
                 fft_block: int = 0, device: int = -1, fft_engine: str = "auto", x_split: str = "auto",
                 fp8_scaling: str = "channel"):
        self.cfg = make_config(nant, nchan, nfft, nbit, lo, bw, is_complex, precision, rotator, autos, x_engine,
                               fft_block, device, fft_engine, x_split, fp8_scaling)
        st = L.lib().gxc_validate_config(C.byref(self.cfg))
        if st != L.GXC_OK:
            raise ValueError(f"invalid FxKernel configuration ({L.status_name(st)})")
        h = C.c_void_p()
        st = L.lib().gxc_create(C.byref(self.cfg), C.byref(h))
        L.check(st, None, "gxc_create")
        self._h = h
        self.nant, self.nchan, self.nfft = int(nant), int(nchan), int(nfft)
        self.nbaselines = L.lib().gxc_num_baselines(C.byref(self.cfg))
        self.bw = float(bw)
        self._keep = None

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            L.lib().gxc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- reference API
    @property
    def bytes_per_antenna(self) -> int:
        return int(L.lib().gxc_input_bytes_per_antenna(C.byref(self.cfg)))

    def setInputData(self, idata: Sequence):
        """idata[a]: uint8 buffer (numpy array, torch tensor on host or GPU, or address)."""
        if len(idata) != self.nant:
            raise ValueError(f"need {self.nant} input buffers")
        ptrs = (C.c_void_p * self.nant)(*[_ptr(x) for x in idata])
        sizes = []
        for x in idata:
            if hasattr(x, "numel"):
                sizes.append(int(x.numel()) * int(x.element_size()))
            elif isinstance(x, np.ndarray):
                sizes.append(int(x.nbytes))
        nbytes = min(sizes) if sizes else self.bytes_per_antenna
        self._keep = list(idata)  # the engine borrows the buffers
        L.check(L.lib().gxc_set_input(self._h, ptrs, C.c_size_t(nbytes)), self._h, "setInputData")

    def setDelays(self, delays, filestartoffsets):
        poly = np.ascontiguousarray(np.asarray(delays, dtype=np.float64).reshape(self.nant, 3))
        fso = np.ascontiguousarray(np.asarray(filestartoffsets, dtype=np.float64).reshape(self.nant))
        L.check(L.lib().gxc_set_delays(self._h, poly.ctypes.data, fso.ctypes.data), self._h, "setDelays")

    def setFrameValidity(self, valid, samples_per_frame: int = 0):
        """Per-antenna frame flags (device uint8 tensors, e.g. from vdif.depacketize), or None to clear."""
        if valid is None:
            L.check(L.lib().gxc_set_frame_validity(self._h, None, 0, 0), self._h, "setFrameValidity")
            self._fvalid = None
            return
        ptrs = (C.c_void_p * self.nant)(*[_ptr(v) if v is not None else None for v in valid])
        nframes = min(int(v.numel()) for v in valid if v is not None)
        L.check(L.lib().gxc_set_frame_validity(self._h, C.cast(ptrs, C.c_void_p), nframes, int(samples_per_frame)),
                self._h, "setFrameValidity")
        self._fvalid = list(valid)

    def process(self, stream: Optional[int] = None, sync: bool = True):
        """One sub-integration; ``stream`` is a cudaStream_t address (torch: stream.cuda_stream)."""
        L.check(L.lib().gxc_process(self._h, C.c_void_p(stream or 0)), self._h, "process")
        if sync:
            self.sync()

    def sync(self):
        L.check(L.lib().gxc_sync(self._h), self._h, "sync")

    def accumulate(self, odata):
        """odata[nbl][4][nchan] complex64 (numpy or torch, host or GPU) += visibilities."""
        if isinstance(odata, np.ndarray):
            if odata.dtype != np.complex64 or not odata.flags.c_contiguous:
                raise TypeError("odata must be a C-contiguous complex64 array")
            if odata.size < self.nbaselines * 4 * self.nchan:
                raise ValueError("odata too small")
        L.check(L.lib().gxc_accumulate(self._h, C.c_void_p(_ptr(odata))), self._h, "accumulate")

    def visibilities(self, out=None):
        """The visibilities [nbl][4][nchan] complex64: a new numpy array, or copied into ``out``
        (a preallocated C-contiguous complex64 numpy array or torch tensor, host or GPU; pinned
        host memory reads back fastest), which is returned."""
        if out is None:
            out = np.zeros((self.nbaselines, 4, self.nchan), dtype=np.complex64)
        elif isinstance(out, np.ndarray):
            if out.dtype != np.complex64 or not out.flags.c_contiguous or out.size < self.nbaselines * 4 * self.nchan:
                raise ValueError("out must be a C-contiguous complex64 array of nbl*4*nchan values")
        elif hasattr(out, "numel"):
            if out.numel() * out.element_size() < self.nbaselines * 4 * self.nchan * 8 or not out.is_contiguous():
                raise ValueError("out must be a contiguous tensor of nbl*4*nchan complex64 values")
        L.check(L.lib().gxc_get_visibilities(self._h, C.c_void_p(_ptr(out))), self._h, "get_visibilities")
        return out

    def device_visibilities_ptr(self) -> int:
        return int(L.lib().gxc_device_visibilities(self._h) or 0)

    def baseline_counts(self) -> np.ndarray:
        out = np.zeros(self.nbaselines, dtype=np.int32)
        L.check(L.lib().gxc_get_baseline_counts(self._h, C.c_void_p(out.ctypes.data)), self._h, "counts")
        return out

    def valid_flags(self) -> np.ndarray:
        out = np.zeros((self.nant, self.nfft), dtype=np.uint8)
        L.check(L.lib().gxc_get_valid_flags(self._h, C.c_void_p(out.ctypes.data)), self._h, "valid_flags")
        return out

    def saveVisibilities(self, outfile: str):
        """Text dump in the reference format (fxkernel/src/fxkernel.cpp:370-412)."""
        from .visio import save_visibilities
        save_visibilities(outfile, self.visibilities(), self.bw)

    # -- accounting
    @property
    def launches(self) -> int:
        return int(L.lib().gxc_last_launch_count(self._h))

    @property
    def fft_block(self) -> int:
        return int(L.lib().gxc_fft_block(self._h))

    @property
    def fft_engine_used(self) -> str:
        """The F-stage engine this handle runs ("tensor" or "cuda_core"; "auto" resolved)."""
        return "tensor" if L.lib().gxc_fft_engine(self._h) == L.GXC_FFT_TENSOR else "cuda_core"

    @property
    def num_blocks(self) -> int:
        """F/X passes of the last process() (one more than nfft / fft_block when host inputs start
        with a short block)."""
        return int(L.lib().gxc_num_blocks(self._h))

    def enable_stage_timing(self, on: bool = True):
        L.check(L.lib().gxc_enable_stage_timing(self._h, int(on)), self._h, "stage timing")

    def stage_times(self):
        f, x, t = C.c_float(), C.c_float(), C.c_float()
        L.check(L.lib().gxc_stage_times(self._h, C.byref(f), C.byref(x), C.byref(t)), self._h, "stage times")
        return float(f.value), float(x.value), float(t.value)
