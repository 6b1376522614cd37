"""Batches of uneven correlation jobs launched as one CUDA graph (gxc_batch_* in include/gxc.h)."""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence

import numpy as np

from . import _lib as L
from .fxkernel import _ptr, make_config


class Batch:
    """jobs: sequence of dicts with keys ``inputs`` (device tensors / addresses, one per
    antenna), ``poly`` [nant,3], ``fso`` [nant] and the FxKernel configuration keys
    (nant, nchan, nfft, nbit, lo, bw, is_complex, precision, rotator, autos,
    x_engine, fft_block, fft_engine, x_split, fp8_scaling)."""

    CFG_KEYS = ("nant", "nchan", "nfft", "nbit", "lo", "bw", "is_complex", "precision", "rotator", "autos",
                "x_engine", "fft_block", "fft_engine", "x_split", "fp8_scaling")

    def __init__(self, jobs: Sequence[dict]):
        self._keep = []
        arr = (L.GxcJob * len(jobs))()
        self.shapes = []
        for i, j in enumerate(jobs):
            kw = {k: j[k] for k in self.CFG_KEYS if k in j}
            cfg = make_config(**kw)
            nant = cfg.nant
            ptrs = (C.c_void_p * nant)(*[_ptr(x) for x in j["inputs"]])
            poly = np.ascontiguousarray(np.asarray(j["poly"], dtype=np.float64).reshape(nant, 3))
            fso = np.ascontiguousarray(np.asarray(j["fso"], dtype=np.float64).reshape(nant))
            self._keep += [ptrs, poly, fso, list(j["inputs"])]
            arr[i].cfg = cfg
            arr[i].inputs = C.cast(ptrs, C.c_void_p)
            arr[i].poly = poly.ctypes.data
            arr[i].fso = fso.ctypes.data
            nbl = L.lib().gxc_num_baselines(C.byref(cfg))
            self.shapes.append((nbl, cfg.nchan))
        h = C.c_void_p()
        st = L.lib().gxc_batch_create(arr, len(jobs), C.byref(h))
        L.check(st, None, "gxc_batch_create")
        self._b = h
        self.njobs = len(jobs)

    def launch(self, stream=None):
        L.check(L.lib().gxc_batch_launch(self._b, C.c_void_p(stream or 0)), None, "gxc_batch_launch")

    @property
    def launches(self) -> int:
        return int(L.lib().gxc_batch_launch_count(self._b))

    def handle(self, i: int):
        return L.lib().gxc_batch_job(self._b, int(i))

    def visibilities(self, i: int) -> np.ndarray:
        nbl, nchan = self.shapes[i]
        out = np.zeros((nbl, 4, nchan), dtype=np.complex64)
        h = self.handle(i)
        L.check(L.lib().gxc_get_visibilities(h, C.c_void_p(out.ctypes.data)), h, "batch visibilities")
        return out

    def baseline_counts(self, i: int) -> np.ndarray:
        nbl, _ = self.shapes[i]
        out = np.zeros(nbl, dtype=np.int32)
        h = self.handle(i)
        L.check(L.lib().gxc_get_baseline_counts(h, C.c_void_p(out.ctypes.data)), h, "batch counts")
        return out

    def close(self):
        if getattr(self, "_b", None):
            L.lib().gxc_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
