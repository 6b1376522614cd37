"""Streaming ingest of consecutive sub-integrations (gxc_pipeline_* in include/gxc.h).

Copies of sub-integration k+1 (host -> device, copy stream) overlap the
correlation of sub-integration k (compute stream); optional long-integration
sum and linear->circular polarisation conversion on the device.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _lib as L
from .fxkernel import _ptr, make_config


class Pipeline:
    def __init__(self, nant, nchan, nfft, nbit=2, lo=8.4e9, bw=64e6, is_complex=False, slots: int = 2,
                 integrate: bool = True, **cfg_kw):
        self.cfg = make_config(nant, nchan, nfft, nbit, lo, bw, is_complex, **cfg_kw)
        self.nant, self.nchan = nant, nchan
        self.nbl = L.lib().gxc_num_baselines(C.byref(self.cfg))
        self._p = C.c_void_p()
        L.check(L.lib().gxc_pipeline_create(C.byref(self.cfg), int(slots), int(integrate), C.byref(self._p)), None,
                "gxc_pipeline_create")
        self._keep = {}

    def _check(self, st, what):
        if st != L.GXC_OK:
            m = L.lib().gxc_pipeline_last_error(self._p)
            raise L.GxcError(st, f"{what}: {L.status_name(st)}: {m.decode() if m else ''}")

    def submit(self, inputs: Sequence, poly, fso, out=None) -> int:
        """inputs: per-antenna buffers (pinned torch tensors / numpy arrays / addresses);
        out: optional host or device buffer of nbl*4*nchan complex64. Returns the sequence number."""
        ptrs = (C.c_void_p * self.nant)(*[_ptr(x) for x in inputs])
        poly = np.ascontiguousarray(np.asarray(poly, dtype=np.float64).reshape(self.nant, 3))
        fso = np.ascontiguousarray(np.asarray(fso, dtype=np.float64).reshape(self.nant))
        seq = C.c_int64()
        self._check(L.lib().gxc_pipeline_submit(self._p, C.cast(ptrs, C.c_void_p), C.c_void_p(poly.ctypes.data),
                                                C.c_void_p(fso.ctypes.data),
                                                C.c_void_p(_ptr(out)) if out is not None else None,
                                                C.byref(seq)), "gxc_pipeline_submit")
        # keep the buffers alive until the sub-integration is waited for
        self._keep[seq.value] = (list(inputs), out)
        return seq.value

    def wait(self, seq: int):
        self._check(L.lib().gxc_pipeline_wait(self._p, C.c_int64(seq)), "gxc_pipeline_wait")
        for k in [k for k in self._keep if k <= seq]:
            del self._keep[k]

    def sync(self):
        self._check(L.lib().gxc_pipeline_sync(self._p), "gxc_pipeline_sync")
        self._keep.clear()

    def integration(self, reset: bool = False):
        out = np.zeros((self.nbl, 4, self.nchan), dtype=np.complex64)
        n = C.c_int()
        self._check(L.lib().gxc_pipeline_integration(self._p, C.c_void_p(out.ctypes.data), int(reset), C.byref(n)),
                    "gxc_pipeline_integration")
        self._keep.clear()
        return out, n.value

    def set_lin2circ(self, enable: bool = True, gains: Optional[np.ndarray] = None):
        g = None
        if gains is not None:
            g = np.ascontiguousarray(np.asarray(gains, dtype=np.complex64).reshape(self.nant, 2, self.nchan))
        self._check(L.lib().gxc_pipeline_set_lin2circ(self._p, int(enable),
                                                      C.c_void_p(g.ctypes.data) if g is not None else None),
                    "gxc_pipeline_set_lin2circ")

    @property
    def handle(self):
        return L.lib().gxc_pipeline_handle(self._p)

    def close(self):
        if getattr(self, "_p", None):
            L.lib().gxc_pipeline_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lin2circ(vis_dev, nant: int, nchan: int, autos: bool, gains_dev=None, stream: int = 0):
    """In-place linear->circular conversion of a device visibility buffer [nbl][4][nchan] complex64."""
    st = L.lib().gxc_lin2circ(C.c_void_p(_ptr(vis_dev)), C.c_void_p(_ptr(gains_dev)) if gains_dev is not None else None,
                              int(nant), int(nchan), int(autos), C.c_void_p(stream))
    L.check(st, None, "gxc_lin2circ")
