"""Harness file formats through the C ABI: .conf files and raw per-antenna voltage files.

read_conf follows parseConfig (fxkernel/src/common.cpp:54-114); RawReader follows
readdata (fxkernel/src/common.cpp:38-52): each read returns the next
bytes_per_antenna bytes of every antenna file, None at the end of any file.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Optional

import numpy as np

from . import _lib as L


def read_conf(path: str) -> dict:
    """Returns {"nant", "nchan", "nfft", "nbit", "npol", "is_complex", "lo", "bw",
    "names", "files", "poly" [nant,3], "fso" [nant]}; antenna file paths are
    returned as written (relative to the working directory, as the reference opens them)."""
    cf = C.c_void_p()
    L.check(L.lib().gxc_conf_read(os.fsencode(path), C.byref(cf)), None, f"reading {path}")
    try:
        g = lambda k: int(L.lib().gxc_conf_int(cf, k.encode()))
        nant = g("NANT")
        poly = np.zeros((nant, 3), np.float64)
        fso = np.zeros(nant, np.float64)
        L.lib().gxc_conf_delays(cf, C.c_void_p(poly.ctypes.data), C.c_void_p(fso.ctypes.data))
        return {"nant": nant, "nchan": g("NCHAN"), "nfft": g("NUMFFTS"), "nbit": g("NBIT"), "npol": g("NPOL"),
                "is_complex": bool(g("COMPLEX")), "lo": float(L.lib().gxc_conf_double(cf, b"LO")),
                "bw": float(L.lib().gxc_conf_double(cf, b"BANDWIDTH")),
                "names": [L.lib().gxc_conf_antenna_name(cf, a).decode() for a in range(nant)],
                "files": [L.lib().gxc_conf_antenna_file(cf, a).decode() for a in range(nant)],
                "poly": poly, "fso": fso}
    finally:
        L.lib().gxc_conf_free(cf)


def write_conf(path: str, nant, nchan, nfft, lo, bw, names, files, poly, fso, nbit=2, is_complex=False, npol=2):
    """Writes a .conf file that read_conf (and the reference's parseConfig) reads back."""
    with open(path, "w") as f:
        f.write(f"NBIT {nbit}\nNPOL {npol}\nCOMPLEX {int(bool(is_complex))}\nNCHAN {nchan}\n")
        f.write(f"LO {float(lo)!r}\nBANDWIDTH {float(bw)!r}\nNUMFFTS {nfft}\nNANT {nant}\n")
        for a in range(nant):
            p = np.asarray(poly[a], dtype=np.float64)
            f.write(f"{names[a]} {files[a]} {float(p[0])!r} {float(p[1])!r} {float(p[2])!r} {float(fso[a])!r}\n")


class RawReader:
    def __init__(self, paths: List[str], bytes_per_antenna: int):
        self.nant = len(paths)
        self.nbytes = int(bytes_per_antenna)
        arr = (C.c_char_p * self.nant)(*[os.fsencode(p) for p in paths])
        self._r = C.c_void_p()
        L.check(L.lib().gxc_reader_open(C.cast(arr, C.c_void_p), self.nant, self.nbytes, C.byref(self._r)), None,
                "gxc_reader_open")

    def read(self, out: Optional[List[np.ndarray]] = None):
        """Fills (or allocates) one buffer per antenna; returns them, or None at the end of data."""
        if out is None:
            out = [np.empty(self.nbytes, np.uint8) for _ in range(self.nant)]
        ptrs = (C.c_void_p * self.nant)(*[int(x.ctypes.data) if isinstance(x, np.ndarray) else int(x.data_ptr())
                                          for x in out])
        st = L.lib().gxc_reader_read(self._r, C.cast(ptrs, C.c_void_p))
        if st == L.GXC_END_OF_DATA:
            return None
        L.check(st, None, "gxc_reader_read")
        return out

    def close(self):
        if getattr(self, "_r", None):
            L.lib().gxc_reader_close(self._r)
            self._r = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def save_visibilities(path: str, vis: np.ndarray, bw_hz: float) -> None:
    """vis.out writer of the library (gxc_save_visibilities)."""
    v = np.ascontiguousarray(np.asarray(vis, dtype=np.complex64))
    nbl, _, nchan = v.shape
    L.check(L.lib().gxc_save_visibilities(os.fsencode(path), C.c_void_p(v.ctypes.data), nbl, nchan, float(bw_hz)),
            None, "gxc_save_visibilities")
