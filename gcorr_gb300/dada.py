"""PSRDADA streams as correlator input (gxc_dada_* in include/gxc.h).

The reference's ingest writes each station's VDIF payloads, headers stripped, into a PSRDADA ring
buffer behind an ASCII header (ingest/src/ingest.c:185-330); a stream saved from such a ring holds
one antenna's samples in the engine's input layout.  ``write_stream`` writes such a stream (used by
the tests and by tools that save ring contents); ``DadaReader`` reads one per antenna, a
sub-integration at a time.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Sequence

import numpy as np

from . import _lib as L


def parse_header(text: bytes) -> L.GxcDadaHeader:
    h = L.GxcDadaHeader()
    L.check(L.lib().gxc_dada_parse_header(text, len(text), C.byref(h)), None, "gxc_dada_parse_header")
    return h


def header_value(text: bytes, key: str) -> str:
    out = C.create_string_buffer(256)
    L.check(L.lib().gxc_dada_header_value(text, len(text), key.encode(), out, 256), None, f"DADA key {key}")
    return out.value.decode()


def make_header(fields: Dict[str, object], hdr_size: int = 4096) -> bytes:
    """An ASCII header of exactly hdr_size bytes ("KEY value" lines, NUL-padded)."""
    lines = ["HEADER DADA", "HDR_VERSION 1.0", f"HDR_SIZE {hdr_size}"]
    lines += [f"{k} {v}" for k, v in fields.items() if k not in ("HDR_SIZE",)]
    text = ("\n".join(lines) + "\n").encode()
    if len(text) > hdr_size:
        raise ValueError("header longer than HDR_SIZE")
    return text + b"\0" * (hdr_size - len(text))


def write_stream(path: str, fields: Dict[str, object], data: np.ndarray, hdr_size: int = 4096) -> None:
    with open(path, "wb") as f:
        f.write(make_header(fields, hdr_size))
        f.write(np.ascontiguousarray(data, dtype=np.uint8).tobytes())


class DadaReader:
    """One DADA stream per antenna; read() fills one buffer per antenna with the next
    bytes_per_read bytes (numpy arrays or host tensors) and returns False at the end of data."""

    def __init__(self, paths: Sequence[str], bytes_per_read: int, offset_binary_8bit: bool = False):
        arr = (C.c_char_p * len(paths))(*[p.encode() for p in paths])
        h = C.c_void_p()
        L.check(L.lib().gxc_dada_open(C.cast(arr, C.c_void_p), len(paths), bytes_per_read, int(offset_binary_8bit),
                                      C.byref(h)), None, "gxc_dada_open")
        self._r, self.nant, self.bytes_per_read = h, len(paths), int(bytes_per_read)

    def header(self, a: int = 0) -> L.GxcDadaHeader:
        h = L.GxcDadaHeader()
        L.check(L.lib().gxc_dada_header_of(self._r, a, C.byref(h)), None, "gxc_dada_header_of")
        return h

    def config(self, **kw):
        """A correlator configuration from antenna 0's header (nbit, complex, bw, lo) plus kw."""
        from .fxkernel import make_config
        cfg = make_config(**kw)
        L.check(L.lib().gxc_dada_config(C.byref(self.header(0)), C.byref(cfg)), None, "gxc_dada_config")
        return cfg

    def read(self, bufs) -> bool:
        ptrs = (C.c_void_p * self.nant)(*[int(b.data_ptr()) if hasattr(b, "data_ptr") else int(b.ctypes.data)
                                          for b in bufs])
        st = L.lib().gxc_dada_read(self._r, C.cast(ptrs, C.c_void_p))
        if st == L.GXC_END_OF_DATA:
            return False
        L.check(st, None, "gxc_dada_read")
        return True

    def close(self):
        if getattr(self, "_r", None):
            L.lib().gxc_dada_close(self._r)
            self._r = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
