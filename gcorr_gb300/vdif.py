"""VDIF frames in and out (gxc_vdif_* in include/gxc.h).

``packetize`` writes an engine input buffer as VDIF frames (host, numpy): used to
make test streams and to export data.  ``parse_header`` decodes a header through
the library; ``depacketize`` runs the GPU depacketiser into an engine input
buffer plus per-frame validity for ``FxKernel.setFrameValidity``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .fxkernel import _ptr


def header_words(seconds, frame, frame_bytes, nchan=2, bits=2, is_complex=False, thread=0, station=0, ref_epoch=0,
                 legacy=False, invalid=False, version=0):
    w0 = (int(invalid) << 31) | (int(legacy) << 30) | (int(seconds) & 0x3FFFFFFF)
    w1 = ((int(ref_epoch) & 0x3F) << 24) | (int(frame) & 0xFFFFFF)
    w2 = ((int(version) & 0x7) << 29) | ((int(nchan).bit_length() - 1) << 24) | ((int(frame_bytes) // 8) & 0xFFFFFF)
    w3 = (int(is_complex) << 31) | (((int(bits) - 1) & 0x1F) << 26) | ((int(thread) & 0x3FF) << 16) | (int(station) & 0xFFFF)
    words = [w0, w1, w2, w3] + ([] if legacy else [0, 0, 0, 0])
    return np.array(words, dtype="<u4")


def samples_per_frame(payload_bytes: int, bits: int, nchan: int = 2, is_complex: bool = False) -> int:
    return payload_bytes * 8 // (bits * nchan * (2 if is_complex else 1))


def packetize(data: np.ndarray, payload_bytes: int, frames_per_second: int, seconds0: int = 0, frame0: int = 0,
              bits: int = 2, is_complex: bool = False, thread: int = 0, station: int = 0, legacy: bool = False,
              signed_to_offset_binary: bool = False) -> np.ndarray:
    """data: one antenna's engine input bytes (length a multiple of payload_bytes).
    Returns uint8 [nframes, frame_bytes]: header + payload per frame, frames numbered
    from (seconds0, frame0) at frames_per_second."""
    data = np.ascontiguousarray(np.asarray(data, dtype=np.uint8))
    if data.size % payload_bytes:
        raise ValueError("data length must be a multiple of payload_bytes")
    n = data.size // payload_bytes
    hdr = 16 if legacy else 32
    fb = hdr + payload_bytes
    if fb % 8:
        raise ValueError("VDIF frame length must be a multiple of 8 bytes")
    out = np.empty((n, fb), np.uint8)
    pay = data.reshape(n, payload_bytes)
    out[:, hdr:] = pay ^ np.uint8(0x80) if signed_to_offset_binary else pay
    for k in range(n):
        f = frame0 + k
        out[k, :hdr] = header_words(seconds0 + f // frames_per_second, f % frames_per_second, fb, 2, bits, is_complex,
                                    thread, station, legacy=legacy).view(np.uint8)
    return out


def parse_header(buf) -> dict:
    b = np.ascontiguousarray(np.asarray(buf, dtype=np.uint8)[:32])
    if b.size < 16:
        raise ValueError("a VDIF header has at least 16 bytes")
    if b.size < 32:
        b = np.concatenate([b, np.zeros(32 - b.size, np.uint8)])
    h = L.GxcVdifHeader()
    L.check(L.lib().gxc_vdif_parse_header(C.c_void_p(b.ctypes.data), C.byref(h)), None, "gxc_vdif_parse_header")
    return {name: getattr(h, name) for name, _ in L.GxcVdifHeader._fields_}


def depacketize(frames_dev, frame_bytes: int, payload_bytes: int, seconds0: int, frame0: int, frames_per_second: int,
                nslots: int, thread_id: int = -1, offset_binary_8bit: bool = False, fill: int = 0, stream: int = 0):
    """frames_dev: device uint8 tensor of back-to-back frames.  Returns (out uint8 [nslots*payload],
    valid uint8 [nslots], stats int64 [3]) as device tensors (enqueued on `stream`)."""
    import torch
    dev = frames_dev.device
    out = torch.empty(nslots * payload_bytes, dtype=torch.uint8, device=dev)
    valid = torch.empty(nslots, dtype=torch.uint8, device=dev)
    stats = torch.zeros(3, dtype=torch.int64, device=dev)
    st = L.lib().gxc_vdif_depacketize(C.c_void_p(_ptr(frames_dev)), frames_dev.numel(), int(frame_bytes),
                                      int(payload_bytes), int(seconds0), int(frame0), int(frames_per_second),
                                      int(thread_id), int(offset_binary_8bit), int(fill) & 0xFF,
                                      C.c_void_p(_ptr(out)), int(nslots), C.c_void_p(_ptr(valid)),
                                      C.c_void_p(_ptr(stats)), C.c_void_p(stream))
    L.check(st, None, "gxc_vdif_depacketize")
    return out, valid, stats
