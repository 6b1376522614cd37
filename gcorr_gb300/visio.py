"""Visibility text I/O in the reference's ``vis.out`` format.

Writer restates FxKernel::saveVisibilities (fxkernel/src/fxkernel.cpp:370-412):
one line per channel: ``chan`` (width 5), the channel-centre frequency in MHz
``(c+0.5)/nchan*bw/1e6`` (width 11, 6 decimals), then for every baseline and
product ``re im amp phase`` (widths 11, 11, 11, 10; 5 decimals).
"""
from __future__ import annotations

import numpy as np


def save_visibilities(path: str, vis: np.ndarray, bw_hz: float) -> None:
    vis = np.asarray(vis, dtype=np.complex64)
    nbl, nprod, nchan = vis.shape
    amp = np.abs(vis).astype(np.float32)
    ph = np.angle(vis).astype(np.float32)
    with open(path, "w") as f:
        for c in range(nchan):
            parts = [f"{c:5d} {(c + 0.5) / nchan * bw_hz / 1e6:11.6f}"]
            for b in range(nbl):
                for p in range(nprod):
                    v = vis[b, p, c]
                    parts.append(f" {v.real:11.5f} {v.imag:11.5f} {amp[b, p, c]:11.5f} {ph[b, p, c]:10.5f}")
            f.write("".join(parts) + "\n")


def load_visibilities(path: str, nbl: int, nprod: int = 4):
    """Reads a vis.out file back: returns (freq_mhz [nchan], vis complex64 [nbl, nprod, nchan])."""
    rows = np.loadtxt(path, ndmin=2)
    nchan = rows.shape[0]
    freq = rows[:, 1]
    body = rows[:, 2:].reshape(nchan, nbl, nprod, 4)
    vis = (body[..., 0] + 1j * body[..., 1]).astype(np.complex64).transpose(1, 2, 0)
    return freq, vis
