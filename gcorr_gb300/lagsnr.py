"""Lag-domain signal-to-noise of visibilities, as util/lagsnr.py:16-31 computes it:
for each baseline-product, lags = |IFFT over channels of the visibility| and
S/N = max(lags) / std(lags), with the lag bin of the maximum.

Command line: python -m gcorr_gb300.lagsnr vis.out  (prints one line per baseline-product).
"""
from __future__ import annotations

import sys

import numpy as np


def lag_snr(vis: np.ndarray):
    """vis: complex [..., nchan].  Returns (snr [...], argmax lag bin [...])."""
    lags = np.abs(np.fft.ifft(np.asarray(vis, dtype=np.complex128), axis=-1))
    with np.errstate(invalid="ignore", divide="ignore"):  # an all-zero product gives nan, as numpy does
        return lags.max(axis=-1) / lags.std(axis=-1), lags.argmax(axis=-1)


def lag_snr_file(path: str):
    """Reads a vis.out text file (columns: chan, freq, then re im amp phase per baseline-product)."""
    rows = np.loadtxt(path, ndmin=2)
    body = rows[:, 2:]
    if body.shape[1] % 4:
        raise ValueError(f"{path}: {rows.shape[1]} columns is not a vis.out layout")
    v = body.reshape(rows.shape[0], -1, 4)
    vis = (v[..., 0] + 1j * v[..., 1]).T  # [blpol, nchan]
    return lag_snr(vis)


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 1:
        print("Usage: python -m gcorr_gb300.lagsnr <vis.out>")
        return 1
    snr, arg = lag_snr_file(argv[0])
    for i, (s, a) in enumerate(zip(snr, arg)):
        print(f"S/N of blpol {i} is {s:.3f} occurring at channel {a}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
