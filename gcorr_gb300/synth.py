"""Seeded synthetic voltage generator for the FX correlator workloads.

Produces packed dual-pol station streams in the exact input format of
``FxKernel::setInputData`` (fxkernel/src/fxkernel.h:40): one buffer per antenna
of ``(nfft+1)`` FFT windows.

* 2-bit real: 4 samples per byte, ``A_t | B_t<<2 | A_t+1<<4 | B_t+1<<6``
  (fxkernel/src/fxkernel.cpp:15-28, generators/bitconversion.c:147-157),
  quantiser thresholds at +-0.98 sigma onto codes {0:-3.3359, 1:-1, 2:+1, 3:+3.3359}.
* 8-bit complex: int8 ``A.re, A.im, B.re, B.im`` per time sample, Gaussian
  sigma=20 per component, rounded and clipped to +-127.

Signal model: each pol carries a common analytic sky signal ``z`` (band
[0, bw) at baseband) seen by antenna j delayed by its quadratic delay model
tau_j(t) (seconds, t in FFT intervals, fxkernel/src/common.h:38), with the LO
phase exp(+2 pi i LO tau_j) applied per sample, mixed with independent
receiver noise at correlation coefficient rho.  Station sample m carries the
wavefront that reaches the array reference at time ``m*Ts + tau_j - fso_j``,
the convention implied by ``offset = i*F - nd`` (fxkernel/src/fxkernel.cpp:289-293).
The fractional part of the delay is applied per FFT-length block in the
frequency domain (overlap-save over a 2F window).

The generator runs on any torch device; the benchmark uses the GPU for the
full-size workloads, the tests use the CPU for small ones.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np
import torch

HIMAG = 3.3359
THRESH_2BIT = 0.98


@dataclasses.dataclass
class Workload:
    nant: int
    nchan: int
    nfft: int
    nbit: int = 2
    is_complex: bool = False
    lo_hz: float = 8.4e9
    bw_hz: float = 64e6
    rho: float = 0.05
    seed: int = 1234
    offset_us: float = 20.0      # uniform +- range of the delay offset
    rate_us_per_s: float = 3.0   # uniform +- range of the delay rate
    accel_us_per_s2: float = 1e-3
    tone_amp: float = 0.0        # narrowband common tone, in units of sigma
    tone_chan: Optional[int] = None
    sigma8: float = 20.0

    @property
    def fft_len(self) -> int:
        return self.nchan if self.is_complex else 2 * self.nchan

    @property
    def sample_time(self) -> float:
        return (1.0 / self.bw_hz) if self.is_complex else 1.0 / (2.0 * self.bw_hz)

    @property
    def fft_time(self) -> float:
        return self.fft_len * self.sample_time

    @property
    def bytes_per_antenna(self) -> int:
        comps = 2 if self.is_complex else 1
        return (self.nfft + 1) * self.fft_len * 2 * comps * self.nbit // 8

    @property
    def input_samples(self) -> int:
        """Input samples of one sub-integration: nant x 2 pols x nfft x F."""
        return self.nant * 2 * self.nfft * self.fft_len


def delay_model(w: Workload):
    """Per-antenna quadratic delay polynomials and file-start offsets.

    Returns ``poly`` [nant, 3] (coefficients of t^2, t, 1; seconds, t in FFT
    intervals) and ``fso`` [nant] (seconds, zero).  Units follow
    util/difx2conf.py:103-106: p2 = offset, p1 = rate*T_F, p0 = accel*T_F^2.
    """
    rng = np.random.default_rng(w.seed)
    tf = w.fft_time
    off = rng.uniform(-1, 1, w.nant) * w.offset_us * 1e-6
    rate = rng.uniform(-1, 1, w.nant) * w.rate_us_per_s * 1e-6
    acc = rng.uniform(-1, 1, w.nant) * w.accel_us_per_s2 * 1e-6
    poly = np.stack([acc * tf * tf, rate * tf, off], axis=1).astype(np.float64)
    fso = np.zeros(w.nant, dtype=np.float64)
    return poly, fso


def _poly_eval(poly_row, u):
    p0, p1, p2 = (float(v) for v in poly_row)
    return (p0 * u + p1) * u + p2


def _station_delay(w: Workload, poly_row, fso: float, m):
    """Delay (s) seen by station sample index m (float64 tensor).

    The polynomial's argument is array-reference time in FFT intervals, and
    station sample m arrives at reference time m*Ts + tau - fso, so tau solves
    tau = poly((m + (tau - fso)/Ts)/F); two fixed-point steps converge (|dtau/dt| << 1).
    """
    F, Ts = w.fft_len, w.sample_time
    tau = _poly_eval(poly_row, m / F)
    for _ in range(2):
        tau = _poly_eval(poly_row, (m + (tau - fso) / Ts) / F)
    return tau


def _common_signal(w: Workload, length: int, gen: torch.Generator, device) -> torch.Tensor:
    """Complex white noise on the reference grid (E|z|^2 = 2 for real data so
    that the half band kept later has unit power; 1 for complex data)."""
    scale = 1.0 if not w.is_complex else math.sqrt(0.5)
    re = torch.randn(length, generator=gen, device=device, dtype=torch.float32)
    im = torch.randn(length, generator=gen, device=device, dtype=torch.float32)
    return torch.complex(re, im) * scale


def _delayed_blocks(w: Workload, z0: torch.Tensor, margin: int, poly_row, fso: float,
                    blk0: int, blk1: int, device) -> torch.Tensor:
    """Common signal as seen by one antenna for FFT blocks [blk0, blk1): returns
    complex64 [nblk*F] (baseband analytic, LO phase applied)."""
    F = w.fft_len
    Ts = w.sample_time
    nb = blk1 - blk0
    m_c = (torch.arange(blk0, blk1, device=device, dtype=torch.float64) + 0.5) * F
    tau_c = _station_delay(w, poly_row, fso, m_c)
    shift = (tau_c - fso) / Ts                      # samples, per block
    k = torch.floor(shift)
    d = (shift - k).to(torch.float32)
    start = (torch.arange(blk0, blk1, device=device, dtype=torch.int64) * F
             + k.to(torch.int64) + margin - F // 2)
    idx = start[:, None] + torch.arange(2 * F, device=device, dtype=torch.int64)[None, :]
    seg = z0[idx]                                   # [nb, 2F]
    spec = torch.fft.fft(seg, dim=1)
    f = torch.fft.fftfreq(2 * F, device=device).to(torch.float32)  # cycles/sample, signed
    ph = torch.exp(2j * math.pi * (f[None, :] * d[:, None]).to(torch.float32))
    spec = spec * ph
    if not w.is_complex:                            # band-limit z0 to |f| < bw/2
        spec = spec * (f.abs() < 0.25)[None, :].to(spec.dtype)
    out = torch.fft.ifft(spec, dim=1)[:, F // 2: F // 2 + F]    # [nb, F]
    # per-sample absolute time of the wavefront and LO phase (FP64, reduced mod 1 turn)
    m = (torch.arange(blk0 * F, blk1 * F, device=device, dtype=torch.float64)).view(nb, F)
    tau = _station_delay(w, poly_row, fso, m)
    lo_turns = torch.remainder(w.lo_hz * tau, 1.0)
    # shift z0 (band [-bw/2,bw/2)) up to [0,bw): exp(i pi bw t_ref), t_ref = (m + shift) Ts
    bb_turns = torch.remainder(0.5 * w.bw_hz * Ts * (m + shift[:, None]), 1.0)
    rot = torch.exp(2j * math.pi * (lo_turns + bb_turns)).to(torch.complex64)
    return (out * rot).reshape(-1)


def _tone(w: Workload, nblk_total: int, poly_row, fso, blk0, blk1, device, phase0: float):
    F = w.fft_len
    Ts = w.sample_time
    chan = w.tone_chan if w.tone_chan is not None else w.nchan // 3
    f_bb = (chan + 0.5) * w.bw_hz / w.nchan
    m = torch.arange(blk0 * F, blk1 * F, device=device, dtype=torch.float64)
    tau = _station_delay(w, poly_row, fso, m)
    t_ref = m * Ts + tau - fso
    turns = torch.remainder(f_bb * t_ref + w.lo_hz * tau + phase0, 1.0)
    return torch.exp(2j * math.pi * turns).to(torch.complex64)


def _pack_2bit(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """a, b: float32 real streams (unit sigma) -> uint8 packed (len/2 bytes)."""
    def codes(x):
        c = torch.full_like(x, 1, dtype=torch.uint8)
        c = torch.where(x >= 0, torch.full_like(c, 2), c)
        c = torch.where(x >= THRESH_2BIT, torch.full_like(c, 3), c)
        c = torch.where(x < -THRESH_2BIT, torch.full_like(c, 0), c)
        return c
    ca = codes(a).view(-1, 2).to(torch.int32)
    cb = codes(b).view(-1, 2).to(torch.int32)
    byte = ca[:, 0] | (cb[:, 0] << 2) | (ca[:, 1] << 4) | (cb[:, 1] << 6)
    return byte.to(torch.uint8)


def _pack_8bit(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """a, b: complex streams scaled to the target sigma -> int8 (re,im,re,im) bytes."""
    st = torch.stack([a.real, a.imag, b.real, b.imag], dim=1)
    q = torch.clamp(torch.round(st), -127, 127).to(torch.int8)
    return q.reshape(-1).view(torch.uint8)


def generate(w: Workload, device="cpu", block_chunk: int = 4096) -> dict:
    """Generate one sub-integration.

    Returns dict with ``inputs`` (list of uint8 tensors, one per antenna, on
    ``device``), ``poly`` [nant,3] float64 numpy, ``fso`` [nant] numpy.
    """
    device = torch.device(device)
    F = w.fft_len
    Ts = w.sample_time
    nblk = w.nfft + 1
    poly, fso = delay_model(w)
    # margin covers the largest delay shift plus the overlap-save half window
    u_end = float(nblk)
    maxshift = 0.0
    for j in range(w.nant):
        for u in (0.0, u_end * 0.5, u_end):
            maxshift = max(maxshift, abs(_poly_eval(poly[j], u) - fso[j]) / Ts)
    margin = int(maxshift) + F + 16
    length = nblk * F + 2 * margin
    gen = torch.Generator(device=device)
    gen.manual_seed(int(w.seed))
    z = [_common_signal(w, length, gen, device) for _ in range(2)]
    tone_phase = [0.123, 0.456]
    sr, sn = math.sqrt(w.rho), math.sqrt(1.0 - w.rho)
    inputs: List[torch.Tensor] = []
    for j in range(w.nant):
        parts = []
        for b0 in range(0, nblk, block_chunk):
            b1 = min(nblk, b0 + block_chunk)
            pols = []
            for p in range(2):
                sig = _delayed_blocks(w, z[p], margin, poly[j], float(fso[j]), b0, b1, device)
                n = (b1 - b0) * F
                if w.is_complex:
                    nre = torch.randn(n, generator=gen, device=device)
                    nim = torch.randn(n, generator=gen, device=device)
                    noise = torch.complex(nre, nim) * math.sqrt(0.5)
                    x = sr * sig + sn * noise
                    if w.tone_amp > 0:  # tone amplitude in units of the per-component sigma
                        x = x + (w.tone_amp / math.sqrt(2.0)) * _tone(w, nblk, poly[j], float(fso[j]),
                                                                     b0, b1, device, tone_phase[p])
                    x = x * (w.sigma8 * math.sqrt(2.0))
                else:
                    noise = torch.randn(n, generator=gen, device=device)
                    x = sr * math.sqrt(2.0) * sig.real + sn * noise
                    if w.tone_amp > 0:  # real tone of amplitude tone_amp * sigma
                        x = x + w.tone_amp * _tone(w, nblk, poly[j], float(fso[j]), b0, b1, device,
                                                   tone_phase[p]).real
                pols.append(x)
            if w.is_complex:
                parts.append(_pack_8bit(pols[0], pols[1]))
            else:
                parts.append(_pack_2bit(pols[0], pols[1]))
        buf = torch.cat(parts)
        assert buf.numel() == w.bytes_per_antenna, (buf.numel(), w.bytes_per_antenna)
        inputs.append(buf)
    return {"inputs": inputs, "poly": poly, "fso": fso}


def random_bytes(w: Workload, device="cpu") -> dict:
    """Uniform random input bytes (every 2-bit code / int8 value), with the same
    delay model: the cheapest input for parity tests that need no physics."""
    gen = torch.Generator(device="cpu")
    gen.manual_seed(int(w.seed))
    poly, fso = delay_model(w)
    inputs = [torch.randint(0, 256, (w.bytes_per_antenna,), generator=gen, dtype=torch.uint8).to(device)
              for _ in range(w.nant)]
    return {"inputs": inputs, "poly": poly, "fso": fso}


# The five workloads of the benchmark suite (sizes, rates and distributions).
def config0() -> Workload:
    """6 antennas, 2-bit real, 128 Ms/s per pol (64 MHz), 0.25 s, nchan 1024."""
    return Workload(nant=6, nchan=1024, nfft=15625, nbit=2, is_complex=False,
                    lo_hz=8.4e9, bw_hz=64e6, rho=0.05)


def config1() -> Workload:
    """16 antennas, 2-bit real, 512 Ms/s per pol (256 MHz), 1.0 s, nchan 4096."""
    return Workload(nant=16, nchan=4096, nfft=62500, nbit=2, is_complex=False,
                    lo_hz=8.4e9, bw_hz=256e6, rho=0.05)


def config2() -> Workload:
    """32 antennas, 2-bit real, 1024 Ms/s per pol, 0.5 s, nchan 8192, rho 0.01, tone 0.3 sigma."""
    return Workload(nant=32, nchan=8192, nfft=31250, nbit=2, is_complex=False,
                    lo_hz=8.4e9, bw_hz=512e6, rho=0.01, tone_amp=0.3, tone_chan=None)


def config4() -> Workload:
    """64 antennas, 8-bit complex, 256 Ms/s per pol, 0.5 s, nchan 32768, rho 0.02."""
    return Workload(nant=64, nchan=32768, nfft=3906, nbit=8, is_complex=True,
                    lo_hz=8.4e9, bw_hz=256e6, rho=0.02)


def config3_jobs(seed: int = 3) -> List[Workload]:
    """8 uneven jobs: nant in {4,6,10,16,24}, nchan in {256,1024,4096,16384},
    2-bit real or 8-bit complex, 64-512 Ms/s, 0.1-0.5 s, each with its own delays."""
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(8):
        nant = int(rng.choice([4, 6, 10, 16, 24]))
        nchan = int(rng.choice([256, 1024, 4096, 16384]))
        cplx = bool(rng.integers(0, 2))
        rate = float(rng.choice([64e6, 128e6, 256e6, 512e6]))
        tsub = float(rng.uniform(0.1, 0.5))
        F = nchan if cplx else 2 * nchan
        nfft = max(1, int(rate * tsub / F))
        bw = rate if cplx else rate / 2.0
        jobs.append(Workload(nant=nant, nchan=nchan, nfft=nfft, nbit=8 if cplx else 2, is_complex=cplx,
                             lo_hz=8.4e9, bw_hz=bw, rho=0.05, seed=seed * 100 + k))
    return jobs
