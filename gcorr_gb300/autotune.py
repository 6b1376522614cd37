"""Autotuner for per-shape launch choices of the correlator.

For one job shape it times process() over the launch plans the shape supports:
FFT block (FFTs per F/X pass), X-stage engine, F-stage plan (CUDA-core radix FFT
or tensor-core four-step DFT products) and the X tile's FFT-range split, and
keeps the fastest.
Results are cached on disk (JSON) by shape, so a shape is measured once per
machine.  Cache file: $GXC_TUNE_CACHE or ~/.cache/gxcorr/tune.json.
"""
from __future__ import annotations

import json
import os
import time
from typing import Dict, Iterable, Optional

from .fxkernel import FxKernel

DEFAULT_BLOCKS = (1024, 4096, 16384)


def cache_path() -> str:
    p = os.environ.get("GXC_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "gxcorr", "tune.json")


def shape_key(nant, nchan, nfft, nbit, is_complex, precision) -> str:
    return f"a{nant}_c{nchan}_f{nfft}_b{nbit}_{'cplx' if is_complex else 'real'}_{precision}"


def _load(path: str) -> Dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path: str, data: Dict) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _time_once(fx: FxKernel, stream: int, reps: int) -> float:
    """Median of `reps` process() durations (CUDA events on the launching stream), after a warm run."""
    import torch
    fx.process(stream=stream, sync=False)  # warm
    s = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()
    ts = []
    for _ in range(reps):
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(s)
        fx.process(stream=stream, sync=False)
        ev1.record(s)
        ev1.synchronize()
        ts.append(ev0.elapsed_time(ev1))
    return sorted(ts)[len(ts) // 2]


def _candidates_f(job: dict, prec: str):
    """F-stage plans for the shape: the CUDA-core radix FFT always; the tensor-core four-step FFT
    for 8192-point windows of 2-bit real data with FP16 / FP8 output."""
    F = job["nchan"] if job.get("is_complex", False) else 2 * job["nchan"]
    out = ["cuda_core"]
    if F == 8192 and not job.get("is_complex", False) and prec != "fp32":
        out.append("tensor")
    return out


def tune(job: dict, blocks: Iterable[int] = DEFAULT_BLOCKS, engines: Iterable[str] = ("tensor", "cuda_core"),
         reps: int = 3, path: Optional[str] = None, force: bool = False) -> dict:
    """job: FxKernel keyword arguments plus ``inputs`` (device buffers), ``poly``, ``fso``.

    Coordinate search over the launch plan of one shape:
      1. FFT block T (FFTs per F/X pass) x X engine (tensor cores / CUDA cores);
      2. for the best pair, the F-stage plan (``fft_engine``: CUDA-core radix FFT or tensor-core
         four-step DFT products, where the shape allows both);
      3. for a tensor X-stage on FP16 / FP8 data, the X tile's FFT-range split (``x_split`` off / on:
         one or two CTAs per channel group and block).
    Each candidate is the median of `reps` timed process() calls.  Returns {"fft_block",
    "x_engine", "fft_engine", "x_split", "ms", "tried": [...]} (cached on disk by shape)."""
    import torch
    path = path or cache_path()
    prec = job.get("precision", "fp32")
    key = shape_key(job["nant"], job["nchan"], job["nfft"], job.get("nbit", 2), job.get("is_complex", False), prec)
    data = _load(path)
    if not force and key in data and "fft_engine" in data[key]:
        return data[key]
    stream = torch.cuda.current_stream().cuda_stream
    tried = []
    kw = {k: job[k] for k in ("nant", "nchan", "nfft", "nbit", "lo", "bw", "is_complex") if k in job}

    def run(plan):
        try:
            fx = FxKernel(precision=prec, rotator=job.get("rotator", "exact"), autos=job.get("autos", True), **plan,
                          **kw)
        except Exception:
            return None  # not available for this shape
        try:
            fx.setInputData(job["inputs"])
            fx.setDelays(job["poly"], job["fso"])
            ms = _time_once(fx, stream, reps)
        finally:
            fx.close()
        tried.append(dict(plan, ms=ms))
        return ms

    best, best_ms = None, None

    def consider(plan):
        nonlocal best, best_ms
        ms = run(plan)
        if ms is not None and (best_ms is None or ms < best_ms):
            best, best_ms = dict(plan), ms

    cands = sorted({min(int(b), int(job["nfft"])) for b in blocks})
    for eng in engines:
        for T in cands:
            consider({"x_engine": eng, "fft_block": T, "fft_engine": "cuda_core", "x_split": "auto"})
    if best is None:
        raise RuntimeError(f"no candidate could run shape {key}")
    for fe in _candidates_f(job, prec):
        if fe != best["fft_engine"]:
            consider(dict(best, fft_engine=fe))
    if best["x_engine"] == "tensor" and prec != "fp32":
        for xs in ("off", "on"):
            consider(dict(best, x_split=xs))
    out = dict(best, ms=best_ms, tried=tried, when=time.strftime("%Y-%m-%dT%H:%M:%S"))
    data[key] = out
    _store(path, data)
    return out
