"""Autotuner for per-shape launch choices of the correlator.

For one job shape it times process() over candidate FFT blocks (FFTs per F/X
pass) and X-stage engines that the shape supports, and keeps the fastest.
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
    import torch
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    fx.process(stream=stream, sync=False)  # warm
    s = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()
    ev0.record(s)
    for _ in range(reps):
        fx.process(stream=stream, sync=False)
    ev1.record(s)
    ev1.synchronize()
    return ev0.elapsed_time(ev1) / reps


def tune(job: dict, blocks: Iterable[int] = DEFAULT_BLOCKS, engines: Iterable[str] = ("tensor", "cuda_core"),
         reps: int = 2, path: Optional[str] = None, force: bool = False) -> dict:
    """job: FxKernel keyword arguments plus ``inputs`` (device buffers), ``poly``, ``fso``.
    Returns {"fft_block": T, "x_engine": name, "ms": best time, "tried": [...]} (cached)."""
    import torch
    path = path or cache_path()
    prec = job.get("precision", "fp32")
    key = shape_key(job["nant"], job["nchan"], job["nfft"], job.get("nbit", 2), job.get("is_complex", False), prec)
    data = _load(path)
    if not force and key in data:
        return data[key]
    stream = torch.cuda.current_stream().cuda_stream
    tried = []
    best = None
    cands = sorted({min(int(b), int(job["nfft"])) for b in blocks})
    for eng in engines:
        for T in cands:
            kw = {k: job[k] for k in ("nant", "nchan", "nfft", "nbit", "lo", "bw", "is_complex") if k in job}
            try:
                fx = FxKernel(precision=prec, rotator=job.get("rotator", "exact"), autos=job.get("autos", True),
                              x_engine=eng, fft_block=T, **kw)
            except Exception:
                continue  # engine unavailable for this shape
            fx.setInputData(job["inputs"])
            fx.setDelays(job["poly"], job["fso"])
            ms = _time_once(fx, stream, reps)
            fx.close()
            tried.append({"x_engine": eng, "fft_block": T, "ms": ms})
            if best is None or ms < best["ms"]:
                best = {"x_engine": eng, "fft_block": T, "ms": ms}
    if best is None:
        raise RuntimeError(f"no candidate could run shape {key}")
    best = dict(best, tried=tried, when=time.strftime("%Y-%m-%dT%H:%M:%S"))
    data[key] = best
    _store(path, data)
    return best
