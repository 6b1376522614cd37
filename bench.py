"""Benchmark of the FX correlator hot path (FxKernel::process) on GB300.

Workload (default): 16 antennas x 2 pols, 2-bit real at 512 Msamples/s per pol
(256 MHz), 1.0 s sub-integration, nchan 4096 (8192-point FFTs, 62500 FFTs),
FP32 end to end, 136 baselines (autos included) x 4 products.
Metric: input Gsamples/s = nant * 2 pols * nfft * F / seconds per sub-integration.

value: device-resident inputs, one process() per step, CUDA events on the
launching stream.  e2e: the same sub-integration through the C ABI's streaming
pipeline (gxc_pipeline_submit) from pinned HOST input buffers, the host->device
copy of every step's input and the device->host read of its visibilities inside
the timed region (wall clock); e2e.fxkernel_process: the drop-in path, one
gxc_process on pinned host buffers plus the read-back per step; e2e.h2d_probe_gbs:
the machine's pinned copy bandwidth, measured beside it.  Multi-GPU (torchrun):
independent replicas, one sub-integration per rank per step, no collective on
the data path.

--impl reference times the CPU implementation of the path on all host threads on
a bounded sample of the same workload: the reference's own fxkernel.cpp (compiled
unmodified by oracle/Makefile, one FxKernel per thread) for the jobs it can run,
the FP32 port of it (oracle/fxoracle.c) for the others.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "c0": ("6 antennas, 2-bit real, 128 Ms/s per pol, 0.25 s, nchan 1024", "config0"),
    "c1": ("16 antennas, 2-bit real, 512 Ms/s per pol, 1.0 s, nchan 4096", "config1"),
    "c2": ("32 antennas, 2-bit real, 1024 Ms/s per pol, 0.5 s, nchan 8192, rho 0.01, tone", "config2"),
    "c3": ("8 uneven jobs (nant 4-24, nchan 256-16384, 2-bit real / 8-bit complex, 64-512 Ms/s, 0.1-0.5 s) "
           "in one graph launch", "config3_jobs"),
    "c4": ("64 antennas, 8-bit complex, 256 Ms/s per pol, 0.5 s, nchan 32768, rho 0.02", "config4"),
}


# the X engines every bench run compares (untimed side runs)
XENGINES = (("fp32_cuda_core", "fp32", "cuda_core"), ("fp32_tensor_split", "fp32", "tensor"),
            ("fp16_tensor", "fp16", "tensor"), ("fp8_tensor", "fp8", "tensor"))


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world, backend):
    import torch.distributed as dist
    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend)
    return dist


def reduce_max(x: float, world: int, device=None) -> float:
    """Max over ranks (timing rule: the slowest replica sets the job time)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, path: str):
        self.path = path
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        load = [s for s in sm if mx and s > 0.3 * max(mx)] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def workload(name):
    from gcorr_gb300 import synth
    return getattr(synth, CONFIGS[name][1])()


# ---------------------------------------------------------------- CPU side
def cpu_port_run(w, nfft_sample: int, nthreads: int, seed_inputs=None):
    """Times the FP32 port of fxkernel (oracle) on nfft_sample FFTs of workload w."""
    import dataclasses
    import numpy as np
    from gcorr_gb300 import synth
    from oracle import oracle as O
    ws = dataclasses.replace(w, nfft=nfft_sample)
    if seed_inputs is None:
        d = synth.random_bytes(ws)
        seed_inputs = ([x.numpy() for x in d["inputs"]], d["poly"], d["fso"])
    inputs, poly, fso = seed_inputs
    cfg = O.config_from_workload(ws, O.ROT_FXKERNEL if int(round(w.nchan ** 0.5)) ** 2 == w.nchan else O.ROT_EXACT,
                                 True)
    t0 = time.perf_counter()
    O.port_process(cfg, inputs, poly, fso, nthreads=nthreads)
    dt = time.perf_counter() - t0
    samples = ws.nant * 2 * ws.nfft * ws.fft_len
    return samples / dt, dt, seed_inputs


def cpu_model() -> str:
    """The host CPU as the OS reports it (model name, or the Arm implementer/part codes)."""
    try:
        txt = open("/proc/cpuinfo").read()
    except OSError:
        return "unknown"
    import re
    m = re.search(r"^model name\s*:\s*(.+)$", txt, re.M)
    if m:
        return m.group(1).strip()
    impl = re.search(r"^CPU implementer\s*:\s*(\S+)", txt, re.M)
    part = re.search(r"^CPU part\s*:\s*(\S+)", txt, re.M)
    arm = {("0x41", "0xd4f"): "Arm Neoverse-V2", ("0x41", "0xd40"): "Arm Neoverse-V1", ("0x41", "0xd0c"): "Arm Neoverse-N1"}
    if impl and part:
        key = (impl.group(1).lower(), part.group(1).lower())
        return arm.get(key, f"Arm implementer {key[0]} part {key[1]}")
    return "unknown"


def ref_runnable(w) -> bool:
    """The reference's own process() runs 2-bit real data with a square nchan only
    (fxkernel/src/fxkernel.cpp:46-63, :489-496)."""
    from oracle import oracle as O
    return O.ref_bench_available() and not w.is_complex and w.nbit == 2 and int(round(w.nchan ** 0.5)) ** 2 == w.nchan


def cpu_ref_run(w, nfft_sample: int, nthreads: int, seed_inputs=None):
    """Times the reference's own process() (float-FFT shim build, one FxKernel per thread over
    contiguous FFT slices) on nfft_sample FFTs of workload w."""
    import dataclasses
    from gcorr_gb300 import synth
    from oracle import oracle as O
    ws = dataclasses.replace(w, nfft=nfft_sample)
    if seed_inputs is None:
        d = synth.random_bytes(ws)
        seed_inputs = ([x.numpy() for x in d["inputs"]], d["poly"], d["fso"])
    inputs, poly, fso = seed_inputs
    dt = O.ref_bench(ws.nant, ws.nchan, ws.lo_hz, ws.bw_hz, inputs, poly, fso, 0, ws.nfft, nthreads)
    samples = ws.nant * 2 * ws.nfft * ws.fft_len
    return samples / dt, dt, seed_inputs


def _sized_run(run, w, budget_s: float, nthreads: int):
    n = 4 * nthreads
    _, dt, _ = run(w, n, nthreads)
    n2 = int(max(n, min(w.nfft, budget_s / max(dt / n, 1e-6))))
    n2 -= n2 % nthreads if n2 > nthreads else 0
    rate, dt, _ = run(w, n2, nthreads)
    return rate, dt, n2


def cpu_sample(w, budget_s: float = 12.0):
    """The CPU baseline on a bounded FFT sample of the workload (about budget_s of CPU work on all
    host threads): the reference's own fxkernel.cpp where it can run the workload and its sources
    were staged (kind "reference"), else the FP32 port of it (kind "port"); with the reference,
    the port is timed beside it on the same sample size."""
    nthreads = os.cpu_count() or 1
    host = {"cores": nthreads, "nproc": nthreads, "cpu_model": cpu_model()}
    if ref_runnable(w):
        rate, dt, n2 = _sized_run(cpu_ref_run, w, budget_s, nthreads)
        prate, pdt, _ = cpu_port_run(w, n2, nthreads)
        return {"value": rate / 1e9, "unit": "input Gsamples/s", "kind": "reference", **host,
                "sample": f"{n2} of {w.nfft} FFTs of the same workload (random 2-bit bytes): the reference's "
                          f"fxkernel.cpp, unmodified, one FxKernel per thread over contiguous FFT slices, IPP "
                          f"unavailable (float-FFT shim), {nthreads} threads, {dt:.1f} s",
                "seconds": dt, "port": {"value": prate / 1e9, "seconds": pdt, "kind": "port"}}
    rate, dt, n2 = _sized_run(cpu_port_run, w, budget_s, nthreads)
    return {"value": rate / 1e9, "unit": "input Gsamples/s", "kind": "port", **host,
            "sample": f"{n2} of {w.nfft} FFTs of the same workload (random bytes, FP32 port of fxkernel, "
                      f"{nthreads} threads), {dt:.1f} s", "seconds": dt}


def port_plan(ws, budget_s: float, nthreads: int):
    """Bounded sample of a list of jobs: the same fraction of every job's FFTs, sized so that one
    pass over all of them takes about budget_s on nthreads threads.  Each job runs on the
    reference's own code where it can (ref_runnable), else on the FP32 port."""
    cal = []
    for w in ws:
        run = cpu_ref_run if ref_runnable(w) else cpu_port_run
        n0 = max(1, min(w.nfft, nthreads))
        _, dt, _ = run(w, n0, nthreads)
        cal.append((w, run, dt / n0))
    full = sum(per * w.nfft for w, _, per in cal)
    frac = min(1.0, budget_s / max(full, 1e-9))
    plan = []
    for w, run, per in cal:
        n = int(max(min(w.nfft, nthreads), min(w.nfft, round(frac * w.nfft))))
        n -= n % nthreads if n > nthreads else 0
        _, _, seed = run(w, n, nthreads)
        plan.append((w, n, seed, run))
    return plan


def plan_kind(plan) -> str:
    kinds = {"reference" if run is cpu_ref_run else "port" for _, _, _, run in plan}
    return kinds.pop() if len(kinds) == 1 else "reference+port"


def run_plan(plan, nthreads):
    t = 0.0
    samples = 0
    for w, n, seed, run in plan:
        _, dt, _ = run(w, n, nthreads, seed)
        t += dt
        samples += w.nant * 2 * n * w.fft_len
    return samples, t


def run_reference_arm(args):
    rank, world, local = dist_env()
    if world > 1:
        init_dist(world, "gloo")
        if rank != 0:
            barrier(world)
            return
    w = workload(args.config)
    ws = w if isinstance(w, list) else [w]
    nthreads = os.cpu_count() or 1
    # one step = the port over a bounded FFT sample of every job (about args.ref_step_s of CPU time)
    plan = port_plan(ws, args.ref_step_s, nthreads)
    for _ in range(args.warmup):
        run_plan(plan, nthreads)
    tot = 0.0
    samples = 0
    for _ in range(args.steps):
        s_, t_ = run_plan(plan, nthreads)
        tot += t_
        samples += s_
    val = samples / tot / 1e9
    kind = plan_kind(plan)
    sample = "; ".join(f"{n} of {j.nfft} FFTs ({'reference' if run is cpu_ref_run else 'port'})"
                       for j, n, _, run in plan)
    line = {"impl": "reference", "metric": "input Gsamples/s", "value": val, "unit": "input Gsamples/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": CONFIGS[args.config][0], "sample_ffts_per_step": [n for _, n, _, _ in plan],
                       "nfft": [j.nfft for j in ws], "parallelism": "host threads"},
            "cpu_baseline": {"value": val, "unit": "input Gsamples/s", "cores": nthreads, "nproc": nthreads,
                             "cpu_model": cpu_model(), "kind": kind,
                             "sample": f"{sample} per step; reference = fxkernel.cpp unmodified, one FxKernel per "
                                       f"thread over contiguous FFT slices (float-FFT shim, IPP unavailable); "
                                       f"port = FP32 restatement of it (oracle/fxoracle.c); {nthreads} threads"},
            "e2e": {"value": val, "unit": "input Gsamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    if world > 1:
        barrier(world)


def run_batch_bench(args):
    """Config 3: eight uneven jobs, autotuned per shape, as one graph launch per step."""
    import numpy as np
    import torch
    from gcorr_gb300 import synth
    from gcorr_gb300.autotune import tune
    from gcorr_gb300.batch import Batch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    init_dist(world, "nccl")
    dev = torch.device("cuda", local)
    ws = synth.config3_jobs(seed=3 + 1000 * rank)
    tg = time.perf_counter()
    data = [synth.generate(w, device=dev) for w in ws]
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - tg
    base = []
    for w, d in zip(ws, data):
        base.append(dict(nant=w.nant, nchan=w.nchan, nfft=w.nfft, nbit=w.nbit, lo=w.lo_hz, bw=w.bw_hz,
                         is_complex=w.is_complex, inputs=d["inputs"], poly=d["poly"], fso=d["fso"], autos=True))
    prec = args.precision if args.precision != "fp32" else "fp16"
    tuned = [tune(dict(b, precision=prec)) for b in base]
    jobs16 = [dict(b, precision=prec, x_engine=t["x_engine"], fft_block=t["fft_block"], fft_engine=t["fft_engine"],
                   x_split=t["x_split"]) for b, t in zip(base, tuned)]
    jobs32 = [dict(b, precision="fp32", x_engine="cuda_core") for b in base]
    samples = sum(w.input_samples for w in ws)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream

    def timed(batch, k):
        for _ in range(args.warmup):
            batch.launch(sptr)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            batch.launch(sptr)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    b16 = Batch(jobs16)
    os.makedirs(args.out_dir, exist_ok=True)
    clk = ClockSampler(local, os.path.join(args.out_dir, f"clocks_r{rank}.csv"))
    barrier(world)
    with clk:
        time.sleep(0.3)
        ms = timed(b16, args.steps)
    ms_max = reduce_max(ms, world, dev)
    launches = b16.launches
    vis16 = [b16.visibilities(i) for i in range(len(ws))]
    b32 = Batch(jobs32)
    ms32 = timed(b32, max(1, args.steps // 2))
    vis32 = [b32.visibilities(i) for i in range(len(ws))]
    b32.close()
    err = [float(np.sqrt(np.sum(np.abs(a - b) ** 2) / max(np.sum(np.abs(b) ** 2), 1e-30))) for a, b in zip(vis16, vis32)]

    # e2e: a batch built on pinned HOST inputs: every job's host->device copy is a memcpy node at the
    # head of its own graph branch, so copies of some jobs overlap other jobs' correlation; then a
    # device->host read of every job's visibilities
    e2e = None
    if not args.no_e2e:
        import ctypes as C
        from gcorr_gb300 import _lib as L
        host = [[x.cpu().pin_memory() for x in d["inputs"]] for d in data]
        h2d_gbs = h2d_probe(max((x for hx in host for x in hx), key=lambda t: t.numel()), dev)
        bh = Batch([dict(j, inputs=hx) for j, hx in zip(jobs16, host)])
        outs = [torch.empty((bh.shapes[i][0] * 4 * bh.shapes[i][1],), dtype=torch.complex64).pin_memory()
                for i in range(len(ws))]

        def e2e_step():
            bh.launch(sptr)
            stream.synchronize()
            for i in range(len(ws)):
                h = bh.handle(i)
                L.check(L.lib().gxc_get_visibilities(h, C.c_void_p(outs[i].data_ptr())), h, "get")

        for _ in range(args.warmup):
            e2e_step()
        n_e2e = max(args.steps, 20)  # wall-clock steps, as for the single-job e2e below
        gc.collect()
        gc.disable()
        step_ms = []
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            ts = time.perf_counter()
            e2e_step()
            step_ms.append((time.perf_counter() - ts) * 1e3)
        ems = (time.perf_counter() - t0) / n_e2e * 1e3
        gc.enable()
        ems = reduce_max(ems, world, dev)
        e2e = {"value": samples * world / (ems / 1e3) / 1e9, "unit": "input Gsamples/s", "steps": n_e2e,
               "step_ms_min_median_max": [min(step_ms), statistics.median(step_ms), max(step_ms)],
               "h2d_bytes_per_step": int(sum(x.numel() for hx in host for x in hx)),
               "d2h_bytes_per_step": int(sum(o.numel() * 8 for o in outs)), "ms_per_step": ems,
               "api": "gxc_batch_launch on pinned host inputs (copies inside the graph)",
               "h2d_probe_gbs": h2d_gbs,
               "matches_device_run": bool(all(np.array_equal(outs[i].numpy().reshape(vis16[i].shape), vis16[i])
                                              for i in range(len(ws))))}
        bh.close()
    b16.close()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        plan = port_plan(ws, 12.0, nthreads)
        cs, ct = run_plan(plan, nthreads)
        cpu = {"value": cs / ct / 1e9, "unit": "input Gsamples/s", "cores": nthreads, "nproc": nthreads,
               "cpu_model": cpu_model(), "kind": plan_kind(plan),
               "sample": "; ".join(f"{n} of {j.nfft} FFTs ({'reference' if run is cpu_ref_run else 'port'})"
                                   for j, n, _, run in plan)
                         + f" (random bytes, {nthreads} threads), {ct:.1f} s"}
    if rank == 0:
        pk = peaks()
        line = {
            "metric": "input Gsamples/s", "value": samples * world / (ms_max / 1e3) / 1e9, "unit": "input Gsamples/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f16", "data": "synthetic",
            "config": {"workload": CONFIGS["c3"][0], "parallelism": f"replicas x{world}",
                       "jobs": [{"nant": w.nant, "nchan": w.nchan, "nfft": w.nfft, "nbit": w.nbit,
                                 "complex": w.is_complex, "x_engine": t["x_engine"], "fft_block": t["fft_block"],
                                 "fft_engine": t["fft_engine"], "x_split": t["x_split"], "tuned_ms": t["ms"],
                                 "plans_tried": len(t["tried"])}
                                for w, t in zip(ws, tuned)],
                       "l2": f"inputs larger than L2 ({sum(w.bytes_per_antenna * w.nant for w in ws) / 1e9:.1f} GB)"},
            "fp32_cuda_core_batch_ms": ms32, "speedup_vs_fp32_cuda_core_batch": ms32 / ms,
            "fp16_vs_fp32_rel_rms_per_job": err, "gpu_launches": launches * args.steps,
            "clocks": clk.summary(), "e2e": e2e, "cpu_baseline": cpu, "generator_s": gen_s,
            "roofline": None, "peak_source": pk["source"],
        }
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU side
def sample_errors(w, inputs_dev, poly, fso, args, device, engines=()):
    """Per-product error of the benchmarked path on a sample of the benchmarked workload: FFTs
    [s0, s0+S) from the middle of the sub-integration (the input windows sliced out of the same
    device buffers, the delay polynomial re-expanded about s0), run through the library at the
    bench's precision and engine, against the FP64 oracle (exact rotator, autos included) and,
    with the fxkernel rotator (2-bit real, square nchan), against the reference's own process()
    (oracle/_ref, unmodified fxkernel.cpp) or, where its sources were not staged, the FP32 port.
    Errors are relative RMS over channels per (baseline, product): max and median over products.
    engines: further (name, precision, x_engine) runs compared with the same FP64 oracle output."""
    import dataclasses
    import numpy as np
    from gcorr_gb300 import FxKernel
    from oracle import oracle as O
    nprod = 4 * w.nant * (w.nant + 1) // 2
    S = int(max(2, min(32, 1.5e9 // (nprod * w.nchan), w.nfft)))
    s0 = (w.nfft - S) // 2
    bpf = w.bytes_per_antenna // (w.nfft + 1)
    sl = [x[s0 * bpf:(s0 + S + 1) * bpf] for x in inputs_dev]
    host = [x.cpu().numpy() for x in sl]
    p = np.asarray(poly, dtype=np.float64)
    q = p.copy()
    q[:, 1] = p[:, 1] + 2.0 * p[:, 0] * s0
    q[:, 2] = p[:, 2] + p[:, 1] * s0 + p[:, 0] * s0 * s0
    ws = dataclasses.replace(w, nfft=S)

    def gpu(rotator, autos, precision=args.precision, x_engine=args.x_engine):
        fx = FxKernel(w.nant, w.nchan, S, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, precision=precision,
                      rotator=rotator, autos=autos, x_engine=x_engine, device=device, fft_engine=args.fft_engine)
        fx.setInputData(sl)
        fx.setDelays(q, fso)
        fx.process()
        v, c = fx.visibilities(), fx.baseline_counts()
        fx.close()
        return v, c

    def stats(e, nx):
        return {"max": float(e.max()), "median": float(np.median(e)), "crosses_max": float(e[:nx].max()),
                "crosses_median": float(np.median(e[:nx])) if nx else None,
                "autos_max": float(e[nx:].max()) if e.shape[0] > nx else None}

    nx = w.nant * (w.nant - 1) // 2
    t0 = time.perf_counter()
    vis, cnt = gpu("exact", True)
    ref, rc = O.exact_process(O.config_from_workload(ws, O.ROT_EXACT, True), host, q, fso)
    out = {"ffts": S, "first_fft": s0, "precision": args.precision,
           "vs_fp64": dict(stats(O.rel_rms_per_product(vis, ref), nx), counts_equal=bool(np.array_equal(cnt, rc)))}
    if not w.is_complex and w.nbit == 2 and int(round(w.nchan ** 0.5)) ** 2 == w.nchan and nx > 0:
        vis2, _ = gpu("fxkernel", False)
        if O.ref_available():
            ref2, kind = O.ref_process(w.nant, w.nchan, S, w.lo_hz, w.bw_hz, host, q, fso), "reference"
        else:
            ref2, _ = O.port_process(O.config_from_workload(ws, O.ROT_FXKERNEL, False), host, q, fso)
            kind = "port"
        out["vs_fxkernel"] = dict(stats(O.rel_rms_per_product(vis2, ref2), nx), kind=kind)
    if engines:
        out["engines"] = {}
        for name, prec, eng in engines:
            try:
                v, c = gpu("exact", True, prec, eng)
            except Exception as ex:  # engine not available for this shape
                out["engines"][name] = {"error": str(ex)[:120]}
                continue
            out["engines"][name] = dict(stats(O.rel_rms_per_product(v, ref), nx),
                                        counts_equal=bool(np.array_equal(c, rc)))
    out["seconds"] = time.perf_counter() - t0
    return out


def h2d_probe(buf, dev):
    """Bandwidth of this machine's pinned host->device copy path, GB/s: one antenna's input
    buffer copied alone three times (CUDA events), so an e2e figure can be read against it."""
    import torch
    d = torch.empty(buf.numel(), dtype=buf.dtype, device=dev)
    d.copy_(buf, non_blocking=True)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(3):
        d.copy_(buf, non_blocking=True)
    e1.record()
    torch.cuda.synchronize(dev)
    gbs = 3 * buf.numel() * buf.element_size() / (e0.elapsed_time(e1) / 1e3) / 1e9
    del d
    return gbs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gxcorr", choices=["gxcorr", "reference"])
    ap.add_argument("--config", default="c1", choices=sorted(CONFIGS))
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp16", "fp8"])
    ap.add_argument("--x-engine", default="auto", choices=["auto", "cuda_core", "tensor"])
    ap.add_argument("--fft-engine", default="auto", choices=["auto", "cuda_core", "tensor"],
                    help="F-stage FFT: tensor cores (8192-point FP16/FP8) or CUDA cores")
    ap.add_argument("--fft-block", type=int, default=0)
    ap.add_argument("--nfft", type=int, default=0, help="override the FFT count (small profiling captures)")
    ap.add_argument("--nchan", type=int, default=0, help="override the channel count (small profiling captures)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-xcompare", action="store_true")
    ap.add_argument("--no-errors", action="store_true", help="skip the per-product error sample")
    ap.add_argument("--ref-step-s", type=float, default=6.0)
    ap.add_argument("--out-dir", default=os.path.join(ROOT, "bench_out"), help="clock samples are written here")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.config == "c3":
        return run_batch_bench(args)

    import numpy as np
    import torch
    import gcorr_gb300 as G
    from gcorr_gb300 import synth

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = init_dist(world, "nccl")
    dev = torch.device("cuda", local)
    w = synth.Workload(**{**workload(args.config).__dict__, "seed": 1234 + 7919 * rank})
    if args.nfft > 0:
        w = synth.Workload(**{**w.__dict__, "nfft": args.nfft})
    if args.nchan > 0:
        w = synth.Workload(**{**w.__dict__, "nchan": args.nchan})
    tg = time.perf_counter()
    d = synth.generate(w, device=dev)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - tg
    inputs_dev = d["inputs"]
    stream = torch.cuda.Stream(device=dev)

    fx = G.FxKernel(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, precision=args.precision,
                    rotator="exact", autos=True, x_engine=args.x_engine, fft_block=args.fft_block, device=local,
                    fft_engine=args.fft_engine)
    fx.setInputData(inputs_dev)
    fx.setDelays(d["poly"], d["fso"])
    sptr = stream.cuda_stream

    def step():
        fx.process(stream=sptr, sync=False)

    # per-launch stage events stay on through the timed steps: the roofline below uses the
    # last timed step's F and X launch durations, recorded on the launching stream
    fx.enable_stage_timing(True)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    launches_per_step = fx.launches

    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    os.makedirs(args.out_dir, exist_ok=True)
    clk = ClockSampler(local, os.path.join(args.out_dir, f"clocks_r{rank}.csv"))
    barrier(world)
    torch.cuda.synchronize()
    with clk:
        time.sleep(0.3)
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = ev0.elapsed_time(ev1) / args.steps
    ms_max = reduce_max(ms, world, dev)
    clocks = clk.summary()

    f_ms, x_ms, tot_ms = fx.stage_times()
    fx.enable_stage_timing(False)
    fft_block = fx.fft_block
    nlaunch = fx.num_blocks  # F (and X) launches of one step
    f_engine = fx.fft_engine_used
    vis0 = fx.visibilities()

    # X-stage comparison (untimed): the same sub-integration through each X engine
    xcmp = {}
    if not args.no_xcompare:
        for name, prec, eng in XENGINES:
            try:
                fy = G.FxKernel(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, precision=prec,
                                rotator="exact", autos=True, x_engine=eng, fft_block=args.fft_block, device=local,
                                fft_engine=args.fft_engine)
            except Exception as ex:  # engine not available for this shape
                xcmp[name] = {"error": str(ex)[:120]}
                continue
            fy.setInputData(inputs_dev)
            fy.setDelays(d["poly"], d["fso"])
            fy.enable_stage_timing(True)
            fy.process(stream=sptr, sync=False)
            fy.sync()
            fy.process(stream=sptr, sync=False)
            a, b, c = fy.stage_times()
            v = fy.visibilities()
            den = float(np.sqrt(np.sum(np.abs(vis0.astype(np.complex128)) ** 2)))
            xcmp[name] = {"x_ms": b, "f_ms": a, "total_ms": c,
                          "rel_rms_vs_default": float(np.sqrt(np.sum(np.abs(v - vis0) ** 2)) / max(den, 1e-30))}
            fy.close()
        if "fp32_cuda_core" in xcmp and "x_ms" in xcmp["fp32_cuda_core"]:
            base = xcmp["fp32_cuda_core"]["x_ms"]
            for k_, v_ in xcmp.items():
                if "x_ms" in v_:
                    v_["speedup_vs_fp32_cuda_core"] = base / v_["x_ms"]

    samples = w.nant * 2 * w.nfft * w.fft_len
    value = samples * world / (ms_max / 1e3) / 1e9

    # e2e: pinned host inputs through the streaming-ingest C ABI (gxc_pipeline_*): every step
    # copies its sub-integration host->device (overlapping the previous step's correlation on a
    # second input slot) and its visibilities device->host; wall clock, synchronised both ends
    e2e = None
    if not args.no_e2e:
        from gcorr_gb300.pipeline import Pipeline
        host = [x.cpu().pin_memory() for x in inputs_dev]
        h2d_gbs = h2d_probe(host[0], dev)
        pipe = Pipeline(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, slots=2, integrate=False,
                        precision=args.precision, rotator="exact", autos=True, x_engine=args.x_engine,
                        fft_block=args.fft_block, device=local, fft_engine=args.fft_engine)
        outs = [torch.empty((pipe.nbl, 4, w.nchan), dtype=torch.complex64).pin_memory() for _ in range(2)]
        for i in range(args.warmup):
            pipe.submit(host, d["poly"], d["fso"], out=outs[i % 2])
        pipe.sync()
        barrier(world)
        # wall-clock steps: at least 20, so that one slow host copy (tens of ms, seen on some
        # hosts) moves the mean by little
        n_e2e = max(args.steps, 20)
        # Python's cyclic garbage collector is paused in the host-side timed loops (the library's
        # calls are C; a full collection of the interpreter's objects took ~0.1 s at times)
        gc.collect()
        gc.disable()
        t0 = time.perf_counter()
        for i in range(n_e2e):
            pipe.submit(host, d["poly"], d["fso"], out=outs[i % 2])
        pipe.sync()
        ems = (time.perf_counter() - t0) / n_e2e * 1e3
        gc.enable()
        ems = reduce_max(ems, world, dev)
        h2d = sum(int(x.numel()) for x in host)
        d2h = int(outs[0].numel()) * 8
        vis_h = outs[(n_e2e - 1) % 2].numpy()

        def rel_rms(a, b):
            return float(np.sqrt(np.mean(np.abs(a - b) ** 2) / max(np.mean(np.abs(b) ** 2), 1e-300)))

        e2e = {"value": samples * world / (ems / 1e3) / 1e9, "unit": "input Gsamples/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": ems,
               "api": "gxc_pipeline_submit (2 input slots, copy/compute overlap)",
               "h2d_probe_gbs": h2d_gbs, "steps": n_e2e,
               "matches_device_run": bool(np.array_equal(vis_h, vis0)),
               # another handle: where the device memory budget caps the FFT block, its blocks (the
               # accumulation order) can differ from the device run's
               "rel_rms_vs_device_run": rel_rms(vis_h, vis0)}
        pipe.close()
        if world == 1:
            # the drop-in path: FxKernel-style process() of one sub-integration on pinned host
            # buffers (input copies in time-ordered chunks on the handle's copy stream), then the
            # visibilities read back; one sub-integration at a time, nothing overlaps across steps
            from gcorr_gb300 import FxKernel
            fxh = FxKernel(w.nant, w.nchan, w.nfft, w.nbit, w.lo_hz, w.bw_hz, w.is_complex, precision=args.precision,
                           rotator="exact", autos=True, x_engine=args.x_engine, fft_block=args.fft_block, device=local,
                           fft_engine=args.fft_engine)
            fxh.setInputData(host)
            fxh.setDelays(d["poly"], d["fso"])
            # the visibilities read back into one preallocated pinned buffer, as the C++ drop-in class
            # reads them into the vector it allocates once
            vbuf = torch.empty((fxh.nbaselines, 4, w.nchan), dtype=torch.complex64).pin_memory()
            for _ in range(max(1, args.warmup)):
                fxh.process()
                fxh.visibilities(out=vbuf)
            step_ms = []
            gc.collect()
            gc.disable()
            for _ in range(n_e2e):
                t0 = time.perf_counter()
                fxh.process()
                fxh.visibilities(out=vbuf)
                step_ms.append((time.perf_counter() - t0) * 1e3)
            gc.enable()
            fms = sum(step_ms) / n_e2e
            e2e["fxkernel_process"] = {"value": samples / (fms / 1e3) / 1e9, "ms_per_step": fms,
                                       "step_ms_min_median_max": [min(step_ms), statistics.median(step_ms),
                                                                  max(step_ms)],
                                       "api": "gxc_set_input (pinned host) + gxc_process + gxc_get_visibilities",
                                       # host inputs start with a shorter FFT block (the first
                                       # correlation waits for less copying): the accumulation
                                       # order, not the arithmetic, differs from the device run
                                       "rel_rms_vs_device_run": rel_rms(vbuf.numpy(), vis0)}
            fxh.close()

    # roofline of the dominant kernel, per launch: algorithmic bytes of one launch (units = FFTs
    # of all streams it processes) over that kernel's average launch duration in the timed step
    pk = peaks()
    esz = {"fp32": 8, "fp16": 4, "fp8": 2}[args.precision]
    in_bytes = w.bytes_per_antenna * w.nant
    chan_bytes = w.nant * 2 * w.nfft * w.nchan * esz
    nprod = 4 * w.nant * (w.nant + 1) // 2
    xflops = 8.0 * nprod * w.nchan * w.nfft
    fftflops = 5.0 * w.fft_len * np.log2(w.fft_len) * 2 * w.nant * w.nfft
    ffts_per_launch = w.nfft / nlaunch
    f_launch_ms, x_launch_ms = f_ms / nlaunch, x_ms / nlaunch
    f_bytes = (in_bytes + chan_bytes) / nlaunch
    x_bytes = chan_bytes / nlaunch
    fp32_peak = 152 * 128 * 2 * (clocks.get("sm_mhz") or 2070.0) * 1e6 / 1e12  # FP32 FMA lanes, nominal
    tdata = {}
    tfile = os.path.join(ROOT, "profiles", f"traffic_{args.config}_{args.precision}.json")
    if os.path.exists(tfile):
        tdata = json.load(open(tfile))

    def traffic(key):
        t = tdata.get(key)
        return None if not t else t["per_fft"] * ffts_per_launch + t.get("per_launch_const", 0)

    # the F-stage kernel this FFT length and precision runs
    tc_f = f_engine == "tensor"  # the F-stage kernel the handle ran
    if tc_f:
        fkern = "fstage_tc_kernel"
    elif w.fft_len == 8192:
        fkern = "fstage_pair_kernel"
    elif w.fft_len >= 16384 and args.precision != "fp32":
        fkern = "fstage_h_kernel"
    elif w.fft_len == 32768:
        fkern = "fstage_cluster_kernel"
    else:
        fkern = "fstage_kernel"
    if f_ms >= x_ms:
        roof = {"kernel": fkern + " (unpack+rotate+FFT+frac-delay)", "bound": "hbm",
                "achieved": f_bytes / (f_launch_ms / 1e3) / 1e9, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "traffic": traffic("fstage_tc_kernel" if tc_f else "fstage_kernel"),
                "algorithmic_bytes_per_launch": f_bytes,
                "launch_ms": f_launch_ms, "launches_per_step": nlaunch, "ffts_per_launch": ffts_per_launch,
                "fft_tflops": fftflops / (f_ms / 1e3) / 1e12, "fp32_peak_tflops_nominal": fp32_peak}
        roof["fp32_pipe_frac_nominal"] = roof["fft_tflops"] / fp32_peak
        if tc_f:
            # issued MMA work of the four-step DFT products: per window (both pols) 2 x 2*128*128*64
            # (step 1, the real levels against the window's A1) + 2*128*128*256 (step 2) flops
            mma_flops = w.nant * w.nfft * (2 * 2 * 128 * 128 * 64 + 2 * 128 * 128 * 256)
            roof["mma_tflops"] = mma_flops / (f_ms / 1e3) / 1e12
            roof["mma_frac_of_bf16_peak"] = roof["mma_tflops"] / pk["bf16_tflops"]
    else:
        roof = {"kernel": "xstage", "bound": "hbm", "achieved": x_bytes / (x_launch_ms / 1e3) / 1e9,
                "peak": pk["hbm_gbs"], "unit": "GB/s", "traffic": traffic("xstage"),
                "algorithmic_bytes_per_launch": x_bytes, "launch_ms": x_launch_ms, "launches_per_step": nlaunch,
                "ffts_per_launch": ffts_per_launch, "x_tflops": xflops / (x_ms / 1e3) / 1e12}
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["peak_source"] = pk["source"] + " (MEASURED_PEAKS.json hbm_gbs)" if pk["source"] == "measured" else "fallback"

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_sample(w)
    errs = None
    if rank == 0 and not args.no_errors:
        errs = sample_errors(w, inputs_dev, d["poly"], d["fso"], args, local,
                             engines=() if args.no_xcompare else XENGINES)

    if rank == 0:
        line = {
            "metric": "input Gsamples/s", "value": value, "unit": "input Gsamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp32": "f32", "fp16": "f16", "fp8": "e4m3 data, f32 accumulate"}[args.precision],
            "data": "synthetic",
            "config": {"workload": CONFIGS[args.config][0], "nant": w.nant, "nchan": w.nchan, "nfft": w.nfft,
                       "fft_len": w.fft_len, "nbit": w.nbit, "precision": args.precision,
                       "x_engine": args.x_engine, "fft_engine": args.fft_engine, "fft_engine_used": f_engine, "fft_block": fx.fft_block,
                       "autos": True,
                       "parallelism": f"replicas x{world}",
                       "l2": f"inputs larger than L2 ({in_bytes / 1e9:.1f} GB packed, "
                             f"{chan_bytes / 1e9:.1f} GB channelised per step)"},
            "stage_ms": {"f": f_ms, "x": x_ms, "total": tot_ms},
            "x_engines": xcmp,
            "errors": errs,
            "x_tflops": xflops / (x_ms / 1e3) / 1e12,
            "gpu_launches": launches_per_step * args.steps,
            "roofline": roof,
            "clocks": clocks,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "generator_s": gen_s,
        }
        print(json.dumps(line), flush=True)
    fx.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
