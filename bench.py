#!/usr/bin/env python
"""Benchmark of the FFTFPGA C2C path on GB300.

Workload (default): 256^3 complex64 3D FFT, batch 8, one step = forward then
inverse of the whole batch, inputs resident in HBM (1 GiB per direction, far
above the 129 MB L2, so no flush is needed between steps; workloads that fit
in L2 get a 512 MiB flush write before every step, outside the timing).  Reported as
algorithmic GB/s: P_min (= 2 HBM round trips for grids above 2 MiB) x
read+write x batch x points x 8 B per direction, divided by time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload NAME]

N > 1 runs under torchrun: the global batch (batch x N) is split by the batch
partitioner (fftgb.shard), every rank transforms its own grids with no
exchange (weak scaling).  Prints one JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "fft3d-fpga_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "256^3 C2C FFT GB/s vs HBM roofline; TC-split/FP32 speedup at <=2e-6 rel L2"

WORKLOADS = {
    # name: dims (slowest first), batch, P_min
    "c2c3d_256x8": ((256, 256, 256), 8, 2),
    "c2c3d_256x2": ((256, 256, 256), 2, 2),  # small case for ncu captures
    "c2c3d_512x1": ((512, 512, 512), 1, 2),
    "c2c2d_1024x64": ((1024, 1024), 64, 2),
    "c2c1d_65536x1024": ((65536,), 1024, 1),
    "c2c3d_64x1": ((64, 64, 64), 1, 1),
    # small case of the 512-point column pass for ncu captures (256 MiB)
    "c2c3d_512x512x128": ((512, 512, 128), 1, 2),
    # small case of the 2D kernels for ncu captures (256 MiB)
    "c2c2d_1024x32": ((1024, 1024), 32, 2),
}
# special workloads: 48 ragged grids (~2 GiB), Poisson-filter loss fwd+bwd
SPECIAL = ("ragged48", "poisson4x128")


def run_special(args) -> None:
    """ragged48: forward + inverse of the 48-grid ragged batch (one
    persistent launch each); poisson4x128: loss + gradient of the spectral
    Poisson filter over 4 grids of 128^3 (4 FFT3 calls per step)."""
    import numpy as np
    import torch

    dev = torch.device("cuda", 0)
    import __graft_entry__ as ge
    ge.build()
    from fftgb import synthetic
    from fftgb.plan import RaggedPlan

    stream = torch.cuda.current_stream(dev)
    if args.workload == "ragged48":
        shapes, seed = synthetic.ragged_shapes()
        rp = RaggedPlan(shapes)
        g = torch.Generator(device=dev).manual_seed(8)
        x = torch.view_as_complex((torch.rand(rp.points, 2, device=dev, generator=g) * 2 - 1).contiguous())
        y = torch.empty_like(x)
        z = torch.empty_like(x)
        bytes_step = 0
        for s in shapes:
            n = int(np.prod(s))
            pmin = 1 if n * 8 <= 2 * 2 ** 20 else 2
            bytes_step += 2 * pmin * 2 * n * 8

        def step():
            rp(x, out=y, stream=stream)
            rp(y, inverse=True, out=z, stream=stream)
        launches = 2 * rp.launches
        cfg = {"workload": "ragged48", "grids": len(shapes), "seed": seed,
               "bytes": rp.points * 8, "directions": ["forward", "inverse"],
               "form": "persistent" if rp.launches == 1 else "graph of plans"}
    else:
        from fftgb import autograd as ag
        dims = (128, 128, 128)
        gk = ag.poisson_filter(dims).to(dev)
        rho = torch.from_numpy(synthetic.spectral_field(dims, 4, seed=9).reshape((4,) + dims)).to(dev)
        pht = torch.from_numpy(synthetic.spectral_field(dims, 4, seed=10).reshape((4,) + dims)).to(dev)
        rho.requires_grad_(True)
        n = 4 * 128 ** 3
        bytes_step = 4 * (2 * 2 * n * 8)  # four FFT3 calls, two passes each

        def step():
            rho.grad = None
            loss = ag.poisson_loss(rho, pht, gk)
            loss.backward()
        launches = 4 * 2
        cfg = {"workload": "poisson4x128", "grids": 4, "dims": list(dims),
               "step": "loss + gradient (4 FFT3 calls: 2 forward, 2 adjoint)"}
    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize(dev)
    flush = None
    if args.workload == "poisson4x128":  # 64 MiB per field: flush L2 per step
        flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    cfg["l2"] = _l2_note(cfg.get("bytes", 4 * 128 ** 3 * 8), flush is not None)
    with clock_sampler(0) as clk:
        ms = _timed_steps(step, args.steps, stream, flush)
        torch.cuda.synchronize(dev)
    value = bytes_step * args.steps / (ms * 1e-3) / 1e9
    peaks = _peaks()
    line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (complex64)",
            "data": "synthetic (seeded)", "config": cfg,
            "roofline": {"bound": "hbm", "whole_step_frac": value / peaks["hbm_gbs"],
                         "peak": peaks["hbm_gbs"], "unit": "GB/s"},
            "clocks": clk.summary(), "gpu_launches": launches * args.steps}
    print(json.dumps(line), flush=True)


L2_FLUSH_BELOW = 512 * 2 ** 20
FLUSH_BYTES = 512 * 2 ** 20


def _timed_steps(step, steps: int, stream, flush) -> float:
    """Device milliseconds of ``steps`` calls of ``step`` on ``stream``.
    Without ``flush``: one event pair around the loop.  With it: the buffer
    is overwritten before every step (evicting the 129 MB L2) and only the
    steps are inside the event pairs."""
    import torch
    if flush is None:
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(steps):
            step()
        e.record(stream)
        e.synchronize()
        return s.elapsed_time(e)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    with torch.cuda.stream(stream):
        for s, e in ev:
            flush.fill_(0x5a5a)
            s.record(stream)
            step()
            e.record(stream)
    ev[-1][1].synchronize()
    return sum(s.elapsed_time(e) for s, e in ev)


def _l2_note(bytes_per_grid_set: int, flushed: bool) -> str:
    mib = bytes_per_grid_set / 2 ** 20
    if flushed:
        return f"input {mib:.0f} MiB per direction fits L2: 512 MiB flush write before every step, outside the timing"
    return f"input {mib:.0f} MiB per direction > 129 MB L2; no flush"


def _peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


def _traffic(pass_name: str, workload: str):
    """dram bytes per launch of `pass_name` from the committed ncu summary
    (profiles/ncu_traffic.txt: `<workload> <pass> <bytes per launch>`)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if len(parts) >= 3 and not line.startswith("#"):
            if parts[0] == workload and parts[1] == pass_name:
                return float(parts[2])
    return None


class NvmlSampler:
    """Read-only NVML queries (SM clock, max SM clock, clock-event reasons)
    every ~2 ms from a thread, for the duration of a `with` block."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown",
               0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, gpu_index: int):
        import ctypes
        import threading
        self.ct = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        if self.lib.nvmlDeviceGetHandleByIndex_v2(gpu_index, ctypes.byref(self.h)) != 0:
            raise RuntimeError("nvml handle")
        self.samples = []
        self.stop = threading.Event()
        self.thread = threading.Thread(target=self._run, daemon=True)
        fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
        self.reasons_fn = fn or self.lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def _run(self):
        ct = self.ct
        clk, mx, rs = ct.c_uint(), ct.c_uint(), ct.c_ulonglong()
        while not self.stop.is_set():
            ok = self.lib.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(clk)) == 0
            ok &= self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, ct.byref(mx)) == 0
            ok &= self.reasons_fn(self.h, ct.byref(rs)) == 0
            if ok:
                self.samples.append((clk.value, mx.value, rs.value))
            self.stop.wait(0.002)

    def __enter__(self):
        self.thread.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.thread.join()
        self.lib.nvmlShutdown()

    def summary(self) -> dict:
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0,
                    "source": "nvml"}
        reasons = set()
        for _, _, r in self.samples:
            for bit, name in self.REASONS.items():
                if r & bit:
                    reasons.add(name)
        return {"sm_mhz": statistics.median(s[0] for s in self.samples),
                "sm_max_mhz": max(s[1] for s in self.samples),
                "reasons": sorted(reasons), "samples": len(self.samples),
                "source": "nvml"}


def clock_sampler(gpu_index: int):
    try:
        return NvmlSampler(gpu_index)
    except Exception:
        return ClockSampler(gpu_index)


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _reduce_max(value: float, world: int, device) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _cpu_sample_batch(dims, batch: int) -> int:
    """Transforms per CPU sample: about 2^24 points (128 MiB), at least one
    grid and at most the workload's batch, so threaded CPU FFTs of small
    transforms have enough independent work."""
    n = 1
    for d in dims:
        n *= d
    return max(1, min(batch, (1 << 24) // n))


def cpu_baseline_leg(dims, batch, pmin, reps: int) -> dict:
    from oracle import cpu_baseline as cb
    sb = _cpu_sample_batch(dims, batch)
    r = cb.time_transform(dims, batch=sb, reps=reps)
    n = 1
    for d in dims:
        n *= d
    bytes_step = sb * 2 * pmin * 2 * n * 8  # fwd + inv of the sample
    # the CPU single-precision FFT's own forward error against FP64
    from oracle import fft_oracle as orc
    import numpy as np
    x = orc.uniform_c64(n, seed=77)
    y32 = cb.fft_c64(x.reshape(dims), tuple(range(len(dims))), False, r["workers"])
    rel = orc.rel_l2(y32.reshape(-1), orc.c2c_nd(x, dims, False))
    return {"value": bytes_step / r["seconds"] / 1e9, "unit": "GB/s",
            "rel_l2_fwd_vs_fp64": rel,
            "cores": r["workers"], "kind": "port",
            "sample": (f"{sb} of the {batch} {'x'.join(map(str, dims))} complex64 "
                       f"transforms, forward+inverse, median of {reps}; pocketfft "
                       "(scipy.fft) threaded over all host cores, FFTW absent on this machine"),
            "seconds_per_step": r["seconds"]}


def tc_split_leg(dev, reps: int = 10) -> dict:
    """Precision form on 512^3: plain FP32 vs split-FP16 / split-BF16 tensor
    cores, time per forward transform (CUDA events) and rel-L2 against an
    FP64 FFT (scipy pocketfft) on (a) uniform and (b) plane-wave-density
    inputs."""
    import numpy as np
    import scipy.fft as sf
    import torch
    from fftgb import synthetic
    from fftgb.plan import Plan

    n = 512
    dims = (n, n, n)
    workers = len(os.sched_getaffinity(0))
    inputs = {"uniform": synthetic.uniform_c64(n ** 3, seed=6),
              "plane_wave": synthetic.plane_wave_density(dims, seed=7)}
    refs = {k: sf.fftn(v.reshape(dims).astype(np.complex128), workers=workers)
            for k, v in inputs.items()}
    out = {"workload": "512^3 complex64, forward", "ms": {}, "rel_l2": {}}
    stream = torch.cuda.current_stream(dev)
    for prec in ("fp32", "tc_fp16", "tc_bf16"):
        p = Plan(dims, 1, precision=prec)
        out.setdefault("kernels", {})[prec] = p.pass_names()
        errs = {}
        for k, v in inputs.items():
            x = torch.from_numpy(v).to(dev)
            y = p(x, stream=stream).cpu().numpy().reshape(dims)
            r = refs[k]
            errs[k] = float(np.linalg.norm(y - r) / np.linalg.norm(r))
        x = torch.from_numpy(inputs["uniform"]).to(dev)
        y = torch.empty_like(x)
        for _ in range(3):
            p(x, out=y, stream=stream)
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(reps):
            p(x, out=y, stream=stream)
        e.record(stream)
        torch.cuda.synchronize(dev)
        out["ms"][prec] = s.elapsed_time(e) / reps
        out["rel_l2"][prec] = errs
        del p, x, y
        torch.cuda.empty_cache()
    out["speedup_vs_fp32"] = {k: out["ms"]["fp32"] / out["ms"][k]
                              for k in ("tc_fp16", "tc_bf16")}
    out["tolerance"] = 2e-6
    return out


def run_reference(args) -> None:
    world, rank, _ = _dist()
    if rank != 0:
        return
    dims, batch, pmin = WORKLOADS[args.workload]
    from oracle import cpu_baseline as cb
    n = 1
    for d in dims:
        n *= d
    # warm-up steps, then K timed steps; each step a bounded sample of the
    # batch (about 2^24 points, at least one grid)
    sb = _cpu_sample_batch(dims, batch)
    cb.time_transform(dims, batch=sb, reps=max(1, args.warmup), seed=1)
    r = cb.time_transform(dims, batch=sb, reps=max(1, args.steps), seed=2)
    bytes_step = sb * 2 * pmin * 2 * n * 8
    value = bytes_step / r["seconds"] / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["seconds"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (complex64)",
        "data": "synthetic: seeded U[-1,1) complex64",
        "config": {"workload": args.workload, "dims": list(dims), "batch": batch,
                   "sample_batch": sb, "directions": ["forward", "inverse"]},
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": r["workers"],
                         "kind": "port",
                         "sample": f"{sb} transform(s) of the batch per step, "
                                   "forward+inverse; pocketfft complex64 over all "
                                   "host cores (the reference's FFTW is absent on this machine)"},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    import numpy as np
    import torch

    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    import __graft_entry__ as ge
    ge.build()
    from fftgb import api
    from fftgb.plan import Plan
    from oracle import fft_oracle as orc

    dims, batch, pmin = WORKLOADS[args.workload]
    # weak scaling: the global batch is batch x world, split by the batch
    # partitioner so every rank transforms `batch` grids of its own
    from fftgb.shard import BatchShard
    sh = BatchShard(dims, batch * world, world=world, rank=rank)
    assert sh.count == batch
    plan = sh.plan()
    n = plan.points
    grid_points = n // batch
    bytes_dir = pmin * 2 * n * 8
    bytes_step = 2 * bytes_dir

    g = torch.Generator(device=dev).manual_seed(1234 + rank)
    x = torch.view_as_complex((torch.rand(n, 2, device=dev, generator=g) * 2 - 1).contiguous())
    y = torch.empty_like(x)
    z = torch.empty_like(x)
    stream = torch.cuda.current_stream(dev)

    def step():
        plan(x, out=y, stream=stream)
        plan(y, inverse=True, scale=1.0 / grid_points, out=z, stream=stream)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize(dev)

    # accuracy on grid 0 against the FP64 oracle (outside the timed region)
    rel = None
    if rank == 0:
        x0 = x[:grid_points].cpu().numpy()
        rel = orc.rel_l2(y[:grid_points].cpu().numpy(),
                         orc.c2c_nd(x0, dims, False))
        rt = orc.rel_l2(z[:grid_points].cpu().numpy(), x0)

    # working sets under ~4x the 129 MB L2 are timed step by step with an L2
    # flush (a 512 MiB write) between steps, outside the events
    flush = None
    if 3 * n * 8 < L2_FLUSH_BELOW:
        flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    # per-pass CUDA events (the roofline's launch times) inside the timed
    # region: on every step for large grids; on the first two steps only for
    # grids under 64 MiB, whose ~20 us steps the extra event records (and the
    # plain launches profiling falls back to) would visibly slow
    prof_steps = args.steps if n * 8 >= 64 * 2 ** 20 else min(2, args.steps)
    plan.profile_begin(2 * prof_steps)
    _barrier(world)
    torch.cuda.synchronize(dev)
    with clock_sampler(local) as clk:
        ms = _timed_steps(step, args.steps, stream, flush)
        torch.cuda.synchronize(dev)
    _barrier(world)
    pass_ms, nexec = plan.profile_end()
    ms = _reduce_max(ms, world, dev)
    ms_per_step = ms / args.steps
    value = world * bytes_step * args.steps / (ms * 1e-3) / 1e9

    # dominant kernel roofline (CUDA events on the launching stream)
    names = plan.pass_names()
    i_dom = max(range(len(pass_ms)), key=lambda i: pass_ms[i])
    avg_ms = pass_ms[i_dom] / max(1, nexec)
    bytes_launch = 2 * n * 8
    peaks = _peaks()
    achieved = bytes_launch / (avg_ms * 1e-3) / 1e9
    traffic = _traffic(names[i_dom], args.workload)
    roofline = {"bound": "hbm", "kernel": names[i_dom], "achieved": achieved,
                "peak": peaks["hbm_gbs"], "peak_src": peaks["src"],
                "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                "traffic": traffic, "bytes_alg_per_launch": bytes_launch,
                "avg_launch_ms": avg_ms, "profiled_steps": prof_steps,
                "passes": {names[i]: pass_ms[i] / max(1, nexec) for i in range(len(names))},
                "whole_step_frac": (bytes_step / (ms_per_step * 1e-3) / 1e9) / peaks["hbm_gbs"]}

    # end to end through the reference-facing C ABI with pinned host buffers
    e2e = None
    L = api._lib.lib()
    N = dims[-1]
    if len(dims) == 3 and batch >= 2:
        abi = "fftfpgaf_c2c_3d_ddr_batch"
        call = lambda a, b, inv: L.fftfpgaf_c2c_3d_ddr_batch(N, a, b, inv, False, batch)
    elif len(dims) == 3:
        abi = "fftfpgaf_c2c_3d_ddr"
        call = lambda a, b, inv: L.fftfpgaf_c2c_3d_ddr(N, a, b, inv)
    elif len(dims) == 2:
        abi = "fftfpgaf_c2c_2d_bram"
        call = lambda a, b, inv: L.fftfpgaf_c2c_2d_bram(N, a, b, inv, False, batch)
    else:
        abi = "fftfpgaf_c2c_1d"
        call = lambda a, b, inv: L.fftfpgaf_c2c_1d(N, a, b, inv, batch)
    if len(set(dims)) == 1:
        hx = torch.empty(n, dtype=torch.complex64, pin_memory=True)
        hy = torch.empty_like(hx, pin_memory=True)
        hz = torch.empty_like(hx, pin_memory=True)
        hx.copy_(x.cpu())

        def e2e_step():
            t1 = call(hx.data_ptr(), hy.data_ptr(), False)
            t2 = call(hy.data_ptr(), hz.data_ptr(), True)
            return t1.valid and t2.valid
        for _ in range(2):
            assert e2e_step()
        e2e_steps = max(3, args.steps // 4)
        _barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            assert e2e_step()
        el = time.perf_counter() - t0
        el = _reduce_max(el, world, dev)
        e2e = {"value": world * bytes_step * e2e_steps / el / 1e9, "unit": "GB/s",
               "h2d_bytes_per_step": 2 * n * 8, "d2h_bytes_per_step": 2 * n * 8,
               "steps": e2e_steps, "api": f"{abi} (host pinned buffers)",
               "ms_per_step": el / e2e_steps * 1e3}
        del hx, hy, hz

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline_leg(dims, batch, pmin, reps=3)

    tc = None
    if rank == 0 and args.workload == "c2c3d_256x8" and not args.no_tc:
        del x, y, z
        torch.cuda.empty_cache()
        tc = tc_split_leg(dev)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (complex64)",
            "data": "synthetic: seeded U[-1,1) complex64 on device",
            "config": {"workload": args.workload, "dims": list(dims), "batch": batch,
                       "directions": ["forward", "inverse"], "p_min": pmin,
                       "bytes_alg_per_step": bytes_step,
                       "l2": _l2_note(n * 8, flush is not None),
                       "parallelism": f"batch-sharded x{world} (no collective)"},
            "accuracy": {"rel_l2_fwd_vs_fp64": rel, "rel_l2_round_trip": rt,
                         "snr_db_fwd": -20.0 * math.log10(rel) if rel else None,
                         "tolerance": 2e-6},
            "gflops": world * batch * 2 * 5 * grid_points * math.log2(grid_points)
                      * args.steps / (ms * 1e-3) / 1e9,
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "tc_split": tc,
            "clocks": clk.summary(),
            "gpu_launches": args.steps * 2 * plan.launches,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + list(SPECIAL),
                    default="c2c3d_256x8")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-tc", action="store_true",
                    help="skip the tensor-core precision-form comparison")
    args = ap.parse_args()
    if args.impl == "reference":
        if args.workload in SPECIAL:
            print(json.dumps({"impl": "reference", "unavailable":
                              f"{args.workload} has no CPU reference arm"}))
            return
        run_reference(args)
    elif args.workload in SPECIAL:
        run_special(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
