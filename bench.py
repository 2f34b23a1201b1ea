#!/usr/bin/env python
"""Benchmark of the FFTFPGA C2C path on GB300.

Headline workload: 256^3 complex64 3D FFT, batch 8, one step = forward then
inverse of the whole batch, inputs resident in HBM (1 GiB per direction, far
above the 129 MB L2, so no flush is needed between steps).  Reported as
algorithmic GB/s: P_min (2 HBM round trips for transforms above 2 MiB, 1 up
to 2 MiB) x read+write x batch x points x 8 B per direction, divided by the
device time.

The default N=1 run also measures every other configuration of the path in
the same JSON line, under "configs" (each with its own device-timed GB/s,
dominant-kernel roofline, CPU baseline, end-to-end figure through the
matching C entry point and error against an FP64 FFT):

  c2c3d_64x1        64^3 x 1, forward + inverse (fftfpgaf_c2c_3d_bram)
  c2c3d_512x1       512^3 x 1 (1 GiB; fftfpgaf_c2c_3d_ddr)
  c2c2d_1024x64     2D 1024^2 x 64 (fftfpgaf_c2c_2d_bram, how_many 64)
  c2c1d_65536x1024  1D 65536 x 1024 (fftfpgaf_c2c_1d)
  ragged48          48 ragged 3D grids, ~2 GiB, one persistent launch each way
  poisson4x128      spectral Poisson-filter loss + gradient, 4 x 128^3
and "tc_split": the tensor-core split-precision form against plain FP32 on
512^3.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload NAME] [--no-configs] [--no-cpu] [--no-tc]

--gpus N > 1: when not already started by torchrun, bench.py starts N rank
processes itself (RANK / LOCAL_RANK / WORLD_SIZE / MASTER_ADDR=127.0.0.1),
one GPU each.  The global batch (batch x N) is split by the batch
partitioner (fftgb.shard); every rank transforms its own grids with no
exchange (weak scaling); the time is the max over ranks.  Rank 0 prints one
JSON line.  --dry-run exercises only the launch and reduction logic (no GPU,
no transform; gloo), for tests on machines without a GPU.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import socket
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
TOL = 2e-6

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
    # small case of the 1D kernels for ncu captures (128 MiB)
    "c2c1d_65536x256": ((65536,), 256, 1),
}
# special workloads: 48 ragged grids (~2 GiB), Poisson-filter loss fwd+bwd
SPECIAL = ("ragged48", "poisson4x128")
HEADLINE = "c2c3d_256x8"
# the other configurations of the path, measured in the default N=1 run
SUBCONFIGS = ("c2c3d_64x1", "c2c3d_512x1", "c2c2d_1024x64", "c2c1d_65536x1024",
              "ragged48", "poisson4x128")

L2_FLUSH_BELOW = 512 * 2 ** 20
FLUSH_BYTES = 512 * 2 ** 20


# ------------------------------------------------------------------ helpers
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


def _capture_graph(step, stream, dev):
    """`step` captured once in a CUDA graph (torch.cuda.graph, after warm-up
    on a side stream, with garbage collection off so no earlier object's
    device memory is freed during the capture).  Returns (graph, "") or
    (None, reason)."""
    import gc
    import torch
    try:
        side = torch.cuda.Stream(dev)
        side.wait_stream(stream)
        with torch.cuda.stream(side):
            for _ in range(3):
                step()
        stream.wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        gc.collect()
        gc.disable()
        try:
            with torch.cuda.graph(graph, capture_error_mode="thread_local"):
                step()
        finally:
            gc.enable()
        graph.replay()
        torch.cuda.synchronize(dev)
        return graph, ""
    except Exception as exc:
        import traceback
        traceback.print_exc()
        return None, f"graph capture unavailable: {exc!r}"[:300]


def _l2_note(bytes_per_grid_set: int, flushed: bool) -> str:
    mib = bytes_per_grid_set / 2 ** 20
    if flushed:
        return (f"input {mib:.0f} MiB per direction fits L2: 512 MiB flush write "
                "before every step, outside the timing")
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
    (profiles/ncu_traffic.txt: `<workload> <pass> <bytes per launch> ...`)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if len(parts) >= 3 and not line.startswith("#"):
            if parts[0] == workload and parts[1] == pass_name:
                return float(parts[2])
    return None


def _pass_times(names, pass_ms, nexec) -> dict:
    """Average launch ms per pass, keyed by kernel name (a repeated name gets
    its pass index appended)."""
    out = {}
    for i, nm in enumerate(names):
        key = nm if names.count(nm) == 1 else f"{nm}#{i}"
        out[key] = pass_ms[i] / max(1, nexec)
    return out


def _pmin(points: int) -> int:
    """HBM round trips per direction of one transform of `points` complex64
    points: 1 when it fits on chip (<= 2 MiB), else 2."""
    return 1 if points * 8 <= 2 * 2 ** 20 else 2


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


def clock_sampler(gpu_index: int):
    try:
        return NvmlSampler(gpu_index)
    except Exception:
        return ClockSampler(gpu_index)


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


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch_ranks(n: int, argv) -> int:
    """Start n rank processes of this script (one per GPU) with the torchrun
    environment, pass rank 0's standard output through and return the first
    non-zero exit status (0 if all ranks succeed)."""
    port = _free_port()
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n),
                   LOCAL_WORLD_SIZE=str(n), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen(
            [sys.executable, os.path.abspath(__file__)] + list(argv), env=env,
            stdout=None if r == 0 else subprocess.DEVNULL))
    rc = 0
    for p in procs:
        c = p.wait()
        rc = rc or c
    return rc


# ------------------------------------------------------------ CPU baseline
def _cpu_sample_batch(dims, batch: int) -> int:
    """Transforms per CPU sample: about 2^24 points (128 MiB), at least one
    grid and at most the workload's batch, so threaded CPU FFTs of small
    transforms have enough independent work."""
    n = math.prod(dims)
    return max(1, min(batch, (1 << 24) // n))


def cpu_baseline_leg(dims, batch, pmin, reps: int) -> dict:
    from oracle import cpu_baseline as cb
    sb = _cpu_sample_batch(dims, batch)
    r = cb.time_transform(dims, batch=sb, reps=reps)
    n = math.prod(dims)
    bytes_step = sb * 2 * pmin * 2 * n * 8  # fwd + inv of the sample
    return {"value": bytes_step / r["seconds"] / 1e9, "unit": "GB/s",
            "cores": r["workers"], "kind": "port",
            "sample": (f"{sb} of the {batch} {'x'.join(map(str, dims))} complex64 "
                       f"transforms, forward+inverse, median of {reps}; pocketfft "
                       "(scipy.fft) threaded over all host cores, FFTW absent on "
                       "this machine"),
            "seconds_per_step": r["seconds"]}


def _cpu_fwd_error(x0, dims, ref) -> float:
    """The CPU single-precision FFT's own forward rel-L2 against FP64 on the
    same grid as the GPU accuracy check."""
    from oracle import cpu_baseline as cb
    from oracle import fft_oracle as orc
    y32 = cb.fft_c64(x0.reshape(dims), tuple(range(len(dims))), False, cb.host_cores())
    return orc.rel_l2(y32.reshape(-1), ref)


# -------------------------------------------------------------- uniform legs
_ABI = {
    # workload dims/batch -> (C entry point, call(lib, N, a, b, inv, batch))
    "3d_batch": ("fftfpgaf_c2c_3d_ddr_batch",
                 lambda L, N, a, b, inv, m: L.fftfpgaf_c2c_3d_ddr_batch(N, a, b, inv, False, m)),
    "3d_bram": ("fftfpgaf_c2c_3d_bram",
                lambda L, N, a, b, inv, m: L.fftfpgaf_c2c_3d_bram(N, a, b, inv, False)),
    "3d_ddr": ("fftfpgaf_c2c_3d_ddr",
               lambda L, N, a, b, inv, m: L.fftfpgaf_c2c_3d_ddr(N, a, b, inv)),
    "2d_bram": ("fftfpgaf_c2c_2d_bram",
                lambda L, N, a, b, inv, m: L.fftfpgaf_c2c_2d_bram(N, a, b, inv, False, m)),
    "1d": ("fftfpgaf_c2c_1d",
           lambda L, N, a, b, inv, m: L.fftfpgaf_c2c_1d(N, a, b, inv, m)),
}


def _abi_for(dims, batch):
    if len(dims) == 3 and len(set(dims)) == 1:
        if batch >= 2:
            return _ABI["3d_batch"]
        return _ABI["3d_bram"] if _pmin(math.prod(dims)) == 1 else _ABI["3d_ddr"]
    if len(dims) == 2 and len(set(dims)) == 1:
        return _ABI["2d_bram"]
    if len(dims) == 1:
        return _ABI["1d"]
    return None


def uniform_leg(workload: str, dev, steps: int, warmup: int, world: int = 1,
                rank: int = 0, local: int = 0, cpu: bool = True) -> dict:
    """Forward + inverse of a uniform batch: device-timed GB/s, dominant
    kernel roofline, FP64 accuracy of grid 0, e2e through the matching C
    entry point with pinned host buffers, CPU baseline (rank 0, N=1)."""
    import torch
    from fftgb import api
    from fftgb.shard import BatchShard
    from oracle import fft_oracle as orc

    dims, batch, pmin = WORKLOADS[workload]
    # weak scaling: the global batch is batch x world, split by the batch
    # partitioner so every rank transforms `batch` grids of its own
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

    # the current stream (the timing stream, or a graph's capture stream)
    def step():
        plan(x, out=y)
        plan(y, inverse=True, scale=1.0 / grid_points, out=z)

    for _ in range(max(3, warmup)):
        step()
    torch.cuda.synchronize(dev)

    # accuracy on grid 0 against the FP64 oracle (outside the timed region)
    acc = None
    if rank == 0:
        x0 = x[:grid_points].cpu().numpy()
        ref = orc.c2c_nd(x0, dims, False)
        rel = orc.rel_l2(y[:grid_points].cpu().numpy(), ref)
        acc = {"rel_l2_fwd_vs_fp64": rel,
               "rel_l2_round_trip": orc.rel_l2(z[:grid_points].cpu().numpy(), x0),
               "snr_db_fwd": -20.0 * math.log10(rel) if rel else None,
               "cpu_fp32_rel_l2_fwd_vs_fp64": _cpu_fwd_error(x0, dims, ref) if cpu else None,
               "grids_checked": 1, "tolerance": TOL, "ok": rel <= TOL}
        del ref

    # working sets under ~4x the 129 MB L2 are timed step by step with an L2
    # flush (a 512 MiB write) between steps, outside the events
    flush = None
    if 3 * n * 8 < L2_FLUSH_BELOW:
        flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    # per-pass CUDA events (the roofline's launch times) inside the timed
    # region: on every step for large grids; on the first two steps only for
    # grids under 64 MiB, whose ~20 us steps the extra event records (and the
    # plain launches profiling falls back to) would visibly slow
    prof_steps = steps if n * 8 >= 64 * 2 ** 20 else min(2, steps)
    # small working sets: a step of a few tens of microseconds is two or four
    # dependent launches, so a slow host would put its own launch latency
    # between the events; their step is also captured in a CUDA graph (the
    # same kernels) and the replays are what is timed, the eager step beside
    graph, timing = None, "eager launches"
    eager_ms = None
    if flush is not None:
        z_eager = z.clone()
        graph, gnote = _capture_graph(step, stream, dev)
        if graph is not None:
            # the replay must recompute the output: clear it first
            y.zero_()
            z.zero_()
            graph.replay()
            torch.cuda.synchronize(dev)
            if not torch.equal(z, z_eager):
                graph, gnote = None, "graph replay differs from the eager step"
        timing = gnote or timing
        plan.profile_begin(2 * prof_steps)
        eager_ms = _timed_steps(step, steps, stream, flush)
        torch.cuda.synchronize(dev)
        pass_ms, nexec = plan.profile_end()
        prof_steps = min(prof_steps, nexec // 2)
    else:
        plan.profile_begin(2 * prof_steps)
    _barrier(world)
    torch.cuda.synchronize(dev)
    with clock_sampler(local) as clk:
        if graph is not None:
            ms = _timed_steps(graph.replay, steps, stream, flush)
            timing = "replays of the step captured in one CUDA graph (same kernels as eager)"
        elif eager_ms is not None:
            ms = eager_ms
        else:
            ms = _timed_steps(step, steps, stream, flush)
        torch.cuda.synchronize(dev)
    _barrier(world)
    if flush is None:
        pass_ms, nexec = plan.profile_end()
    ms = _reduce_max(ms, world, dev)
    ms_per_step = ms / steps
    value = world * bytes_step * steps / (ms * 1e-3) / 1e9

    # dominant kernel roofline (CUDA events on the launching stream)
    names = plan.pass_names()
    i_dom = max(range(len(pass_ms)), key=lambda i: pass_ms[i])
    avg_ms = pass_ms[i_dom] / max(1, nexec)
    # a pass reads and writes the whole batch once; a single-pass plan is
    # its own whole direction
    bytes_launch = 2 * n * 8
    peaks = _peaks()
    achieved = bytes_launch / (avg_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": names[i_dom], "achieved": achieved,
                "peak": peaks["hbm_gbs"], "peak_src": peaks["src"],
                "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                "traffic": _traffic(names[i_dom], workload),
                "bytes_alg_per_launch": bytes_launch,
                "avg_launch_ms": avg_ms, "profiled_steps": prof_steps,
                "passes": _pass_times(names, pass_ms, nexec),
                "whole_step_frac": (bytes_step / (ms_per_step * 1e-3) / 1e9) / peaks["hbm_gbs"]}

    # end to end through the reference-facing C ABI with pinned host buffers
    e2e = None
    abi = _abi_for(dims, batch)
    if abi is not None:
        name, call = abi
        L = api._lib.lib()
        N = dims[-1]
        hx = torch.empty(n, dtype=torch.complex64, pin_memory=True)
        hy = torch.empty_like(hx, pin_memory=True)
        hz = torch.empty_like(hx, pin_memory=True)
        hx.copy_(x.cpu())

        def e2e_step():
            t1 = call(L, N, hx.data_ptr(), hy.data_ptr(), False, batch)
            t2 = call(L, N, hy.data_ptr(), hz.data_ptr(), True, batch)
            return t1.valid and t2.valid
        for _ in range(2):
            assert e2e_step(), f"{name} returned valid=false"
        e2e_steps = max(3, steps // 4)
        _barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            assert e2e_step(), f"{name} returned valid=false"
        el = time.perf_counter() - t0
        el = _reduce_max(el, world, dev)
        e2e = {"value": world * bytes_step * e2e_steps / el / 1e9, "unit": "GB/s",
               "h2d_bytes_per_step": 2 * n * 8, "d2h_bytes_per_step": 2 * n * 8,
               "steps": e2e_steps, "api": f"{name} (host pinned buffers)",
               "ms_per_step": el / e2e_steps * 1e3}
        del hx, hy, hz

    cpu_leg = None
    if rank == 0 and world == 1 and cpu:
        cpu_leg = cpu_baseline_leg(dims, batch, pmin, reps=3)

    leg = {
        "value": value, "unit": "GB/s", "ms_per_step": ms_per_step, "steps": steps,
        "config": {"workload": workload, "dims": list(dims), "batch": batch,
                   "directions": ["forward", "inverse"], "p_min": pmin,
                   "bytes_alg_per_step": bytes_step, "variant": plan.variant,
                   "l2": _l2_note(n * 8, flush is not None), "timing": timing,
                   "eager_ms_per_step": (eager_ms / steps) if eager_ms is not None else None,
                   "parallelism": f"batch-sharded x{world} (no collective)"},
        "accuracy": acc,
        "gflops": world * batch * 2 * 5 * grid_points * math.log2(grid_points)
                  * steps / (ms * 1e-3) / 1e9,
        "roofline": roofline, "cpu_baseline": cpu_leg, "e2e": e2e,
        "clocks": clk.summary(), "gpu_launches": steps * 2 * plan.launches,
    }
    del x, y, z, plan
    torch.cuda.empty_cache()
    return leg


# -------------------------------------------------------------- ragged leg
def _ragged_grouped(s) -> bool:
    """Grids the ragged plan runs as grouped launches of the uniform TMA pass
    pair (the rule of shim/ragged.cu): nz = ny = 256, nx 128 or 256."""
    nz, ny, nx = s
    return nz == 256 and ny == 256 and nx in (128, 256)


def _ragged_parts(shapes, dev, reps: int = 5) -> list:
    """Per-direction device ms of each part of the ragged plan, each run as a
    ragged plan of its own on fresh buffers: the work-list kernel over the
    grids it keeps, and each grouped shape's pass pair.  Returns (name,
    shapes, ms per direction, launches per direction) tuples."""
    import torch
    from fftgb.plan import RaggedPlan
    rest = [s for s in shapes if not _ragged_grouped(s)]
    parts = [("k_ragged", rest)] if rest else []
    for s in sorted({s for s in shapes if _ragged_grouped(s)}, reverse=True):
        grp = [t for t in shapes if t == s]
        parts.append((f"k_xy_tma<{s[2]},64>+k_rz_tma<256,4,8> x {len(grp)} "
                      f"({s[0]}x{s[1]}x{s[2]})", grp))
    out = []
    stream = torch.cuda.current_stream(dev)
    for name, sh in parts:
        rp = RaggedPlan(sh)
        x = torch.zeros(rp.points, dtype=torch.complex64, device=dev)
        y = torch.empty_like(x)
        for _ in range(2):
            rp(x, out=y, stream=stream)
            rp(y, inverse=True, out=x, stream=stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            rp(x, out=y, stream=stream)
            rp(y, inverse=True, out=x, stream=stream)
        e1.record(stream)
        e1.synchronize()
        out.append((name, sh, e0.elapsed_time(e1) / reps / 2, rp.launches))
        del x, y, rp
        torch.cuda.empty_cache()
    return out


def ragged_leg(dev, steps: int, warmup: int, cpu: bool = True) -> dict:
    """Forward + inverse of the 48-grid ragged batch (~2 GiB): the grids of
    256 x 256 x {128, 256} as grouped launches of the uniform TMA pass pair,
    the rest in one persistent work-list launch per direction."""
    import numpy as np
    import torch
    from fftgb import synthetic
    from fftgb.plan import RaggedPlan
    from oracle import fft_oracle as orc

    shapes, seed = synthetic.ragged_shapes()
    rp = RaggedPlan(shapes)
    stream = torch.cuda.current_stream(dev)
    g = torch.Generator(device=dev).manual_seed(8)
    x = torch.view_as_complex((torch.rand(rp.points, 2, device=dev, generator=g) * 2 - 1)
                              .contiguous())
    y = torch.empty_like(x)
    z = torch.empty_like(x)
    sizes = [math.prod(s) for s in shapes]
    bytes_dir = sum(_pmin(m) * 2 * m * 8 for m in sizes)
    bytes_step = 2 * bytes_dir

    def step():
        rp(x, out=y, stream=stream)
        rp(y, inverse=True, out=z, stream=stream)

    for _ in range(max(3, warmup)):
        step()
    torch.cuda.synchronize(dev)
    assert rp.status() == 0, "a persistent-kernel dependency wait gave up"

    # accuracy: the first four grids against the FP64 oracle
    xh = x[: sum(sizes[:4])].cpu().numpy()
    yh = y[: sum(sizes[:4])].cpu().numpy()
    num = den = 0.0
    off = 0
    for s, m in zip(shapes[:4], sizes[:4]):
        ref = orc.c2c_nd(xh[off:off + m], s, False)
        num += float(np.sum(np.abs(yh[off:off + m] - ref) ** 2))
        den += float(np.sum(np.abs(ref) ** 2))
        off += m
    rel = math.sqrt(num / den)

    with clock_sampler(0) as clk:
        ms = _timed_steps(step, steps, stream, None)
        torch.cuda.synchronize(dev)
    value = bytes_step * steps / (ms * 1e-3) / 1e9
    peaks = _peaks()
    dir_ms = ms / steps / 2
    form = "persistent work list + grouped uniform pass pairs"
    # the dominant part of a direction, each part timed on its own after the
    # timed region (device events): its algorithmic bytes per launch over
    # its average launch time
    parts = _ragged_parts(shapes, dev)
    name, psh, pms, plaunch = max(parts, key=lambda t: t[2])
    pbytes = sum(_pmin(math.prod(s)) * 2 * math.prod(s) * 8 for s in psh)
    achieved = pbytes / (pms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": name, "achieved": achieved,
                "peak": peaks["hbm_gbs"], "peak_src": peaks["src"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"],
                "traffic": _traffic("k_ragged" if name == "k_ragged" else
                                    "grouped_" + "x".join(str(v) for v in psh[0]), "ragged48"),
                "bytes_alg_per_launch": pbytes / plaunch, "avg_launch_ms": pms / plaunch,
                "passes": {n: round(m, 4) for n, _, m, _ in parts},
                "whole_step_frac": value / peaks["hbm_gbs"],
                "note": "ms per direction of each part, run on its own"}

    # end to end: pinned host batch -> device, forward, inverse, -> host
    hx = torch.empty(rp.points, dtype=torch.complex64, pin_memory=True)
    hz = torch.empty_like(hx, pin_memory=True)
    hx.copy_(x.cpu())

    def e2e_step():
        x.copy_(hx, non_blocking=True)
        step()
        hz.copy_(z, non_blocking=True)
        torch.cuda.synchronize(dev)
    for _ in range(2):
        e2e_step()
    e2e_steps = max(3, steps // 4)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    el = time.perf_counter() - t0
    e2e = {"value": bytes_step * e2e_steps / el / 1e9, "unit": "GB/s",
           "h2d_bytes_per_step": rp.points * 8, "d2h_bytes_per_step": rp.points * 8,
           "steps": e2e_steps, "ms_per_step": el / e2e_steps * 1e3,
           "api": "fftgb_ragged_exec forward + inverse, pinned host copies in and out"}
    del hx, hz

    cpu_leg = None
    if cpu:
        cpu_leg = ragged_cpu(shapes, reps=3)
    leg = {"value": value, "unit": "GB/s", "ms_per_step": ms / steps, "steps": steps,
           "config": {"workload": "ragged48", "grids": len(shapes), "seed": seed,
                      "bytes": rp.points * 8, "directions": ["forward", "inverse"],
                      "form": form, "p_min": "per grid: 1 up to 2 MiB, else 2",
                      "bytes_alg_per_step": bytes_step,
                      "l2": _l2_note(rp.points * 8, False)},
           "accuracy": {"rel_l2_fwd_vs_fp64": rel, "grids_checked": 4,
                        "tolerance": TOL, "ok": rel <= TOL},
           "gflops": sum(2 * 5 * m * math.log2(m) for m in sizes) * steps / (ms * 1e-3) / 1e9,
           "roofline": roofline, "cpu_baseline": cpu_leg, "e2e": e2e,
           "clocks": clk.summary(), "gpu_launches": 2 * rp.launches * steps}
    del x, y, z, rp
    torch.cuda.empty_cache()
    return leg


def ragged_cpu(shapes, reps: int) -> dict:
    """pocketfft complex64 over all host cores on a sample of the ragged
    grids (the first grids up to ~2^24 points), forward + inverse."""
    from oracle import cpu_baseline as cb
    sample, pts = [], 0
    for s in shapes:
        if sample and pts + math.prod(s) > (1 << 24):
            break
        sample.append(s)
        pts += math.prod(s)
    secs = 0.0
    for s in sample:
        secs += cb.time_transform(s, batch=1, reps=reps)["seconds"]
    bytes_step = sum(2 * _pmin(math.prod(s)) * 2 * math.prod(s) * 8 for s in sample)
    return {"value": bytes_step / secs / 1e9, "unit": "GB/s", "cores": cb.host_cores(),
            "kind": "port", "seconds_per_step": secs,
            "sample": (f"the first {len(sample)} of the 48 grids ({pts} points), each "
                       f"forward+inverse, median of {reps}; pocketfft complex64 over "
                       "all host cores")}


# -------------------------------------------------------------- Poisson leg
def poisson_leg(dev, steps: int, warmup: int, cpu: bool = True) -> dict:
    """Loss + gradient of the spectral Poisson filter over 4 grids of 128^3
    (4 FFT3 calls per step: two forward, two adjoint) through the fused
    autograd function (fftgb.autograd.poisson_loss_fused)."""
    import numpy as np
    import torch
    from fftgb import autograd as ag
    from fftgb import synthetic
    from oracle import fft_oracle as orc

    dims = (128, 128, 128)
    nb = 4
    n3 = math.prod(dims)
    gk = ag.poisson_filter(dims).to(dev)
    rho_h = synthetic.spectral_field(dims, nb, seed=9).reshape((nb,) + dims)
    pht_h = synthetic.spectral_field(dims, nb, seed=10).reshape((nb,) + dims)
    rho = torch.from_numpy(rho_h).to(dev)
    pht = torch.from_numpy(pht_h).to(dev)
    rho.requires_grad_(True)
    n = nb * n3
    bytes_step = 4 * (2 * 2 * n * 8)  # four FFT3 calls, two passes each
    stream = torch.cuda.current_stream(dev)
    plan = ag.plan_for(dims, nb)

    def step():
        rho.grad = None
        loss = ag.poisson_loss_fused(rho, pht)
        loss.backward()
        return loss

    # the same step captured once in a CUDA graph (forward, backward and the
    # gradient's allocation, as torch.cuda.graph captures a training step)
    # and replayed: the kernels are the same, the host dispatch between them
    # is gone
    rho.grad = None
    holder = {}

    def cstep():
        holder["loss"] = step()
    graph, graph_note = _capture_graph(cstep, stream, dev)
    if graph is not None:
        g_loss = holder["loss"]
        g_graph = rho.grad.detach().cpu().numpy()

    for _ in range(max(3, warmup)):
        step()
    torch.cuda.synchronize(dev)
    loss = step()
    g_dev = rho.grad.detach().cpu().numpy()
    if graph is not None:
        rel_graph = orc.rel_l2(g_graph, g_dev)
        if not (rel_graph <= 1e-6 and abs(g_loss.item() - loss.item()) <= 1e-6 * abs(loss.item())):
            graph = None
            graph_note = f"graph replay differs from the eager step (grad rel-L2 {rel_graph:.1e})"

    # accuracy: the loss and its gradient against the FP64 analytic gradient
    # 2 A^H (A rho - phi_t), A = IFFT3(G . FFT3(.)) / N^3, on the host
    ref_loss, ref_grad = _poisson_fp64(rho_h, pht_h, gk.cpu().numpy().astype(np.float64))
    rel_grad = float(np.linalg.norm(g_dev - ref_grad) / np.linalg.norm(ref_grad))
    rel_loss = abs(float(loss.item()) - ref_loss) / abs(ref_loss)

    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    prof = min(2, steps)
    plan.profile_begin(4 * prof)
    eager_ms = _timed_steps(step, steps, stream, flush)
    torch.cuda.synchronize(dev)
    pass_ms, nexec = plan.profile_end()
    with clock_sampler(0) as clk:
        if graph is not None:
            ms = _timed_steps(graph.replay, steps, stream, flush)
            graph_note = ("timed as replays of the step captured in one CUDA graph "
                          f"(grad rel-L2 against the eager step {rel_graph:.1e})")
        else:
            ms = eager_ms
        torch.cuda.synchronize(dev)
    value = bytes_step * steps / (ms * 1e-3) / 1e9
    names = plan.pass_names()
    i_dom = max(range(len(pass_ms)), key=lambda i: pass_ms[i])
    avg_ms = pass_ms[i_dom] / max(1, nexec)
    peaks = _peaks()
    achieved = 2 * n * 8 / (avg_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": names[i_dom], "achieved": achieved,
                "peak": peaks["hbm_gbs"], "peak_src": peaks["src"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"],
                "traffic": _traffic(names[i_dom], "poisson4x128"),
                "bytes_alg_per_launch": 2 * n * 8, "avg_launch_ms": avg_ms,
                "profiled_steps": prof,
                "passes": _pass_times(names, pass_ms, nexec),
                "whole_step_frac": value / peaks["hbm_gbs"]}

    # end to end: rho from pinned host memory, loss and gradient back
    hr = torch.empty(rho.shape, dtype=rho.dtype, pin_memory=True)
    hg = torch.empty_like(hr, pin_memory=True)
    hr.copy_(rho.detach().cpu())
    hl = torch.empty((), dtype=torch.float32, pin_memory=True)

    def e2e_step():
        with torch.no_grad():
            rho.copy_(hr, non_blocking=True)
        loss = step()
        hg.copy_(rho.grad, non_blocking=True)
        hl.copy_(loss.detach(), non_blocking=True)
        torch.cuda.synchronize(dev)
    for _ in range(2):
        e2e_step()
    e2e_steps = max(3, steps // 4)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    el = time.perf_counter() - t0
    e2e = {"value": bytes_step * e2e_steps / el / 1e9, "unit": "GB/s",
           "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8 + 4,
           "steps": e2e_steps, "ms_per_step": el / e2e_steps * 1e3,
           "api": "fftgb.autograd.poisson_loss_fused + backward, eager (fftgb_exec_"
                  "filtered / fftgb_exec / fftgb_residual_sq, adjoints), rho in from "
                  "pinned host memory, loss and gradient out"}

    cpu_leg = None
    if cpu:
        cpu_leg = poisson_cpu(rho_h, pht_h, gk.cpu().numpy(), bytes_step, reps=3)
    leg = {"value": value, "unit": "GB/s", "ms_per_step": ms / steps, "steps": steps,
           "config": {"workload": "poisson4x128", "grids": nb, "dims": list(dims),
                      "step": "loss + gradient (4 FFT3 calls: 2 forward, 2 adjoint; "
                              "G(k) applied inside the transforms, residual and loss "
                              "in one kernel)",
                      "p_min": 2, "bytes_alg_per_step": bytes_step,
                      "l2": _l2_note(n * 8, True), "timing": graph_note,
                      "eager_ms_per_step": eager_ms / steps},
           "accuracy": {"rel_l2_grad_vs_fp64": rel_grad, "rel_loss_vs_fp64": rel_loss,
                        "tolerance_grad": 1e-5, "ok": rel_grad <= 1e-5},
           "roofline": roofline, "cpu_baseline": cpu_leg, "e2e": e2e,
           "clocks": clk.summary(), "gpu_launches": (4 * plan.launches + 1) * steps}
    del rho, pht, gk
    torch.cuda.empty_cache()
    return leg


def _poisson_fp64(rho, pht, g):
    """Loss and analytic gradient 2 A^H (A rho - phi_t) in FP64 on the host
    (A = IFFT3(G . FFT3(.)) / N^3; A^H = A for the real symmetric G)."""
    import numpy as np
    import scipy.fft as sf
    from oracle import cpu_baseline as cb
    w = cb.host_cores()
    axes = (1, 2, 3)

    def A(v):
        return sf.ifftn(sf.fftn(v, axes=axes, workers=w) * g, axes=axes, workers=w)
    r = A(rho.astype(np.complex128)) - pht.astype(np.complex128)
    loss = float(np.sum(np.abs(r) ** 2))
    # A = F^-1 G F with F the unnormalised DFT and F^-1 = F^H / N^3, so
    # A^H = F^H G F^-H = F^-1 G F = A for the real G
    return loss, 2.0 * A(r)


def poisson_cpu(rho, pht, g, bytes_step, reps: int) -> dict:
    """The same loss + gradient in complex64 with pocketfft over all host
    cores (4 FFT3 calls of 4 x 128^3)."""
    import numpy as np
    from oracle import cpu_baseline as cb
    w = cb.host_cores()
    axes = (1, 2, 3)
    g32 = g.astype(np.float32)
    n3 = g.size

    def once():
        rk = cb.fft_c64(rho, axes, False, w)
        phi = cb.fft_c64(rk * g32, axes, True, w) / n3
        r = (phi - pht).astype(np.complex64)
        float(np.sum(np.abs(r) ** 2))
        gk = cb.fft_c64(r, axes, False, w) * g32
        return 2.0 * cb.fft_c64(gk, axes, True, w) / n3
    once()
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        once()
        times.append(time.perf_counter() - t0)
    times.sort()
    s = times[len(times) // 2]
    return {"value": bytes_step / s / 1e9, "unit": "GB/s", "cores": w, "kind": "port",
            "seconds_per_step": s,
            "sample": (f"the whole step (4 grids of 128^3, loss + gradient, 4 FFT3 "
                       f"calls) in complex64 numpy with pocketfft, median of {reps}")}


# ------------------------------------------------------- tensor-core leg
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
        assert p.status() == 0, "a tensor-core completion wait gave up"
        del p, x, y
        torch.cuda.empty_cache()
    out["speedup_vs_fp32"] = {k: out["ms"]["fp32"] / out["ms"][k]
                              for k in ("tc_fp16", "tc_bf16")}
    out["tolerance"] = TOL
    out["c2c3d_256x8"] = _tc_256x8(dev, reps)
    return out


def _tc_256x8(dev, reps: int) -> dict:
    """The same comparison on the headline workload, 256^3 x 8 forward: the
    default FP32 plan (two fused passes fed by TMA) against the split-FP16
    and split-BF16 plans (three axis passes whose radix-16 stages run on the
    tensor cores); rel-L2 of grid 0 against an FP64 FFT."""
    import torch
    from fftgb.plan import Plan
    from oracle import fft_oracle as orc

    dims, batch = (256, 256, 256), 8
    out = {"workload": "256^3 x 8 complex64, forward", "ms": {}, "rel_l2_grid0": {},
           "kernels": {}}
    stream = torch.cuda.current_stream(dev)
    n3 = 256 ** 3
    g = torch.Generator(device=dev).manual_seed(2)
    x = torch.view_as_complex((torch.rand(n3 * batch, 2, device=dev, generator=g) * 2 - 1)
                              .contiguous())
    y = torch.empty_like(x)
    x0 = x[:n3].cpu().numpy()
    ref = orc.c2c_nd(x0, dims, False)
    for prec in ("fp32", "tc_fp16", "tc_bf16"):
        p = Plan(dims, batch, precision=prec)
        out["kernels"][prec] = p.pass_names()
        for _ in range(3):
            p(x, out=y, stream=stream)
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(reps):
            p(x, out=y, stream=stream)
        e.record(stream)
        torch.cuda.synchronize(dev)
        assert p.status() == 0, "a tensor-core completion wait gave up"
        out["ms"][prec] = s.elapsed_time(e) / reps
        out["rel_l2_grid0"][prec] = orc.rel_l2(y[:n3].cpu().numpy(), ref)
        del p
    out["speedup_vs_fp32"] = {k: out["ms"]["fp32"] / out["ms"][k]
                              for k in ("tc_fp16", "tc_bf16")}
    del x, y
    torch.cuda.empty_cache()
    return out


# -------------------------------------------------------------- the arms
def _line(leg: dict, args, world: int) -> dict:
    """The contract keys around one measured leg."""
    line = {"metric": METRIC, "value": leg["value"], "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": leg["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (complex64)",
            "data": "synthetic: seeded U[-1,1) complex64 on device"}
    for k, v in leg.items():
        if k not in ("value", "unit", "ms_per_step", "steps"):
            line[k] = v
    return line


def run_ours(args) -> None:
    import torch

    world, rank, local = _dist()
    if world != args.gpus:
        raise SystemExit(f"--gpus {args.gpus} but WORLD_SIZE={world}")
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    # one rank compiles (the others would write the same objects at once);
    # after the barrier every rank finds the library up to date and loads it
    import __graft_entry__ as ge
    if rank == 0:
        ge.build()
    _barrier(world)
    if rank != 0:
        ge.build()
    cpu = not args.no_cpu
    if args.workload == "ragged48":
        leg = ragged_leg(dev, args.steps, args.warmup, cpu=cpu)
    elif args.workload == "poisson4x128":
        leg = poisson_leg(dev, args.steps, args.warmup, cpu=cpu)
    else:
        leg = uniform_leg(args.workload, dev, args.steps, args.warmup, world=world,
                          rank=rank, local=local, cpu=cpu)
    line = _line(leg, args, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank != 0:
        return
    if world == 1 and args.workload == HEADLINE and not args.no_configs:
        configs = {}
        for name in SUBCONFIGS:
            if name == "ragged48":
                configs[name] = ragged_leg(dev, args.steps, args.warmup, cpu=cpu)
            elif name == "poisson4x128":
                configs[name] = poisson_leg(dev, args.steps, args.warmup, cpu=cpu)
            else:
                configs[name] = uniform_leg(name, dev, args.steps, args.warmup, cpu=cpu)
        line["configs"] = configs
        line["configs_note"] = ("every other configuration of the path, measured "
                                "in this run on this GPU (N=1 only)")
    if args.workload == HEADLINE and world == 1 and not args.no_tc:
        line["tc_split"] = tc_split_leg(dev)
    print(json.dumps(line), flush=True)


def _reference_leg(workload: str, steps: int, warmup: int) -> dict:
    """The reference's CPU path (its FFTW stand-in, pocketfft complex64 over
    all host cores) on a bounded sample of one workload."""
    from oracle import cpu_baseline as cb
    if workload == "ragged48":
        from fftgb import synthetic
        shapes, _ = synthetic.ragged_shapes()
        d = ragged_cpu(shapes, reps=max(1, steps))
        return {"value": d["value"], "ms_per_step": d["seconds_per_step"] * 1e3,
                "cpu_baseline": d, "config": {"workload": workload}}
    if workload == "poisson4x128":
        import numpy as np
        from fftgb import synthetic
        dims = (128, 128, 128)
        rho = synthetic.spectral_field(dims, 4, seed=9).reshape((4,) + dims)
        pht = synthetic.spectral_field(dims, 4, seed=10).reshape((4,) + dims)
        k = np.meshgrid(*[np.fft.fftfreq(m, d=1.0 / m) for m in dims], indexing="ij")
        k2 = sum(v ** 2 for v in k)
        g = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0).astype(np.float32)
        bytes_step = 4 * (2 * 2 * 4 * math.prod(dims) * 8)
        d = poisson_cpu(rho, pht, g, bytes_step, reps=max(1, steps))
        return {"value": d["value"], "ms_per_step": d["seconds_per_step"] * 1e3,
                "cpu_baseline": d, "config": {"workload": workload}}
    dims, batch, pmin = WORKLOADS[workload]
    n = math.prod(dims)
    # warm-up steps, then K timed steps; each step a bounded sample of the
    # batch (about 2^24 points, at least one grid)
    sb = _cpu_sample_batch(dims, batch)
    cb.time_transform(dims, batch=sb, reps=max(1, warmup), seed=1)
    r = cb.time_transform(dims, batch=sb, reps=max(1, steps), seed=2)
    bytes_step = sb * 2 * pmin * 2 * n * 8
    value = bytes_step / r["seconds"] / 1e9
    return {"value": value, "ms_per_step": r["seconds"] * 1e3,
            "config": {"workload": workload, "dims": list(dims), "batch": batch,
                       "sample_batch": sb, "directions": ["forward", "inverse"]},
            "cpu_baseline": {"value": value, "unit": "GB/s", "cores": r["workers"],
                             "kind": "port",
                             "sample": f"{sb} transform(s) of the batch per step, "
                                       "forward+inverse; pocketfft complex64 over all "
                                       "host cores (the reference's FFTW is absent on "
                                       "this machine)"}}


def run_reference(args) -> None:
    world, rank, _ = _dist()
    if rank != 0:
        return
    leg = _reference_leg(args.workload, args.steps, args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": leg["value"], "unit": "GB/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": leg["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (complex64)",
        "data": "synthetic: seeded complex64",
        "config": leg["config"], "cpu_baseline": leg["cpu_baseline"],
        "e2e": {"value": leg["value"], "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if args.workload == HEADLINE and not args.no_configs:
        line["configs"] = {}
        for name in SUBCONFIGS:
            d = _reference_leg(name, max(1, min(3, args.steps)), 1)
            line["configs"][name] = {"value": d["value"], "unit": "GB/s",
                                     "ms_per_step": d["ms_per_step"],
                                     "cpu_baseline": d["cpu_baseline"]}
    print(json.dumps(line), flush=True)


def run_dry(args) -> None:
    """Launch and reduction logic only (no GPU, no transform): every rank
    reports a made-up time of 1 + rank ms, rank 0 prints the max over ranks."""
    import torch
    world, rank, _ = _dist()
    if world != args.gpus:
        raise SystemExit(f"--gpus {args.gpus} but WORLD_SIZE={world}")
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    ms = _reduce_max(1.0 + rank, world, torch.device("cpu"))
    _barrier(world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps({"metric": METRIC, "value": None, "unit": "GB/s",
                          "n_gpus": world, "ms_per_step": ms, "dry_run": True}),
              flush=True)


def run_case(args, spec: str) -> None:
    """A small fixed case for an ncu capture: a few forward transforms of one
    plan (with --pairs, then a timed forward + inverse loop).  SPEC is `NZxNYxNX` (slowest axis
    first) with an optional `:BATCH`, a 1D `N:BATCH`, or `ragged:K` for the
    first K grids of the 48-grid ragged workload, or `ragged:NZxNYxNX*C,...`
    for C grids of each listed shape."""
    import torch
    import __graft_entry__ as ge
    ge.build()
    from fftgb.plan import Plan, RaggedPlan
    from fftgb import synthetic
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    if spec.startswith("real:"):
        run_real_case(args, spec, dev)
        return
    if spec.startswith("ragged:"):
        arg = spec.split(":", 1)[1]
        if "x" in arg:
            shapes = []
            for item in arg.split(","):
                dims, _, count = item.partition("*")
                shapes += [tuple(int(v) for v in dims.split("x"))] * int(count or 1)
        else:
            shapes = synthetic.ragged_shapes()[0][:int(arg)]
        p = RaggedPlan(shapes, precision=args.precision)
        desc = f"ragged {len(p.shapes)} grids, {p.launches} launch(es)"
    else:
        dims_s, _, batch_s = spec.partition(":")
        dims = tuple(int(v) for v in dims_s.split("x"))
        p = Plan(dims, int(batch_s or 1), precision=args.precision)
        desc = f"{p.variant}: {', '.join(p.pass_names())}"
    g = torch.Generator(device=dev).manual_seed(11)
    x = torch.randn(p.points, dtype=torch.complex64, device=dev, generator=g)
    for _ in range(args.reps):
        y = p(x)
    torch.cuda.synchronize(dev)
    st = p.status()
    print(f"case {spec} ({p.points} points): {desc}; {args.reps} forward; status {st}",
          flush=True)
    if args.pairs > 0 and not spec.startswith("ragged:"):
        # forward + inverse pairs, device-timed on the plan's stream (3 warm-up pairs)
        stream = torch.cuda.current_stream(dev)
        for _ in range(3):
            p(x, out=y)
            p(y, out=x, inverse=True)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.pairs):
            p(x, out=y)
            p(y, out=x, inverse=True)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / args.pairs
        npass = len(p.pass_names())
        gbs = 2 * npass * 2 * p.points * 8 / (ms * 1e-3) / 1e9
        print(f"case {spec}: {ms:.4f} ms per forward + inverse pair ({args.pairs} pairs), "
              f"{gbs:.0f} GB/s per pass ({npass} passes, one read + one write each)",
              flush=True)
    del y
    if st != 0:
        raise SystemExit(1)


def run_real_case(args, spec: str, dev) -> None:
    """`real:NZxNYxNX[:BATCH]`: a few R2C transforms of a real-data plan and,
    with --pairs, device-timed R2C + C2R pairs."""
    import torch
    from fftgb.plan import RealPlan
    dims_s, _, batch_s = spec.split(":", 1)[1].partition(":")
    dims = tuple(int(v) for v in dims_s.split("x"))
    p = RealPlan(dims, int(batch_s or 1))
    g = torch.Generator(device=dev).manual_seed(11)
    x = torch.randn(p.real_points, dtype=torch.float32, device=dev, generator=g)
    y = torch.empty(p.spectrum_points, dtype=torch.complex64, device=dev)
    for _ in range(args.reps):
        p.r2c(x, out=y)
    torch.cuda.synchronize(dev)
    print(f"case {spec} ({p.real_points} reals, {p.spectrum_points} spectrum points): "
          f"{args.reps} r2c", flush=True)
    if args.pairs > 0:
        stream = torch.cuda.current_stream(dev)
        for _ in range(3):
            p.r2c(x, out=y)
            p.c2r(y, out=x)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.pairs):
            p.r2c(x, out=y)
            p.c2r(y, out=x)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / args.pairs
        print(f"case {spec}: {ms:.4f} ms per r2c + c2r pair ({args.pairs} pairs)", flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + list(SPECIAL),
                    default=HEADLINE)
    ap.add_argument("--no-configs", action="store_true",
                    help="measure only --workload (skip the other configurations)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline legs")
    ap.add_argument("--no-tc", action="store_true",
                    help="skip the tensor-core precision-form comparison")
    ap.add_argument("--dry-run", action="store_true",
                    help="launch/reduction logic only: no GPU, no transform")
    ap.add_argument("--case", metavar="SPEC", action="append",
                    help="only run a few forward transforms of one small case "
                         "(NZxNYxNX[:BATCH], N:BATCH, ragged:K, "
                         "ragged:NZxNYxNX*C,... or real:NZxNYxNX[:BATCH]) for a "
                         "profiler; repeat for several")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "tc_fp16", "tc_bf16"],
                    help="with --case: the plan's precision form")
    ap.add_argument("--reps", type=int, default=3, help="with --case: forward transforms")
    ap.add_argument("--pairs", type=int, default=0,
                    help="with --case: then time this many forward + inverse pairs")
    args = ap.parse_args()
    if args.case:
        for spec in args.case:
            run_case(args, spec)
        return
    if args.gpus < 1:
        raise SystemExit("--gpus must be >= 1")
    if args.impl == "ours" and args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # started without torchrun: one process per GPU, started here
        sys.exit(launch_ranks(args.gpus, sys.argv[1:]))
    if args.dry_run:
        run_dry(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
