#!/usr/bin/env python3
"""Benchmark of the complex-baseband filtering path on GB300 — one JSON line on stdout.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload fir1025|fir63|pfb64|pfb1024|batch256] [--no-secondary]

A step is one pass of the hot path over one batch of synthetic input. The headline workload is
the long FIR (2^24 cf32 samples = 8 tones over 60 dB + AWGN at 10 dB SNR, 1025 Kaiser-windowed-
sinc taps), the one the headline metric (Msamples/s, FIR 1025 taps) is quoted on; by default
the line also carries, under "workloads", the same figures for the other four: fir63 (2^24
samples, 63 taps), pfb64 (64-channel channelizer, 2^24 samples, 1024 taps), pfb1024
(1024-channel channelizer, 2^26 samples, 32768 taps) and batch256 (256 captures of 2^12 .. 2^22
samples, each with its own 31 .. 1025 taps). --workload W reports W alone as the headline.

Timing: per workload, every implementation (arm) gets W untimed steps, then R rounds; a round
times exactly K steps of each arm in turn, between a barrier + device synchronize on both
sides, with CUDA events on the launching stream (max over ranks). The K steps of a round (each
the library's launch call for that arm, alternating buffer sets) are captured once, before the
timed rounds, into one CUDA graph that each round replays (every arm alike): the device
timeline holds the steps' kernels back to back, as a captured launch loop in an application,
not the host side of each call. Each arm's figure is the
median over the rounds; R >= 5 and large enough that the headline arm runs >= 0.5 s in total
(so the clock sampler sees the load). Two input/output buffer pairs alternate, so each step
touches more than the 129 MB L2 and nothing is served from L2 across steps. `value` = all
ranks' samples / time. Errors are over the whole output against the float64 oracle. `e2e` = the
same metric from host buffers through the library's host-facing calls: the FIRs through
rfx_fir_stream (pinned capture, chunks whose upload, kernel and download overlap), the
channelizers through rfx_channelize_host, the batch as one upload, the batch launch and one
download per step.

--impl reference: the project's CPU implementation of the path in float64 (the oracle's threaded
C restatement over every host core) on a bounded prefix of the same workload (rank 0 only).

Under torchrun with N > 1 every rank runs its own replica of the workload (the path needs no
exchange between GPUs): weak scaling.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "gpu-rf-pipeline_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Msamples/s (FIR 1025 taps, 64-ch PFB) tensor-core vs FP32, rel err <=2e-6"
L2_BYTES = 129 * 1024 * 1024


# --- distributed plumbing (one process per GPU under torchrun) ----------------------------

def dist_env() -> tuple[int, int, int]:
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init_dist(world: int, backend: str):
    if world <= 1:
        return None
    import torch.distributed as dist

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(value: float, dist, device=None) -> float:
    """Max of a float over all ranks (the timing reduction; no data-path collective)."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist, device=None) -> None:
    if dist is not None:
        if device is not None and device.type == "cuda":
            dist.barrier(device_ids=[device.index])
        else:
            dist.barrier()


# --- clocks during the timed region ---------------------------------------------------------

class ClockSampler:
    """SM clock, utilization and clock-event reasons every 10 ms during the timed region, read
    through NVML (libnvidia-ml, read-only queries); nvidia-smi -lms 200 when NVML is absent."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, cuda_index: int) -> None:
        self.cuda_index = cuda_index
        self.rows: list[dict] = []
        self.max_mhz = None
        self._stop = threading.Event()
        self._thread = None
        self._proc = None
        self.source = None

    def _nvml_handle(self):
        import ctypes

        nvml = ctypes.CDLL("libnvidia-ml.so.1")
        if nvml.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        handle = ctypes.c_void_p()
        try:
            import torch

            uuid = str(torch.cuda.get_device_properties(self.cuda_index).uuid)
            uuid = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
            if nvml.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(handle)) != 0:
                raise OSError
        except Exception:
            if nvml.nvmlDeviceGetHandleByIndex_v2(self.cuda_index, ctypes.byref(handle)) != 0:
                raise OSError("no NVML handle")
        return nvml, handle

    def _poll_nvml(self, nvml, handle) -> None:
        import ctypes

        class Util(ctypes.Structure):
            _fields_ = [("gpu", ctypes.c_uint), ("memory", ctypes.c_uint)]

        clk = ctypes.c_uint()
        reasons = ctypes.c_ulonglong()
        util = Util()
        get_reasons = getattr(nvml, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nvml.nvmlDeviceGetCurrentClocksThrottleReasons
        while not self._stop.is_set():
            if nvml.nvmlDeviceGetClockInfo(handle, 1, ctypes.byref(clk)) == 0:
                get_reasons(handle, ctypes.byref(reasons))
                nvml.nvmlDeviceGetUtilizationRates(handle, ctypes.byref(util))
                self.rows.append({"sm": float(clk.value), "util": float(util.gpu),
                                  "reasons": [v for k, v in self.REASONS.items()
                                              if reasons.value & k]})
            self._stop.wait(0.01)

    def __enter__(self):
        try:
            import ctypes

            nvml, handle = self._nvml_handle()
            mx = ctypes.c_uint()
            if nvml.nvmlDeviceGetMaxClockInfo(handle, 1, ctypes.byref(mx)) == 0:
                self.max_mhz = float(mx.value)
            self._thread = threading.Thread(target=self._poll_nvml, args=(nvml, handle),
                                            daemon=True)
            self.source = "nvml"
        except Exception:
            try:
                self._proc = subprocess.Popen(
                    ["nvidia-smi", "-i", str(self.cuda_index),
                     "--query-gpu=clocks.sm,clocks.max.sm,utilization.gpu,"
                     "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                     "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                     "--format=csv,noheader,nounits", "-lms", "200"],
                    stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
                self._thread = threading.Thread(target=self._poll_smi, daemon=True)
                self.source = "nvidia-smi"
            except OSError:
                self._thread = None
        if self._thread is not None:
            self._thread.start()
        return self

    def _poll_smi(self) -> None:
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            try:
                self.max_mhz = float(parts[1])
                self.rows.append({"sm": float(parts[0]), "util": float(parts[2]),
                                  "reasons": [n for n, v in zip(names, parts[3:7])
                                              if v.lower() == "active"]})
            except (ValueError, IndexError):
                continue

    def __exit__(self, *exc) -> None:
        self._stop.set()
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        if self._thread is not None:
            self._thread.join(timeout=2)

    def summary(self) -> dict:
        rows = self.rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": [], "samples": 0,
                    "source": self.source}
        busy = [r for r in rows if r["util"] > 0] or rows
        return {"sm_mhz": statistics.median(r["sm"] for r in busy), "sm_max_mhz": self.max_mhz,
                "reasons": sorted({x for r in busy for x in r["reasons"]}),
                "samples": len(busy), "source": self.source}


# --- the workloads ---------------------------------------------------------------------------

def load_workload(name: str):
    from rfx import signals

    if name == "fir1025":
        return signals.long_fir(1 << 24)
    if name == "fir63":
        return signals.plain_fir(1 << 24)
    if name == "pfb64":
        return signals.channelizer64(1 << 24)
    if name == "pfb1024":
        return signals.channelizer1024(1 << 26)
    if name == "batch256":
        return signals.batched_fir()
    raise SystemExit(f"unknown workload {name}")


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained"),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "source": "fallback"}


def capture_graph(enqueue):
    """A CUDA graph holding what `enqueue(stream)` puts on a stream (run once on a side stream
    first, outside the capture)."""
    import torch

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        enqueue(side)
    side.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side, capture_error_mode="relaxed"):
        enqueue(side)
    torch.cuda.synchronize()
    return graph


class RoundGraphs:
    """The K steps of a timed round as one CUDA graph, replayed once per round (captured before
    the timed rounds, one per parity of the round's first step): consecutive launches inside a
    graph start without a host submission between them, as a launch loop captured in a graph
    runs in an application."""

    def prepare(self, steps: int) -> None:
        self.round_graphs = {}
        for parity in (0, 1) if steps % 2 else (0,):
            self.round_graphs[parity] = capture_graph(
                lambda st, p=parity: [self.enqueue_step(p + i, st) for i in range(steps)])
        self.round_steps = steps

    def run_round(self, first: int, steps: int) -> None:
        assert steps == self.round_steps
        self.round_graphs[first % 2 if steps % 2 else 0].replay()


class Arm(RoundGraphs):
    """One implementation on one single-capture workload: its device buffers and one step's
    launch, replayed from a CUDA graph (one per buffer set, each captured once after a warm-up
    run), as the batch arm's step: a step's device work is the launch's kernels alone, and the
    host side of a launch (argument checks, tensor-map encoding) stays off the device timeline.
    The same for every arm."""

    def __init__(self, rfx, w, impl: str, device) -> None:
        import torch

        self.rfx, self.w, self.impl = rfx, w, impl
        n = int(w.x.size)
        self.n = n
        self.xs = [torch.from_numpy(w.x).to(device) for _ in range(2)]
        self.h = torch.from_numpy(w.taps).to(device)
        if w.channels:
            m = w.channels
            f = rfx.frames(n, m)
            self.outs = [torch.empty((f, m), dtype=torch.complex64, device=device)
                         for _ in range(2)]
            self.plan = rfx.ChanPlan(m, n, impl)
            self.launches_per_step = chan_launches(m, impl)
            uses_tc = impl == "tc_split" or (impl == "auto" and w.channels == 64)
            self.kernel = "tc_split" if uses_tc else "plain"
        else:
            self.outs = [torch.empty_like(self.xs[0]) for _ in range(2)]
            self.launches_per_step = 1
            self.kernel = rfx.fir_impl_used(impl, w.taps.size, n)
        self.dtype = "f16x3->f32" if self.kernel == "tc_split" else "f32"
        self.graphs = [capture_graph(lambda st, i=i: self.enqueue_step(i, st)) for i in range(2)]

    def enqueue_step(self, i: int, stream) -> None:
        """One step on buffer set i % 2, through the library's launch call on `stream`."""
        if self.w.channels:
            self.plan.launch(self.xs[i % 2], self.h, self.outs[i % 2], stream=stream)
        else:
            self.rfx.fir_launch(self.impl, self.xs[i % 2], self.h, self.outs[i % 2],
                                stream=stream)

    def launch(self, i: int) -> None:
        self.graphs[i % 2].replay()

    def error(self, ref) -> dict:
        """This arm's whole output against the float64 oracle's (`ref`): the normwise error
        max|y - ref| / max|ref|, per channel for a channelizer, and for the plain FIR whether
        every output equals the float32 chain of the project's kernels bit for bit."""
        import torch
        from oracle import rf_oracle as orc

        w = self.w
        self.launch(0)
        torch.cuda.synchronize()
        got = self.outs[0].cpu().numpy()
        out = {"max_rel_err_vs_f64": orc.normwise_error(got, ref),
               "checked": f"whole output ({got.size} values)"}
        if w.channels:
            out["max_channel_rel_err_vs_f64"] = float(orc.per_channel_error(got, ref).max())
        elif self.kernel == "plain":
            chain = orc.fir_f32_seq(w.x, w.taps)
            out["bit_exact_vs_f32_chain"] = bool(np.array_equal(got.view(np.uint32),
                                                                chain.view(np.uint32)))
        return out

    def release(self) -> None:
        self.graphs = self.round_graphs = None
        self.xs = self.outs = None
        if self.w.channels:
            self.plan.close()


class BatchArm(RoundGraphs):
    """The batched workload: every capture with its own taps, device-resident. auto and tc_split:
    one step is one run of a batch plan (rfx_fir_batch_plan_create, made once before timing):
    ONE persistent launch over all captures. plain: one rfx_fir_batch_launch that runs one
    launch per capture, as the project runs a batch. Either step is replayed from a CUDA graph
    captured once."""

    def __init__(self, rfx, w, impl: str, device) -> None:
        import torch

        self.rfx, self.w, self.impl = rfx, w, impl
        # All captures packed in one buffer (each starting on a 16-byte boundary).
        self.offsets, total = [], 0
        for x, _ in w.captures:
            self.offsets.append(total)
            total += x.size + (x.size & 1)
        self.host = np.zeros(total, np.complex64)
        for (x, _), o in zip(w.captures, self.offsets):
            self.host[o:o + x.size] = x
        self.X = torch.from_numpy(self.host).to(device)
        self.Y = torch.zeros_like(self.X)
        self.caps = []
        for (x, h), o in zip(w.captures, self.offsets):
            self.caps.append((self.X[o:o + x.size], self.Y[o:o + x.size],
                              torch.from_numpy(h).to(device)))
        self.n = int(sum(x.size for x, _ in w.captures))
        self.kernels = [rfx.fir_impl_used(impl, h.size, x.size, batch=True)
                        for x, h in w.captures]
        tc = sum(1 for k in self.kernels if k == "tc_split")
        self.dtype = ("f32" if tc == 0 else "f16x3->f32" if tc == len(self.kernels)
                      else "f16x3->f32 (tensor-core captures) + f32")
        self.kernel = "tc_split" if impl == "tc_split" else "plain" if impl == "plain" else "mixed"
        self.graph = None
        self.plan = None
        if impl == "plain":
            self.arr = (rfx.FirCapture * len(self.caps))()
            for i, (xd, yd, hd) in enumerate(self.caps):
                self.arr[i] = rfx.FirCapture(xd.data_ptr(), yd.data_ptr(), hd.data_ptr(),
                                             xd.numel(), hd.numel(), 0)
            self.launches_per_step = sum(1 for x, _ in w.captures if x.size)
        else:
            self.plan = rfx.FirBatchPlan(self.caps, impl)
            info = self.plan.info()
            self.launches_per_step = info["launches"]
            self.plan_info = info
        # One step captured into a CUDA graph (after a warm-up run), replayed per step.
        self.graph = capture_graph(lambda st: self.enqueue_step(0, st))

    def enqueue_step(self, i: int, stream) -> None:
        """One step through the library's call on `stream` (the same buffers every step)."""
        if self.plan is not None:
            self.plan.run(stream)
        else:
            self.rfx._check(self.rfx.load().rfx_fir_batch_launch(
                self.rfx.parse_fir_impl(self.impl), self.arr, len(self.caps),
                self.rfx._stream_ptr(stream)))

    def launch(self, i: int) -> None:
        self.graph.replay()

    def error(self, ref=None) -> dict:
        """Every capture's whole output against the float64 oracle: the largest normwise error
        over all captures, and separately over the captures each kernel ran (the plain kernel's
        are also checked bit for bit against the float32 chain of the project's kernels)."""
        import torch
        from oracle import rf_oracle as orc

        self.launch(0)
        torch.cuda.synchronize()
        y_all = self.Y.cpu().numpy()
        worst = {"tc_split": 0.0, "plain": 0.0}
        exact = True
        for (x, h), o, kernel in zip(self.w.captures, self.offsets, self.kernels):
            got = y_all[o:o + x.size]
            worst[kernel] = max(worst[kernel], orc.normwise_error(got, orc.fir_fast(x, h)))
            if kernel == "plain":
                exact &= bool(np.array_equal(got.view(np.uint32),
                                             orc.fir_f32_seq(x, h).view(np.uint32)))
        out = {"max_rel_err_vs_f64": max(worst.values()),
               "checked": f"every capture, whole output ({self.n} values)"}
        if "tc_split" in self.kernels:
            out["max_rel_err_tensor_core_captures"] = worst["tc_split"]
        if "plain" in self.kernels:
            out["max_rel_err_plain_captures"] = worst["plain"]
            out["bit_exact_vs_f32_chain"] = exact
        return out

    def release(self) -> None:
        if self.plan is not None:
            self.plan.close()
        self.caps = self.X = self.Y = self.graph = self.plan = self.round_graphs = None


def chan_launches(channels: int, impl: str) -> int:
    """Kernel launches per channelizer step: plain = branch sums + cuFFT's inverse (counted as
    one of ours); tensor core = one fused kernel at 64 channels, branch sums + DFT kernel at
    1024; auto = the tensor-core form at 64 channels, plain otherwise."""
    tc = impl == "tc_split" or (impl == "auto" and channels == 64)
    return 1 if tc and channels == 64 else 2


def arm_order(w) -> list[str]:
    """Arms to time, the headline first: auto first where it is not simply the tensor-core
    form at the headline's own configuration (the short FIR, where it picks the short-filter
    tensor-core form over the exact plain kernel; the batch; and the channelizer above 64
    channels, whose plain form is faster) — it is the arm a user runs."""
    auto_first = bool(w.captures or (not w.channels and w.taps.size < 160)
                      or (w.channels and w.channels != 64))
    return ["auto", "tc_split", "plain"] if auto_first else ["tc_split", "plain"]


def make_arm(rfx, w, impl: str, device):
    return BatchArm(rfx, w, impl, device) if w.captures else Arm(rfx, w, impl, device)


def time_round(launch, steps: int, dist, device, first: int = 0, run_round=None) -> float:
    """Seconds for exactly `steps` steps (`launch(i)` per step, or `run_round(first, steps)` for
    all of them): barrier + synchronize on both sides, CUDA events on the current (launching)
    stream, max over ranks."""
    import torch

    torch.cuda.synchronize()
    barrier(dist, device)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record()
    if run_round is not None:
        run_round(first, steps)
    else:
        for i in range(steps):
            launch(first + i)
    stop.record()
    torch.cuda.synchronize()
    barrier(dist, device)
    return max_over_ranks(start.elapsed_time(stop) / 1e3, dist, device)


MIN_ROUNDS = 5          # the median is taken over at least this many interleaved rounds
TIMED_TARGET_S = 0.5    # and over enough rounds that the headline arm runs this long in total
MAX_ROUNDS = 400


def rounds_for(round_s: float) -> int:
    return int(max(MIN_ROUNDS, min(MAX_ROUNDS, -(-TIMED_TARGET_S // max(round_s, 1e-6)))))


def measure_arms(rfx, w, impls, args, dist, device, sampler=None):
    """Times every available implementation of workload `w`: W warm-up steps each, then R
    rounds, each round timing exactly K steps of every arm in turn (arms interleaved, so drift
    in clocks or the host affects them alike); per arm the median over rounds. R >= 5, and
    enough that the headline arm (the first) runs >= 0.5 s in total. Returns {impl: result}."""
    arms = {}
    for impl in impls:
        try:
            arm = make_arm(rfx, w, impl, device)
            arm.launch(0)
        except rfx.RfxError:
            continue   # not available for this workload in this library
        arms[impl] = arm
    for arm in arms.values():
        for i in range(args.warmup):
            arm.launch(i)
        arm.prepare(args.steps)
    first = next(iter(arms))
    rounds = rounds_for(time_round(arms[first].launch, args.steps, dist, device,
                                   run_round=arms[first].run_round))
    seconds = {impl: [] for impl in arms}
    ctx = sampler if sampler is not None else _Null()
    with ctx:
        for r in range(rounds):
            for impl, arm in arms.items():
                seconds[impl].append(time_round(arm.launch, args.steps, dist, device,
                                                first=r * args.steps, run_round=arm.run_round))
    world = dist.get_world_size() if dist is not None else 1
    out = {}
    for impl, arm in arms.items():
        s = seconds[impl]
        rates = [world * arm.n * args.steps / t / 1e6 for t in s]
        step_s = statistics.median(s) / args.steps
        out[impl] = {"msamples_s": statistics.median(rates), "ms_per_step": step_s * 1e3,
                     "step_s": step_s, "rounds": rounds, "steps_per_round": args.steps,
                     "round_msamples_s": [min(rates), max(rates)],
                     "timed_s": sum(s), "launches_per_step": arm.launches_per_step,
                     "kernel": arm.kernel, "dtype": arm.dtype}
    return arms, out


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return None


# --- CPU baselines (the oracle, timed on the host cores) --------------------------------------

def _grow(fn, size: int, target_s: float, start: int = 1 << 14) -> tuple[int, float]:
    """Runs fn(n) on a doubling prefix length until one pass takes target_s (or n = size)."""
    n = start
    while True:
        n = min(n, size)
        t0 = time.perf_counter()
        fn(n)
        dt = time.perf_counter() - t0
        if dt >= target_s or n == size:
            return n, dt
        n *= 2


def cpu_baseline_of(w, target_s: float = 2.0) -> dict:
    """Two CPU figures for workload `w`, in Msamples/s, each over a bounded prefix:
    * the oracle's threaded C float64 restatement on every host core (kind "port");
    * `numpy_one_core`: the algorithm of the project's own CPU implementation
      (tools/reference.py) on one core — np.convolve in float64 for the FIR, NumPy polyphase
      branch sums and an inverse FFT for the channelizer."""
    from oracle import rf_oracle as orc

    threads = os.cpu_count() or 1
    if w.captures:
        def run_caps(fn, target):
            done, count = 0, 0
            t0 = time.perf_counter()
            for x, h in w.captures:
                fn(x, h)
                done += x.size
                count += 1
                if time.perf_counter() - t0 >= target:
                    break
            return done, count, time.perf_counter() - t0

        done, count, dt = run_caps(lambda x, h: orc.fir_fast(x, h, threads=threads), target_s)
        port = {"value": done / dt / 1e6, "unit": "Msamples/s", "cores": threads,
                "kind": "port", "sample": f"first {count} captures of the batch ({done} "
                f"samples, own taps each), float64, {dt:.2f} s on {threads} threads"}
        done1, count1, dt1 = run_caps(lambda x, h: orc.fir_convolve(x, h), target_s / 2)
        port["numpy_one_core"] = {"value": done1 / dt1 / 1e6, "cores": 1, "sample":
                                  f"np.convolve float64 over the first {count1} captures "
                                  f"({done1} samples), {dt1:.2f} s"}
        return port
    if w.channels:
        m = w.channels
        n, dt = _grow(lambda k: orc.channelize_fast(w.x[:k], w.taps, m, threads=threads),
                      w.x.size, target_s)
        n1, dt1 = _grow(lambda k: orc.channelize(w.x[:k], w.taps, m), w.x.size, target_s / 2,
                        start=1 << 12)
        what = f"M={m}, {w.taps.size} taps"
    else:
        n, dt = _grow(lambda k: orc.fir_fast(w.x[:k], w.taps, threads=threads), w.x.size,
                      target_s)
        n1, dt1 = _grow(lambda k: orc.fir_convolve(w.x[:k], w.taps), w.x.size, target_s / 2,
                        start=1 << 12)
        what = f"{w.taps.size} taps"
    return {"value": n / dt / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"first {n} samples of the workload, {what}, float64, {dt:.2f} s on "
                      f"{threads} threads",
            "numpy_one_core": {"value": n1 / dt1 / 1e6, "cores": 1,
                               "sample": f"first {n1} samples, {what}, "
                                         f"{'NumPy branch sums + ifft' if w.channels else 'np.convolve'}"
                                         f" float64, {dt1:.2f} s"}}


def config_of(w, impl: str, n: int) -> dict:
    if w.captures:
        ks = sorted({int(h.size) for _, h in w.captures})
        return {"workload": w.name, "impl": impl, "captures": len(w.captures), "samples": n,
                "taps": ks, "channels": None,
                "l2": f"inputs larger than L2: {16 * n / 1e9:.2f} GB moved per step",
                "seed": w.meta.get("seed")}
    return {"workload": w.name, "impl": impl, "samples": n, "taps": int(w.taps.size),
            "channels": w.channels or None,
            "l2": "inputs larger than L2: two input/output buffer sets alternate",
            "seed": w.meta.get("seed")}


# --- end to end through the host-facing calls ----------------------------------------------

STREAM_CHUNK = 1 << 21
STREAM_DEPTH = 4


def fir_stream_e2e(rfx, w, impl: str, args) -> dict:
    """The FIR end to end through rfx_fir_stream (the project's streaming path): the capture
    in pinned host memory, chunks of 2^21 samples through a ring of four CUDA streams, upload,
    kernel and download of different chunks overlapping; each pass is timed by the library from
    the first chunk to the last output on the host. Bytes moved: every chunk with its history."""
    import torch

    n = int(w.x.size)
    xp = torch.from_numpy(w.x).pin_memory()
    yp = torch.empty_like(xp).pin_memory()
    times = []
    chunks = 0
    for i in range(args.warmup + args.steps):
        _, ms, chunks = rfx.fir_stream(xp, w.taps, impl=impl, chunk=STREAM_CHUNK,
                                       depth=STREAM_DEPTH, memory="registered", out=yp)
        if i >= args.warmup:
            times.append(ms)
    step_ms = statistics.median(times)
    # Upload per chunk: its outputs widened to the kernel's tile plus one tile (tensor core)
    # or K - 1 samples (plain) of history.
    tc = rfx.fir_impl_used(impl, w.taps.size, n) == "tc_split"
    tile = 96 * 128 if tc else 1
    hist = tile if tc else w.taps.size - 1
    up = 0
    for start in range(0, n, STREAM_CHUNK):
        end = min(n, start + STREAM_CHUNK)
        c0 = start // tile * tile
        c1 = min(n, -(-end // tile) * tile)
        up += c1 - max(0, c0 - hist)
    return {"value": n / (step_ms / 1e3) / 1e6, "unit": "Msamples/s",
            "h2d_bytes_per_step": up * 8 + w.taps.size * 4, "d2h_bytes_per_step": n * 8,
            "step_ms": step_ms, "via": f"rfx_fir_stream (registered pinned buffers, "
                                     f"{chunks} chunks of {STREAM_CHUNK}, depth {STREAM_DEPTH})"}


def ci16_recording(x: np.ndarray) -> np.ndarray:
    """The workload as a ci16 SigMF receiver stores it: each component round(v / max|x| * 0.5 *
    32767) as int16, interleaved."""
    scale = 0.5 * 32767 / float(np.max(np.abs(x)))
    c = np.empty(2 * x.size, dtype="<i2")
    c[0::2] = np.round(x.real.astype(np.float64) * scale)
    c[1::2] = np.round(x.imag.astype(np.float64) * scale)
    return c


def fir_stream_e2e_ci16(rfx, w, impl: str, args) -> dict:
    """The same streamed FIR over the workload recorded as ci16: 4 bytes per sample cross the
    host link instead of 8 and the kernels convert them. The output is the FIR of the
    converted samples (not of the float workload), so this line has no error entry."""
    import torch

    n = int(w.x.size)
    cp = torch.from_numpy(ci16_recording(w.x)).pin_memory()
    yp = torch.empty(n, dtype=torch.complex64).pin_memory()
    times = []
    chunks = 0
    for i in range(args.warmup + args.steps):
        _, ms, chunks = rfx.fir_stream(cp, w.taps, impl=impl, chunk=STREAM_CHUNK,
                                       depth=STREAM_DEPTH, memory="registered", out=yp,
                                       fmt="ci16")
        if i >= args.warmup:
            times.append(ms)
    step_ms = statistics.median(times)
    return {"value": n / (step_ms / 1e3) / 1e6, "unit": "Msamples/s",
            "h2d_bytes_per_step": n * 4, "d2h_bytes_per_step": n * 8, "step_ms": step_ms,
            "via": f"rfx_fir_stream_format (ci16, registered pinned buffers, {chunks} chunks of "
                   f"{STREAM_CHUNK}, depth {STREAM_DEPTH}); h2d bytes exclude the per-chunk "
                   f"history"}


def batch_e2e(rfx, w, impl: str, args, device) -> dict:
    """The batch end to end: every step copies the packed captures from pinned host memory,
    runs rfx_fir_batch_launch and copies every output back, timed with CUDA events."""
    import torch

    arm = BatchArm(rfx, w, impl, device)
    xp = torch.from_numpy(arm.host).pin_memory()
    yp = torch.empty_like(xp).pin_memory()

    def step(i: int) -> None:
        arm.X.copy_(xp, non_blocking=True)
        arm.launch(i)
        yp.copy_(arm.Y, non_blocking=True)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for i in range(args.steps):
        step(i)
    b.record()
    torch.cuda.synchronize()
    step_ms = a.elapsed_time(b) / args.steps
    bytes_ = int(xp.numel()) * 8
    arm.release()
    return {"value": arm.n / (step_ms / 1e3) / 1e6, "unit": "Msamples/s",
            "h2d_bytes_per_step": bytes_, "d2h_bytes_per_step": bytes_, "step_ms": step_ms,
            "via": "rfx_fir_batch_launch between one pinned upload and one download per step "
                   "(captures packed in one buffer; the taps stay resident)"}


def chan_e2e(rfx, w, impl: str, args, fmt: str = "cf32") -> dict:
    """The channelizer end to end through rfx_channelize_host[_format] (pinned host buffers):
    upload, compute and download per run, timed by the library with CUDA events."""
    import torch

    n = int(w.x.size)
    lib = rfx.load()
    zp = torch.empty(rfx.frames(n, w.channels) * w.channels, dtype=torch.complex64).pin_memory()
    b = rfx.Bench(warmup=args.warmup, runs=args.steps)
    if fmt == "cf32":
        xp = torch.from_numpy(w.x).pin_memory()
        rfx._check(lib.rfx_channelize_host(rfx.parse_chan_impl(impl), xp.data_ptr(), n,
                                           w.taps.ctypes.data, w.taps.size, w.channels,
                                           zp.data_ptr(), rfx.ctypes.byref(b)))
        up = n * 8
        via = "rfx_channelize_host (pinned host buffers)"
    else:
        cp = torch.from_numpy(ci16_recording(w.x)).pin_memory()
        rfx._check(lib.rfx_channelize_host_format(
            rfx.parse_chan_impl(impl), 1, 0, cp.data_ptr(), n, w.taps.ctypes.data,
            w.taps.size, w.channels, zp.data_ptr(), rfx.ctypes.byref(b)))
        up = n * 4
        via = "rfx_channelize_host_format (ci16, converted in the kernel's load stage)"
    step_ms = b.h2d_ms_mean + b.kernel_ms_mean + b.d2h_ms_mean
    return {"value": n / (step_ms / 1e3) / 1e6, "unit": "Msamples/s",
            "h2d_bytes_per_step": up + w.taps.size * 4, "d2h_bytes_per_step": zp.numel() * 8,
            "h2d_ms": b.h2d_ms_mean, "kernel_ms": b.kernel_ms_mean, "d2h_ms": b.d2h_ms_mean,
            "via": via}


def e2e_of(rfx, w, impl: str, args, device, with_ci16: bool) -> tuple[dict, dict | None]:
    if w.captures:
        return batch_e2e(rfx, w, impl, args, device), None
    if w.channels:
        return (chan_e2e(rfx, w, impl, args),
                chan_e2e(rfx, w, impl, args, fmt="ci16") if with_ci16 else None)
    return (fir_stream_e2e(rfx, w, impl, args),
            fir_stream_e2e_ci16(rfx, w, impl, args) if with_ci16 else None)


# --- the reference arm -------------------------------------------------------------------------

WORKLOADS = ["fir1025", "fir63", "pfb64", "pfb1024", "batch256"]


def run_reference(args) -> None:
    """The project's CPU implementation of the path (float64) on the host cores: the oracle's
    threaded C restatement, each step a bounded prefix of the workload (rank 0 only)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    head = args.workload or WORKLOADS[0]
    w = load_workload(head)
    times = []
    base = None
    for i in range(args.warmup + args.steps):
        b = cpu_baseline_of(w, target_s=1.0) if i == args.warmup + args.steps - 1 else \
            cpu_port_only(w, target_s=1.0)
        if i >= args.warmup:
            times.append(b["value"])
            base = b
    value = statistics.median(times)
    n = sum(int(x.size) for x, _ in w.captures) if w.captures else int(w.x.size)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Msamples/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {**config_of(w, "reference", n), "l2": "n/a (CPU)"},
        "cpu_baseline": {**base, "value": value},
        "e2e": {"value": value, "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if args.workload is None and not args.no_secondary:
        line["workloads"] = {name: cpu_baseline_of(load_workload(name), target_s=1.0)
                             for name in WORKLOADS[1:]}
    print(json.dumps(line), flush=True)


def cpu_port_only(w, target_s: float) -> dict:
    """The threaded C oracle alone (one reference-arm step)."""
    from oracle import rf_oracle as orc

    threads = os.cpu_count() or 1
    if w.captures:
        done, t0 = 0, time.perf_counter()
        for x, h in w.captures:
            orc.fir_fast(x, h, threads=threads)
            done += x.size
            if time.perf_counter() - t0 >= target_s:
                break
        return {"value": done / (time.perf_counter() - t0) / 1e6}
    if w.channels:
        n, dt = _grow(lambda k: orc.channelize_fast(w.x[:k], w.taps, w.channels,
                                                    threads=threads), w.x.size, target_s)
    else:
        n, dt = _grow(lambda k: orc.fir_fast(w.x[:k], w.taps, threads=threads), w.x.size,
                      target_s)
    return {"value": n / dt / 1e6}


def magnitude_fusion(rfx, w, args, dist, device) -> dict:
    """Steps of |channelize(x)| on the tensor-core plan: fused (rfx_channelize_magnitude_launch,
    4 bytes written per output) against channelize then rfx_magnitude_launch (the complex
    outputs written, read back, and the magnitudes written)."""
    import torch

    n = int(w.x.size)
    f = rfx.frames(n, w.channels)
    xs = [torch.from_numpy(w.x).to(device) for _ in range(2)]
    h = torch.from_numpy(w.taps).to(device)
    mags = [torch.empty((f, w.channels), dtype=torch.float32, device=device) for _ in range(2)]
    z = torch.empty((f, w.channels), dtype=torch.complex64, device=device)
    out = {}
    with rfx.ChanPlan(w.channels, n, "tc_split") as plan:
        def fused(i):
            plan.launch_magnitude(xs[i % 2], h, mags[i % 2])

        def unfused(i):
            plan.launch(xs[i % 2], h, z)
            rfx.magnitude_launch(z, mags[i % 2])

        for fn in (fused, unfused):
            for i in range(args.warmup):
                fn(i)
        secs = {"fused": [], "unfused": []}
        for r in range(MIN_ROUNDS):
            for name, fn in (("fused", fused), ("unfused", unfused)):
                secs[name].append(time_round(fn, args.steps, dist, device))
        for name, s in secs.items():
            t = statistics.median(s)
            out[name] = {"ms_per_step": t / args.steps * 1e3,
                         "msamples_s": n * args.steps / t / 1e6}
    out["speedup_fused"] = out["unfused"]["ms_per_step"] / out["fused"]["ms_per_step"]
    return out


# --- our arm ---------------------------------------------------------------------------------

# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu capture of it on the
# workload (dram__bytes_read.sum + dram__bytes_write.sum); writes still in L2 at the kernel's end
# are not counted by that capture.
NCU_TRAFFIC_BYTES = {
    ("fir1025_tones", "tc_split"): 134.5e6 + 80.1e6,   # profiles/fir_tc_fir1025_full.md
    ("fir63_white", "plain"): 134.2e6 + 89.1e6,        # profiles/fir_plain_fir63_full.md
    ("fir63_white", "tc_split"): 134.3e6 + 79.6e6,     # profiles/fir_tcs_fir63_full.md
    ("pfb64", "tc_split"): 134.4e6 + 83.2e6,           # profiles/chan_tc_pfb64_full.md
}


def useful_flops(w) -> float:
    """Useful arithmetic per step: the FIR's 4 N K flops (summed over captures for the batch);
    the channelizer's branch sums, 4 N ceil(L / M)."""
    if w.captures:
        return sum(4.0 * h.size * x.size for x, h in w.captures)
    n = int(w.x.size)
    if w.channels:
        return 4.0 * n * (-(-w.taps.size // w.channels))
    return 4.0 * n * w.taps.size


def roofline_of(w, res: dict, n: int, pk: dict) -> dict:
    """Roofline of one arm's step: tensor-bound (useful FIR flops over the measured bf16 peak)
    for the long-filter tensor-core FIR (over 129 taps) and the tensor-core batch; HBM-bound (16 B
    per sample: 8 read and 8 written, over the measured copy bandwidth) for everything else,
    including the short-filter tensor-core form, which moves each sample through HBM once and
    whose tensor work is a fraction of its time."""
    step_s = res["step_s"]
    gbs = 16.0 * n / step_s / 1e9
    kernel = res["kernel"]
    short_tc = kernel == "tc_split" and not w.channels and not w.captures and w.taps.size <= 129
    if kernel == "tc_split" and not w.channels and not short_tc:
        tflops = useful_flops(w) / step_s / 1e12
        r = {"bound": "tensor", "achieved": tflops, "peak": pk["bf16_tflops"],
             "unit": "TFLOP/s", "frac": tflops / pk["bf16_tflops"], "traffic": None,
             "hbm_achieved_gbs": gbs, "hbm_frac": gbs / pk["hbm_gbs"]}
        if w.captures:
            r["note"] = "useful FIR flops sum 4 N_i K_i over the captures"
        else:
            c = (w.taps.size + 126) // 128
            r["note"] = ("useful FIR flops 4 N K; executed tensor flops are "
                         "3 * 4 N (128 + 128 C) with C = floor((K + 126) / 128)")
            r["tensor_executed_tflops"] = 3.0 * 4.0 * n * 128 * (c + 1) / step_s / 1e12
    else:
        r = {"bound": "hbm", "achieved": gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
             "frac": gbs / pk["hbm_gbs"], "traffic": None}
    r["peak_source"] = pk["source"] + " (MEASURED_PEAKS.json burst figures)" \
        if pk["source"] == "measured" else pk["source"]
    r["timing"] = (f"CUDA events over the timed rounds: median of {res['rounds']} rounds of "
                   f"{res['steps_per_round']} steps (one CUDA-graph replay per round), "
                   f"{res['launches_per_step']} launch(es) per step")
    traffic = NCU_TRAFFIC_BYTES.get((w.name, kernel))
    if traffic is not None:
        r["traffic"] = traffic
        r["traffic_unit"] = "bytes per launch (ncu, one capture)"
    return r


def measure_workload(rfx, name: str, args, dist, device, rank: int, pk: dict,
                     headline: bool) -> dict:
    """Everything the bench line reports for one workload: every arm timed (interleaved rounds),
    the headline arm's roofline, each arm's error over the whole output, the end-to-end figure,
    the CPU baselines and the clocks seen during the timed rounds."""
    import torch

    w = load_workload(name)
    n = sum(int(x.size) for x, _ in w.captures) if w.captures else int(w.x.size)
    order = arm_order(w)
    sampler = ClockSampler(device.index if device.index is not None else 0)
    arms, res = measure_arms(rfx, w, order, args, dist, device, sampler)
    clocks = sampler.summary()
    impl = next(iter(res))
    prim = res[impl]
    ref = None
    if rank == 0 and not w.captures:
        from oracle import rf_oracle as orc

        ref = (orc.channelize_fast(w.x, w.taps, w.channels) if w.channels
               else orc.fir_fast(w.x, w.taps))
    for k, arm in arms.items():
        if rank == 0:
            res[k].update(arm.error(ref))
        arm.release()
    del arms, ref
    torch.cuda.empty_cache()

    out = {"value": prim["msamples_s"], "ms_per_step": prim["ms_per_step"],
           "dtype": prim["dtype"], "config": config_of(w, impl, n),
           "max_rel_err_vs_f64": prim.get("max_rel_err_vs_f64"),
           "roofline": roofline_of(w, prim, n, pk), "clocks": clocks,
           "gpu_launches": prim["rounds"] * args.steps * prim["launches_per_step"],
           "timing": {"rounds": prim["rounds"], "steps_per_round": args.steps,
                      "statistic": "median over rounds; arms interleaved within each round",
                      "headline_arm_timed_s": prim["timed_s"]},
           "compare": {k: {kk: vv for kk, vv in v.items() if kk not in ("step_s", "timed_s")}
                       for k, v in res.items()}}
    if "plain" in res and impl != "plain":
        out["speedup_vs_plain_fp32"] = prim["msamples_s"] / res["plain"]["msamples_s"]
    if "plain" in res and not w.channels and not w.captures:
        sm_mhz = clocks.get("sm_mhz") or 1900.0
        fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
        flops = useful_flops(w) / res["plain"]["step_s"] / 1e12
        out["plain_fp32_simt"] = {"achieved_tflops": flops,
                                  "peak_tflops_at_sampled_clock": fp32_peak,
                                  "frac": flops / fp32_peak}
    if w.channels == 64 and "tc_split" in res:
        out["channelize_magnitude"] = magnitude_fusion(rfx, w, args, dist, device)
    if rank == 0:
        e2e, e2e_ci16 = e2e_of(rfx, w, impl, args, device, with_ci16=headline or w.channels)
        out["e2e"] = e2e
        if e2e_ci16 is not None:
            out["e2e_ci16_recording"] = e2e_ci16
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline_of(w, target_s=2.0 if headline else 1.0)
    del w
    torch.cuda.empty_cache()
    return out


def run_ours(args) -> None:
    import torch

    import rfx

    rank, world, local = dist_env()
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    dist = init_dist(world, "nccl")
    rfx.load()
    pk = peaks()

    names = [args.workload] if args.workload else \
        (WORKLOADS[:1] if args.no_secondary else WORKLOADS)
    head = measure_workload(rfx, names[0], args, dist, device, rank, pk, headline=True)
    others = {name: measure_workload(rfx, name, args, dist, device, rank, pk, headline=False)
              for name in names[1:]}

    fault = rfx.device_fault()
    if fault:
        raise SystemExit(f"a kernel recorded fault code {fault:#x}")
    if rank == 0:
        line = {
            "metric": METRIC, "value": head["value"], "unit": "Msamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": head["dtype"], "data": "synthetic",
            **{k: v for k, v in head.items()
               if k not in ("value", "ms_per_step", "dtype")},
        }
        line.setdefault("cpu_baseline", None)
        line.setdefault("e2e", None)
        if others:
            line["workloads"] = others
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default=None, choices=WORKLOADS,
                    help="one workload as the headline (default: fir1025 as the headline and "
                         "the other four reported under 'workloads')")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="only the headline workload")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
