#!/usr/bin/env python3
"""Benchmark of the complex-baseband filtering path on GB300 — one JSON line on stdout.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload fir1025|fir63|pfb64|pfb1024|batch256]

A step is one pass of the hot path over one batch of synthetic input: by default the long FIR
(2^24 cf32 samples = 8 tones over 60 dB + AWGN at 10 dB SNR, 1025 Kaiser-windowed-sinc taps),
the workload the headline metric (Msamples/s, FIR 1025 taps) is quoted on. The other
workloads: fir63 (2^24 samples, 63 taps), pfb64 (64-channel channelizer, 2^24 samples, 1024
taps), pfb1024 (1024-channel channelizer, 2^26 samples, 32768 taps), batch256 (256 captures of
2^12 .. 2^22 samples, each with its own 31 .. 1025 taps).

Timing: W untimed steps, then exactly K steps between a barrier + device synchronize on both
sides, measured with CUDA events on the launching stream; max over ranks. Two input/output
buffer pairs alternate, so each step touches 536 MB (more than the 129 MB L2) and nothing is
served from L2 across steps. `value` = all ranks' samples / time; `e2e` = the same metric from
host buffers through the library's host-facing calls: the FIRs through rfx_fir_stream (the
project's streaming path: pinned capture, chunks whose upload, kernel and download overlap),
the channelizers through rfx_channelize_host (upload + compute + download), the batch as one
upload, the batch launch and one download per step.

--impl reference: the oracle's float64 restatement of the project's tools/reference.py FIR,
threaded over every host core, on a bounded sample of the same workload (rank 0 only).

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


# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu capture of it on the
# workload (dram__bytes_read.sum + dram__bytes_write.sum); writes still in L2 at the kernel's end
# are not counted by that capture.
NCU_TRAFFIC_BYTES = {
    ("fir1025_tones", "tc_split"): 134.5e6 + 80.1e6,   # profiles/fir_tc_fir1025_full.md
    ("fir63_white", "plain"): 134.2e6 + 89.1e6,        # profiles/fir_plain_fir63_full.md
    ("pfb64", "tc_split"): 134.4e6 + 83.2e6,           # profiles/chan_tc_pfb64_full.md
}


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained"),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "source": "fallback"}


class Arm:
    """One implementation on one workload: its device buffers and one step's launch."""

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
        else:
            self.outs = [torch.empty_like(self.xs[0]) for _ in range(2)]
            self.launches_per_step = 1
        if w.channels:
            uses_tc = impl == "tc_split" or (impl == "auto" and w.channels == 64)
        else:
            uses_tc = impl == "tc_split" or (impl == "auto" and auto_picks_tc(w.taps.size, n))
        self.dtype = "f16x3->f32" if uses_tc else "f32"

    def launch(self, i: int) -> None:
        if self.w.channels:
            self.plan.launch(self.xs[i % 2], self.h, self.outs[i % 2])
        else:
            self.rfx.fir_launch(self.impl, self.xs[i % 2], self.h, self.outs[i % 2])

    def error(self) -> float:
        """Normwise error of this arm's output against the float64 oracle, first 2^18 samples."""
        import torch
        from oracle import rf_oracle as orc

        w = self.w
        self.launch(0)
        torch.cuda.synchronize()
        check_n = min(self.n, 1 << 18)
        if w.channels:
            frames = check_n // w.channels
            got = self.outs[0][:frames].cpu().numpy()
            ref = orc.channelize_fast(w.x[: frames * w.channels], w.taps, w.channels)
            return orc.normwise_error(got, ref)
        got = self.outs[0][:check_n].cpu().numpy()
        return orc.normwise_error(got, orc.fir_fast(w.x[:check_n], w.taps))

    def release(self) -> None:
        self.xs = self.outs = None
        if self.w.channels:
            self.plan.close()


class BatchArm:
    """The batched workload: every capture with its own taps, device-resident; one step is
    one rfx_fir_batch_launch over all captures (tensor core: one persistent launch per 96
    captures, replayed from a CUDA graph captured once; plain: one launch per capture, as the
    project runs a batch)."""

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
        self.arr = (rfx.FirCapture * len(self.caps))()
        for i, (xd, yd, hd) in enumerate(self.caps):
            self.arr[i] = rfx.FirCapture(xd.data_ptr(), yd.data_ptr(), hd.data_ptr(), xd.numel(),
                                         hd.numel(), 0)
        self.impl_v = rfx.parse_fir_impl(impl)
        count = len(self.caps)
        sizes = [(int(x.size), int(h.size)) for x, h in w.captures if x.size]
        if impl == "tc_split":
            self.launches_per_step = -(-count // 96)
            self.dtype = "f16x3->f32"
        elif impl == "auto":
            tc = sum(1 for m, k in sizes if auto_picks_tc(k, m))
            self.launches_per_step = -(-(len(sizes) - tc) // 256) + -(-tc // 96)
            self.dtype = "f16x3->f32 (taps >= 160) + f32"
        else:
            self.launches_per_step = len(sizes)
            self.dtype = "f32"
        self.graph = None
        if impl != "plain":
            # One step captured into a CUDA graph (after a warm-up launch that sets the kernels'
            # attributes), replayed per step.
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                self._launch_on(side)
            side.synchronize()
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, stream=side, capture_error_mode="relaxed"):
                self._launch_on(side)
            torch.cuda.synchronize()

    def _launch_on(self, stream) -> None:
        self.rfx._check(self.rfx.load().rfx_fir_batch_launch(
            self.impl_v, self.arr, len(self.caps), self.rfx._stream_ptr(stream)))

    def launch(self, i: int) -> None:
        if self.graph is not None:
            self.graph.replay()
        else:
            self.rfx._check(self.rfx.load().rfx_fir_batch_launch(self.impl_v, self.arr,
                                                                  len(self.caps), None))

    def error(self) -> float:
        """Largest normwise error against the float64 oracle over every 8th capture (first 2^16
        samples of each)."""
        import torch
        from oracle import rf_oracle as orc

        self.launch(0)
        torch.cuda.synchronize()
        worst = 0.0
        for (x, h), (_, yd, _) in list(zip(self.w.captures, self.caps))[::8]:
            m = min(x.size, 1 << 16)
            got = yd[:m].cpu().numpy()
            worst = max(worst, orc.normwise_error(got, orc.fir_fast(x[:m], h)))
        return worst

    def release(self) -> None:
        self.caps = self.arr = self.X = self.Y = self.graph = None


def auto_picks_tc(num_taps: int, n: int) -> bool:
    """The library's built-in auto rule (tuning.cu): tensor core from 160 taps and 2^16 samples."""
    return num_taps >= 160 and n >= (1 << 16)


def chan_launches(channels: int, impl: str) -> int:
    """Kernel launches per channelizer step: plain = branch sums + cuFFT's inverse (counted as
    one of ours); tensor core = one fused kernel at 64 channels, branch sums + DFT kernel at
    1024; auto = the tensor-core form at 64 channels, plain otherwise."""
    tc = impl == "tc_split" or (impl == "auto" and channels == 64)
    return 1 if tc and channels == 64 else 2


def arm_order(w) -> list[str]:
    """Arms to time, the headline first: auto first where it is not simply the tensor-core
    form (the short FIR, the batch, and the channelizer above 64 channels, whose plain form is
    faster) — it is the arm a user runs."""
    auto_first = bool(w.captures or (not w.channels and w.taps.size < 160)
                      or (w.channels and w.channels != 64))
    return ["auto", "tc_split", "plain"] if auto_first else ["tc_split", "plain"]


def make_arm(rfx, w, impl: str, device):
    return BatchArm(rfx, w, impl, device) if w.captures else Arm(rfx, w, impl, device)


def available(rfx, w, impl: str, device) -> bool:
    """Whether this library can run `impl` on workload `w` (tries one launch)."""
    try:
        arm = make_arm(rfx, w, impl, device)
        arm.launch(0)
        arm.release()
        return True
    except rfx.RfxError:
        return False


def time_device(launch, steps: int, warmup: int, dist, device) -> float:
    """Seconds for `steps` launches: barrier + synchronize on both sides, CUDA events on the
    current stream, max over ranks."""
    import torch

    for i in range(warmup):
        launch(i)
    torch.cuda.synchronize()
    barrier(dist, device)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record()
    for i in range(steps):
        launch(i)
    stop.record()
    torch.cuda.synchronize()
    barrier(dist, device)
    elapsed = start.elapsed_time(stop) / 1e3
    return max_over_ranks(elapsed, dist, device)


def kernel_average_s(launch, count: int) -> float:
    """Average duration of one launch, CUDA events on the launching stream, after the timed
    region (for the roofline)."""
    import torch

    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for i in range(count):
        launch(i)
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3 / count


def cpu_fir_baseline(x: np.ndarray, h: np.ndarray, target_s: float = 2.0) -> dict:
    """The oracle's float64 FIR on all host cores over a growing prefix of the workload, until
    one pass takes at least target_s."""
    from oracle import rf_oracle as orc

    threads = os.cpu_count() or 1
    n = 1 << 14
    while True:
        n = min(n, x.size)
        t0 = time.perf_counter()
        orc.fir_fast(x[:n], h, threads=threads)
        dt = time.perf_counter() - t0
        if dt >= target_s or n == x.size:
            break
        n *= 2
    return {"value": n / dt / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"first {n} samples of the workload, {h.size} taps, float64, "
                      f"{dt:.2f} s on {threads} threads"}


def cpu_chan_baseline(x: np.ndarray, h: np.ndarray, m: int, target_s: float = 2.0) -> dict:
    from oracle import rf_oracle as orc

    threads = os.cpu_count() or 1
    n = 1 << 14
    while True:
        n = min(n, x.size)
        t0 = time.perf_counter()
        orc.channelize_fast(x[:n], h, m, threads=threads)
        dt = time.perf_counter() - t0
        if dt >= target_s or n == x.size:
            break
        n *= 2
    return {"value": n / dt / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"first {n} samples of the workload, M={m}, {h.size} taps, float64, "
                      f"{dt:.2f} s on {threads} threads"}


def cpu_batch_baseline(captures, target_s: float = 2.0) -> dict:
    """The oracle's float64 FIR on all host cores over the batch's captures in order, until
    the captures run so far took at least target_s."""
    from oracle import rf_oracle as orc

    threads = os.cpu_count() or 1
    done = 0
    count = 0
    t0 = time.perf_counter()
    for x, h in captures:
        orc.fir_fast(x, h, threads=threads)
        done += x.size
        count += 1
        if time.perf_counter() - t0 >= target_s:
            break
    dt = time.perf_counter() - t0
    return {"value": done / dt / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"first {count} captures of the batch ({done} samples, own taps each), "
                      f"float64, {dt:.2f} s on {threads} threads"}


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
    tc = impl == "tc_split" or (impl == "auto" and auto_picks_tc(w.taps.size, n))
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


def fir_stream_e2e_ci16(rfx, w, impl: str, args) -> dict:
    """The same streamed FIR over the workload recorded as a ci16 SigMF receiver would store
    it (each component round(v / max|x| * 0.5 * 32767), int16): 4 bytes per sample cross the
    host link instead of 8 and the kernels convert them. The output is the FIR of the
    converted samples (not of the float workload), so this line has no error entry."""
    import torch

    n = int(w.x.size)
    scale = 0.5 * 32767 / float(np.max(np.abs(w.x)))
    c = np.empty(2 * n, dtype="<i2")
    c[0::2] = np.round(w.x.real.astype(np.float64) * scale)
    c[1::2] = np.round(w.x.imag.astype(np.float64) * scale)
    cp = torch.from_numpy(c).pin_memory()
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
            "note": "captures packed in one pinned buffer; one copy each way per step; the "
                    "taps stay resident"}


# --- the reference arm -------------------------------------------------------------------------

def run_reference(args) -> None:
    rank, world, _ = dist_env()
    if rank != 0:
        return
    w = load_workload(args.workload)
    times = []
    base = None
    for i in range(args.warmup + args.steps):
        if w.captures:
            b = cpu_batch_baseline(w.captures, target_s=1.0)
        elif w.channels:
            b = cpu_chan_baseline(w.x, w.taps, w.channels, target_s=1.0)
        else:
            b = cpu_fir_baseline(w.x, w.taps, target_s=1.0)
        if i >= args.warmup:
            times.append(b["value"])
            base = b
    value = statistics.median(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Msamples/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {**config_of(w, "reference", sum(int(x.size) for x, _ in w.captures)
                              if w.captures else int(w.x.size)), "l2": "n/a (CPU)"},
        "cpu_baseline": {**base, "value": value},
        "e2e": {"value": value, "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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

        for name, fn in (("fused", fused), ("unfused", unfused)):
            s = time_device(fn, args.steps, args.warmup, dist, device)
            out[name] = {"ms_per_step": s / args.steps * 1e3,
                         "msamples_s": n * args.steps / s / 1e6}
    out["speedup_fused"] = out["unfused"]["ms_per_step"] / out["fused"]["ms_per_step"]
    return out


# --- our arm ---------------------------------------------------------------------------------

def measure_arms(rfx, w, impls, args, dist, device, sample_clocks=False):
    """Times every available implementation of workload `w`; returns {impl: result}."""
    out = {}
    clocks = None
    for impl in impls:
        if not available(rfx, w, impl, device):
            continue
        arm = make_arm(rfx, w, impl, device)
        if sample_clocks and clocks is None:
            with ClockSampler(device.index if device.index is not None else 0) as cs:
                seconds = time_device(arm.launch, args.steps, args.warmup, dist, device)
            clocks = cs.summary()
        else:
            seconds = time_device(arm.launch, args.steps, args.warmup, dist, device)
        kernel_s = kernel_average_s(arm.launch, max(3, min(args.steps, 10)))
        world = dist.get_world_size() if dist is not None else 1
        out[impl] = {"msamples_s": world * arm.n * args.steps / seconds / 1e6,
                     "ms_per_step": seconds / args.steps * 1e3, "kernel_s": kernel_s,
                     "seconds": seconds, "launches_per_step": arm.launches_per_step,
                     "dtype": arm.dtype, "max_rel_err_vs_f64": arm.error()}
        arm.release()
    return out, clocks


def run_ours(args) -> None:
    import torch

    import rfx

    rank, world, local = dist_env()
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    dist = init_dist(world, "nccl")
    rfx.load()
    pk = peaks()

    w = load_workload(args.workload)
    if w.captures:
        ns = [int(x.size) for x, _ in w.captures]
        n = sum(ns)
        useful = sum(4.0 * h.size * m for (_, h), m in zip(w.captures, ns))
    else:
        n = int(w.x.size)
        if w.channels:
            useful = 4.0 * n * (-(-w.taps.size // w.channels))  # branch FIR flops
        else:
            useful = 4.0 * n * w.taps.size                       # FIR flops
    order = arm_order(w)
    arms, clocks = measure_arms(rfx, w, order, args, dist, device, sample_clocks=True)
    impl = next(iter(arms))
    prim = arms[impl]
    value = prim["msamples_s"]
    kernel_s = prim["kernel_s"]

    # Roofline of the dominant kernel.
    extras: dict = {}
    algo_bytes = 16.0 * n  # 8 B read + 8 B written per sample
    achieved_gbs = algo_bytes / kernel_s / 1e9
    if impl == "tc_split" and w.captures:
        roofline = {"bound": "tensor", "achieved": useful / kernel_s / 1e12,
                    "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                    "frac": useful / kernel_s / 1e12 / pk["bf16_tflops"], "traffic": None,
                    "note": "useful FIR flops sum 4*N_i*K_i over the captures; the short-tap "
                            "captures are bound by HBM instead (hbm_achieved_gbs)"}
        extras["hbm_achieved_gbs"] = achieved_gbs
        extras["hbm_frac"] = achieved_gbs / pk["hbm_gbs"]
    elif impl == "tc_split" and not w.channels:
        roofline = {"bound": "tensor", "achieved": useful / kernel_s / 1e12,
                    "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                    "frac": useful / kernel_s / 1e12 / pk["bf16_tflops"], "traffic": None,
                    "note": "useful FIR flops 4*N*K; executed tensor flops are "
                            "3*4*N*(128+128*C) with C = floor((K+126)/128)"}
        c = (w.taps.size + 126) // 128
        executed = 3.0 * 4.0 * n * 128 * (c + 1)
        extras["tensor_executed_tflops"] = executed / kernel_s / 1e12
    else:
        roofline = {"bound": "hbm", "achieved": achieved_gbs, "peak": pk["hbm_gbs"],
                    "unit": "GB/s", "frac": achieved_gbs / pk["hbm_gbs"], "traffic": None}
    roofline["peak_source"] = pk["source"]
    kernel_impl = impl
    if impl == "auto" and not w.captures and not w.channels:
        kernel_impl = "tc_split" if auto_picks_tc(w.taps.size, n) else "plain"
    if impl == "auto" and w.channels:
        kernel_impl = "tc_split" if w.channels == 64 else "plain"
    traffic = NCU_TRAFFIC_BYTES.get((w.name, kernel_impl))
    if traffic is not None:
        roofline["traffic"] = traffic
        roofline["traffic_unit"] = "bytes per launch (ncu, one capture)"
    if "plain" in arms and not w.channels and not w.captures:
        sm_mhz = (clocks or {}).get("sm_mhz") or 1900.0
        fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
        ks = arms["plain"]["kernel_s"]
        extras["plain_fp32_simt"] = {"achieved_tflops": useful / ks / 1e12,
                                     "peak_tflops_at_sampled_clock": fp32_peak,
                                     "frac": useful / ks / 1e12 / fp32_peak}
    compare = {k: {kk: vv for kk, vv in v.items() if kk not in ("seconds",)}
               for k, v in arms.items()}
    if "plain" in arms and impl != "plain":
        extras["speedup_vs_plain_fp32"] = value / arms["plain"]["msamples_s"]

    # channelize |> magnitude: fused in the tensor-core epilogue vs the two kernels in turn.
    if w.channels and "tc_split" in arms:
        extras["channelize_magnitude"] = magnitude_fusion(rfx, w, args, dist, device)

    # The other headline workload (64-channel PFB) in the same run.
    if args.workload == "fir1025" and not args.no_secondary:
        w2 = load_workload("pfb64")
        arms2, _ = measure_arms(rfx, w2, ["tc_split", "plain"], args, dist, device)
        extras["pfb64"] = {k: {kk: vv for kk, vv in v.items() if kk != "seconds"}
                           for k, v in arms2.items()}
        if "plain" in arms2 and len(arms2) > 1:
            first = next(iter(arms2))
            extras["pfb64"]["speedup_vs_plain_fp32"] = (
                arms2[first]["msamples_s"] / arms2["plain"]["msamples_s"])
        del w2

    # End to end through the public host-buffer call, pinned host memory.
    e2e = None
    if rank == 0:
        xp = torch.from_numpy(w.x).pin_memory() if not w.captures else None
        b = rfx.Bench(warmup=args.warmup, runs=args.steps)
        lib = rfx.load()
        if w.captures:
            e2e = batch_e2e(rfx, w, impl, args, device)
        elif w.channels:
            zp = torch.empty(rfx.frames(n, w.channels) * w.channels,
                             dtype=torch.complex64).pin_memory()
            rfx._check(lib.rfx_channelize_host(rfx.parse_chan_impl(impl), xp.data_ptr(), n,
                                               w.taps.ctypes.data, w.taps.size, w.channels,
                                               zp.data_ptr(), rfx.ctypes.byref(b)))
            d2h = zp.numel() * 8
        else:
            e2e = fir_stream_e2e(rfx, w, impl, args)
            extras["e2e_ci16_recording"] = fir_stream_e2e_ci16(rfx, w, impl, args)
        if w.channels:
            step_ms = b.h2d_ms_mean + b.kernel_ms_mean + b.d2h_ms_mean
            e2e = {"value": n / (step_ms / 1e3) / 1e6, "unit": "Msamples/s",
                   "h2d_bytes_per_step": n * 8 + w.taps.size * 4, "d2h_bytes_per_step": d2h,
                   "h2d_ms": b.h2d_ms_mean, "kernel_ms": b.kernel_ms_mean,
                   "d2h_ms": b.d2h_ms_mean}
            # The same through rfx_channelize_host_format over the workload as a ci16
            # recording (components round(v / max|x| * 0.5 * 32767)): half the upload.
            scale = 0.5 * 32767 / float(np.max(np.abs(w.x)))
            c = np.empty(2 * n, dtype="<i2")
            c[0::2] = np.round(w.x.real.astype(np.float64) * scale)
            c[1::2] = np.round(w.x.imag.astype(np.float64) * scale)
            cp = torch.from_numpy(c).pin_memory()
            b2 = rfx.Bench(warmup=args.warmup, runs=args.steps)
            rfx._check(lib.rfx_channelize_host_format(
                rfx.parse_chan_impl(impl), 1, 0, cp.data_ptr(), n, w.taps.ctypes.data,
                w.taps.size, w.channels, zp.data_ptr(), rfx.ctypes.byref(b2)))
            step2 = b2.h2d_ms_mean + b2.kernel_ms_mean + b2.d2h_ms_mean
            extras["e2e_ci16_recording"] = {
                "value": n / (step2 / 1e3) / 1e6, "unit": "Msamples/s",
                "h2d_bytes_per_step": n * 4 + w.taps.size * 4, "d2h_bytes_per_step": d2h,
                "h2d_ms": b2.h2d_ms_mean, "kernel_ms": b2.kernel_ms_mean,
                "d2h_ms": b2.d2h_ms_mean,
                "via": "rfx_channelize_host_format (ci16, converted in the kernel's load stage)"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        if w.captures:
            cpu = cpu_batch_baseline(w.captures)
        elif w.channels:
            cpu = cpu_chan_baseline(w.x, w.taps, w.channels)
        else:
            cpu = cpu_fir_baseline(w.x, w.taps)

    fault = rfx.device_fault()
    if fault:
        raise SystemExit(f"a kernel recorded fault code {fault:#x}")
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Msamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": prim["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": prim["dtype"],
            "data": "synthetic",
            "config": config_of(w, impl, n),
            "max_rel_err_vs_f64": prim["max_rel_err_vs_f64"],
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clocks,
            "gpu_launches": args.steps * prim["launches_per_step"],
            "compare": compare,
            **extras,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="fir1025",
                    choices=["fir1025", "fir63", "pfb64", "pfb1024", "batch256"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the 64-channel PFB measured beside the FIR")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
