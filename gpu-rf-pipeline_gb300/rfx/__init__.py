"""Python binding of librfx.so (include/rfx.h) through ctypes.

Device buffers are PyTorch CUDA tensors (complex64 for cf32 samples, float32 for taps); the
binding passes their pointers and the current PyTorch stream to the C ABI. There is no CPU
path: if the library is missing, every call raises.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

PKG = Path(__file__).resolve().parents[1]
LIB_PATH = PKG / "lib" / "librfx.so"

RFX_OK = 0
FIR_PLAIN, FIR_TC, FIR_AUTO = 0, 1, 2
CHAN_PLAIN, CHAN_TC, CHAN_AUTO = 0, 1, 2

STATUS_NAMES = {0: "RFX_OK", 1: "RFX_ERR_INVALID", 2: "RFX_ERR_CAPACITY",
                3: "RFX_ERR_ALIGNMENT", 4: "RFX_ERR_CUDA", 5: "RFX_ERR_DEVICE_FAULT"}


class RfxError(RuntimeError):
    def __init__(self, status: int, message: str) -> None:
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class FirCapture(ctypes.Structure):
    _fields_ = [("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("taps", ctypes.c_void_p),
                ("num_samples", ctypes.c_int64), ("num_taps", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class Bench(ctypes.Structure):
    _fields_ = [("warmup", ctypes.c_int), ("runs", ctypes.c_int),
                ("h2d_ms_mean", ctypes.c_double), ("h2d_ms_std", ctypes.c_double),
                ("kernel_ms_mean", ctypes.c_double), ("kernel_ms_std", ctypes.c_double),
                ("d2h_ms_mean", ctypes.c_double), ("d2h_ms_std", ctypes.c_double)]


class StreamConfig(ctypes.Structure):
    _fields_ = [("impl", ctypes.c_int), ("memory", ctypes.c_int), ("chunk", ctypes.c_int64),
                ("depth", ctypes.c_int)]


STREAM_MEMORY = {"copy": 0, "registered": 1, "zero-copy": 2}


# name -> (restype, argtypes); every symbol include/rfx.h declares.
_VP, _I, _I64, _SZ = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_size_t
SIGNATURES = {
    "rfx_last_error": (ctypes.c_char_p, []),
    "rfx_device_fault": (_I, [ctypes.POINTER(ctypes.c_uint)]),
    "rfx_version": (ctypes.c_char_p, []),
    "rfx_fir_impl_name": (_I, [_I, ctypes.c_char_p, _SZ]),
    "rfx_chan_impl_name": (_I, [_I, ctypes.c_char_p, _SZ]),
    "rfx_parse_fir_impl": (_I, [ctypes.c_char_p, ctypes.POINTER(_I)]),
    "rfx_parse_chan_impl": (_I, [ctypes.c_char_p, ctypes.POINTER(_I)]),
    "rfx_fir_launch": (_I, [_I, _VP, _VP, _VP, _I64, _I, _VP]),
    "rfx_fir_launch_format": (_I, [_I, _I, _VP, _VP, _VP, _I64, _I, _VP]),
    "rfx_fir_device": (_I, [_I, _VP, _VP, _VP, _I64, _I]),
    "rfx_fir_impl_used": (_I, [_I, _I, _I64, _I, ctypes.POINTER(_I)]),
    "rfx_fir_load_const_taps": (_I, [_VP, _I, _VP]),
    "rfx_fir_batched_device": (_I, [_I, ctypes.POINTER(_VP), ctypes.POINTER(_VP),
                                    ctypes.POINTER(_I64), _I, _VP, _I, _VP]),
    "rfx_fir_batch_launch": (_I, [_I, ctypes.POINTER(FirCapture), _I, _VP]),
    "rfx_fir_batch_plan_create": (_I, [_I, ctypes.POINTER(FirCapture), _I,
                                       ctypes.POINTER(_VP)]),
    "rfx_fir_batch_run": (_I, [_VP, _VP]),
    "rfx_fir_batch_plan_info": (_I, [_VP, ctypes.POINTER(_I), ctypes.POINTER(_I),
                                     ctypes.POINTER(_I)]),
    "rfx_fir_batch_plan_destroy": (_I, [_VP]),
    "rfx_channelize_frames": (_I64, [_I64, _I]),
    "rfx_chan_plan_create": (_I, [_I, _I, _I64, ctypes.POINTER(_VP)]),
    "rfx_chan_plan_destroy": (_I, [_VP]),
    "rfx_channelize_launch": (_I, [_VP, _VP, _VP, _VP, _I64, _I, _VP]),
    "rfx_channelize_branches": (_I, [_VP, _VP, _VP, _I64, _I, _I, _VP]),
    "rfx_channelize_tc_static": (_I, [_VP, _VP, _VP, _I64, _I, _I, _VP]),
    "rfx_channelize_magnitude_launch": (_I, [_VP, _VP, _VP, _VP, _I64, _I, _VP]),
    "rfx_channelize_launch_format": (_I, [_VP, _I, _I, _VP, _VP, _VP, _I64, _I, _VP]),
    "rfx_magnitude_launch": (_I, [_VP, _VP, _I64, _VP]),
    "rfx_fir_stream": (_I, [_VP, _I64, _VP, _I, ctypes.POINTER(StreamConfig), _VP,
                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I)]),
    "rfx_fir_stream_format": (_I, [_I, _VP, _I64, _VP, _I, ctypes.POINTER(StreamConfig), _VP,
                                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I)]),
    "rfx_fir_host": (_I, [_I, _VP, _I64, _VP, _I, _I, _VP, ctypes.POINTER(Bench)]),
    "rfx_fir_host_format": (_I, [_I, _I, _VP, _I64, _VP, _I, _I, _VP, ctypes.POINTER(Bench)]),
    "rfx_channelize_host": (_I, [_I, _VP, _I64, _VP, _I, _I, _VP, ctypes.POINTER(Bench)]),
    "rfx_channelize_magnitude_host": (_I, [_I, _VP, _I64, _VP, _I, _I, _VP,
                                           ctypes.POINTER(Bench)]),
    "rfx_magnitude_host": (_I, [_VP, _I64, _VP, ctypes.POINTER(Bench)]),
    "rfx_channelize_host_format": (_I, [_I, _I, _I, _VP, _I64, _VP, _I, _I, _VP,
                                        ctypes.POINTER(Bench)]),
    "rfx_autotune_fir": (_I, [_I, _I, _I64, ctypes.POINTER(ctypes.c_double)]),
    "rfx_autotune_channelize": (_I, [_I, _I, _I64, ctypes.POINTER(ctypes.c_double)]),
    "rfx_autotune_clear": (_I, []),
    "rfx_autotune_save": (_I, [ctypes.c_char_p]),
    "rfx_autotune_load": (_I, [ctypes.c_char_p]),
}

_lib = None


def load(path: Path | str | None = None) -> ctypes.CDLL:
    """Loads librfx.so (built by gpu-rf-pipeline_gb300/build.py) and declares its symbols."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RfxError(4, f"{p} is not built: run gpu-rf-pipeline_gb300/build.py")
    lib = ctypes.CDLL(str(p))
    for name, (restype, argtypes) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    if path is None:
        _lib = lib
    return lib


def _check(status: int) -> None:
    if status != RFX_OK:
        raise RfxError(status, load().rfx_last_error().decode())


def _stream_ptr(stream) -> int | None:
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def parse_fir_impl(name: str) -> int:
    out = ctypes.c_int()
    _check(load().rfx_parse_fir_impl(name.encode(), ctypes.byref(out)))
    return out.value


def fir_impl_used(impl, num_taps: int, num_samples: int, batch: bool = False) -> str:
    """Name of the kernel ("plain" or "tc_split") a FIR call with these arguments runs
    (rfx_fir_impl_used): auto resolved, and tc_split's hand-offs to the plain kernel shown."""
    out = ctypes.c_int()
    _check(load().rfx_fir_impl_used(_impl(impl), int(num_taps), int(num_samples), int(batch),
                                    ctypes.byref(out)))
    return "tc_split" if out.value == FIR_TC else "plain"


def parse_chan_impl(name: str) -> int:
    out = ctypes.c_int()
    _check(load().rfx_parse_chan_impl(name.encode(), ctypes.byref(out)))
    return out.value


def fir_impl_names() -> list[str]:
    names, buf, i = [], ctypes.create_string_buffer(64), 0
    while load().rfx_fir_impl_name(i, buf, 64) == RFX_OK:
        names.append(buf.value.decode())
        i += 1
    return names


def chan_impl_names() -> list[str]:
    names, buf, i = [], ctypes.create_string_buffer(64), 0
    while load().rfx_chan_impl_name(i, buf, 64) == RFX_OK:
        names.append(buf.value.decode())
        i += 1
    return names


def _impl(impl) -> int:
    return parse_fir_impl(impl) if isinstance(impl, str) else int(impl)


def fir_launch(impl, x, taps, y, stream=None, num_samples: int | None = None) -> None:
    """y[:n] = FIR(x[:n], taps) on the GPU; x, y complex64 CUDA tensors, taps float32."""
    n = x.numel() if num_samples is None else int(num_samples)
    _check(load().rfx_fir_launch(_impl(impl), x.data_ptr(), taps.data_ptr(), y.data_ptr(), n,
                                 taps.numel(), _stream_ptr(stream)))


# rfx_sample_format: the stored forms of an input (SigMF cf32_le, ci16_le, ci8).
SAMPLE_FORMATS = {"cf32": 0, "ci16": 1, "ci8": 2}
_COMPONENT_BYTES = {"cf32": 4, "ci16": 2, "ci8": 1}


def _format(fmt) -> int:
    if isinstance(fmt, str):
        if fmt not in SAMPLE_FORMATS:
            raise ValueError(f"unknown sample format {fmt!r} (cf32, ci16, ci8)")
        return SAMPLE_FORMATS[fmt]
    return int(fmt)


def fir_launch_format(impl, fmt, x, taps, y, stream=None, num_samples: int | None = None) -> None:
    """y[:n] = FIR(x[:n] converted from `fmt`, taps): x a CUDA tensor of interleaved I/Q
    components as stored (int16 for ci16, int8 for ci8, float32 or complex64 for cf32), y
    complex64. The conversion happens in the kernels' load stage."""
    name = fmt if isinstance(fmt, str) else {v: k for k, v in SAMPLE_FORMATS.items()}[int(fmt)]
    n = (x.numel() * x.element_size() // (2 * _COMPONENT_BYTES[name]) if num_samples is None
         else int(num_samples))
    _check(load().rfx_fir_launch_format(_impl(impl), _format(fmt), x.data_ptr(), taps.data_ptr(),
                                        y.data_ptr(), n, taps.numel(), _stream_ptr(stream)))


def fir_format(x, taps, fmt, impl="plain", stream=None):
    """Returns a new complex64 CUDA tensor with the FIR of stored samples x (see
    fir_launch_format)."""
    import torch

    name = fmt if isinstance(fmt, str) else {v: k for k, v in SAMPLE_FORMATS.items()}[int(fmt)]
    n = x.numel() * x.element_size() // (2 * _COMPONENT_BYTES[name])
    y = torch.empty(n, dtype=torch.complex64, device=x.device)
    fir_launch_format(impl, fmt, x, taps, y, stream, n)
    return y


def fir(x, taps, impl="plain", stream=None):
    """Returns a new complex64 CUDA tensor with the FIR of x."""
    import torch

    y = torch.empty_like(x)
    fir_launch(impl, x, taps, y, stream)
    return y


def fir_batched(x_list, y_list, taps, impl="plain", stream=None) -> None:
    """Several captures sharing one tap set in one launch."""
    count = len(x_list)
    xs = (ctypes.c_void_p * count)(*[t.data_ptr() for t in x_list])
    ys = (ctypes.c_void_p * count)(*[t.data_ptr() for t in y_list])
    ns = (ctypes.c_int64 * count)(*[t.numel() for t in x_list])
    _check(load().rfx_fir_batched_device(_impl(impl), xs, ys, ns, count, taps.data_ptr(),
                                         taps.numel(), _stream_ptr(stream)))


def fir_batch(captures, impl="plain", stream=None) -> None:
    """captures: list of (x, y, taps) CUDA tensors, each capture with its own taps."""
    arr = (FirCapture * len(captures))()
    for i, (x, y, taps) in enumerate(captures):
        arr[i] = FirCapture(x.data_ptr(), y.data_ptr(), taps.data_ptr(), x.numel(),
                            taps.numel(), 0)
    _check(load().rfx_fir_batch_launch(_impl(impl), arr, len(captures), _stream_ptr(stream)))


class FirBatchPlan:
    """rfx_fir_batch_plan: a batch of (x, y, taps) device tensors (cf32, cf32, float32), each
    capture with its own taps, run by ONE persistent launch per run(). The tensors must stay
    alive while the plan is used."""

    def __init__(self, captures, impl="auto") -> None:
        self._p = ctypes.c_void_p()
        self.count = len(captures)
        arr = (FirCapture * self.count)()
        for i, (x, y, taps) in enumerate(captures):
            arr[i] = FirCapture(x.data_ptr(), y.data_ptr(), taps.data_ptr(), x.numel(),
                                taps.numel(), 0)
        self._arr = arr
        _check(load().rfx_fir_batch_plan_create(_impl(impl), arr, self.count,
                                                ctypes.byref(self._p)))

    def run(self, stream=None) -> None:
        _check(load().rfx_fir_batch_run(self._p, _stream_ptr(stream)))

    def info(self) -> dict:
        tc, plain, launches = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(load().rfx_fir_batch_plan_info(self._p, ctypes.byref(tc), ctypes.byref(plain),
                                              ctypes.byref(launches)))
        return {"tc_captures": tc.value, "plain_captures": plain.value,
                "launches": launches.value}

    def close(self) -> None:
        if self._p:
            load().rfx_fir_batch_plan_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __enter__(self) -> "FirBatchPlan":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass


class ChanPlan:
    """A channelizer plan (rfx_chan_plan_create); close() or use as a context manager."""

    def __init__(self, channels: int, max_samples: int, impl="plain") -> None:
        self.channels = channels
        impl_v = parse_chan_impl(impl) if isinstance(impl, str) else int(impl)
        handle = ctypes.c_void_p()
        _check(load().rfx_chan_plan_create(impl_v, channels, max_samples, ctypes.byref(handle)))
        self.handle = handle

    def launch(self, x, taps, out, stream=None, num_samples: int | None = None) -> None:
        n = x.numel() if num_samples is None else int(num_samples)
        _check(load().rfx_channelize_launch(self.handle, x.data_ptr(), taps.data_ptr(),
                                            out.data_ptr(), n, taps.numel(),
                                            _stream_ptr(stream)))

    def launch_magnitude(self, x, taps, mag, stream=None, num_samples: int | None = None) -> None:
        """mag[t][k] = |z[t][k]|: float32 (frames, channels)."""
        n = x.numel() if num_samples is None else int(num_samples)
        _check(load().rfx_channelize_magnitude_launch(self.handle, x.data_ptr(), taps.data_ptr(),
                                                      mag.data_ptr(), n, taps.numel(),
                                                      _stream_ptr(stream)))

    def launch_format(self, fmt, x, taps, out, magnitude: bool = False, stream=None,
                      num_samples: int | None = None) -> None:
        """The channelizer over x stored in `fmt` (cf32 / ci16 / ci8 components), converted
        where the kernels read it; out: complex64 z, or float32 |z| with `magnitude`."""
        n = (x.numel() * x.element_size() // (2 * _COMPONENT_BYTES[fmt]) if num_samples is None
             else int(num_samples))
        _check(load().rfx_channelize_launch_format(self.handle, _format(fmt), 1 if magnitude else 0,
                                                   x.data_ptr(), taps.data_ptr(), out.data_ptr(),
                                                   n, taps.numel(), _stream_ptr(stream)))

    def close(self) -> None:
        if self.handle:
            _check(load().rfx_chan_plan_destroy(self.handle))
            self.handle = ctypes.c_void_p()

    def __enter__(self) -> "ChanPlan":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass


def frames(num_samples: int, channels: int) -> int:
    return int(load().rfx_channelize_frames(num_samples, channels))


def channelize(x, taps, channels: int, impl="plain", stream=None):
    """Returns a (frames, channels) complex64 CUDA tensor."""
    import torch

    f = frames(x.numel(), channels)
    out = torch.empty((f, channels), dtype=torch.complex64, device=x.device)
    with ChanPlan(channels, x.numel(), impl) as plan:
        plan.launch(x, taps, out, stream)
        torch.cuda.current_stream().synchronize()
    return out


def channelize_magnitude(x, taps, channels: int, impl="plain", stream=None):
    """Returns the (frames, channels) float32 CUDA tensor |channelize(x)|."""
    import torch

    f = frames(x.numel(), channels)
    mag = torch.empty((f, channels), dtype=torch.float32, device=x.device)
    with ChanPlan(channels, x.numel(), impl) as plan:
        plan.launch_magnitude(x, taps, mag, stream)
        torch.cuda.current_stream().synchronize()
    return mag


def channelize_format(x, taps, channels: int, fmt: str, impl="plain", magnitude: bool = False,
                      stream=None):
    """The channelizer of stored samples x (CUDA tensor of cf32 / int16 / int8 components):
    a (frames, channels) complex64 tensor, or float32 |z| with `magnitude`."""
    import torch

    n = x.numel() * x.element_size() // (2 * _COMPONENT_BYTES[fmt])
    f = frames(n, channels)
    out = torch.empty((f, channels), dtype=torch.float32 if magnitude else torch.complex64,
                      device=x.device)
    with ChanPlan(channels, n, impl) as plan:
        plan.launch_format(fmt, x, taps, out, magnitude, stream, n)
        torch.cuda.current_stream().synchronize()
    return out


def magnitude_launch(x, mag, stream=None, num_samples: int | None = None) -> None:
    """mag[:n] = |x[:n]| on the GPU: x complex64, mag float32 CUDA tensors."""
    n = x.numel() if num_samples is None else int(num_samples)
    _check(load().rfx_magnitude_launch(x.data_ptr(), mag.data_ptr(), n, _stream_ptr(stream)))


def magnitude(x, stream=None):
    """Returns a new float32 CUDA tensor |x| of x's shape."""
    import torch

    mag = torch.empty(x.shape, dtype=torch.float32, device=x.device)
    magnitude_launch(x, mag, stream)
    return mag


def channelize_branches(x, taps, channels: int, stream=None):
    """The float32 branch sums u (frames, channels) of the channelizer, complex64 CUDA tensor."""
    import torch

    f = frames(x.numel(), channels)
    u = torch.empty((f, channels), dtype=torch.complex64, device=x.device)
    _check(load().rfx_channelize_branches(x.data_ptr(), taps.data_ptr(), u.data_ptr(), x.numel(),
                                          channels, taps.numel(), _stream_ptr(stream)))
    return u


def device_fault() -> int:
    code = ctypes.c_uint()
    _check(load().rfx_device_fault(ctypes.byref(code)))
    return code.value


def fir_host(impl, x, taps, block: int = 256, warmup: int = 0, runs: int = 1):
    """The FIR on host NumPy arrays (complex64 x, float32 taps), timed like the project's
    Bench. Returns (y, Bench)."""
    import numpy as np

    x = np.ascontiguousarray(x, dtype=np.complex64)
    taps = np.ascontiguousarray(taps, dtype=np.float32)
    y = np.empty_like(x)
    b = Bench(warmup=warmup, runs=runs)
    _check(load().rfx_fir_host(_impl(impl), x.ctypes.data, x.size, taps.ctypes.data, taps.size,
                               block, y.ctypes.data, ctypes.byref(b)))
    return y, b


def channelize_host(impl, x, taps, channels: int, warmup: int = 0, runs: int = 1):
    """The channelizer on host NumPy arrays. Returns ((frames, channels) complex64, Bench)."""
    import numpy as np

    x = np.ascontiguousarray(x, dtype=np.complex64)
    taps = np.ascontiguousarray(taps, dtype=np.float32)
    f = frames(x.size, channels)
    z = np.empty(f * channels, dtype=np.complex64)
    impl_v = parse_chan_impl(impl) if isinstance(impl, str) else int(impl)
    b = Bench(warmup=warmup, runs=runs)
    _check(load().rfx_channelize_host(impl_v, x.ctypes.data, x.size, taps.ctypes.data,
                                      taps.size, channels, z.ctypes.data, ctypes.byref(b)))
    return z.reshape(f, channels), b


def channelize_magnitude_host(impl, x, taps, channels: int, warmup: int = 0, runs: int = 1):
    """|channelize| on host NumPy arrays. Returns ((frames, channels) float32, Bench)."""
    import numpy as np

    x = np.ascontiguousarray(x, dtype=np.complex64)
    taps = np.ascontiguousarray(taps, dtype=np.float32)
    f = frames(x.size, channels)
    mag = np.empty(f * channels, dtype=np.float32)
    impl_v = parse_chan_impl(impl) if isinstance(impl, str) else int(impl)
    b = Bench(warmup=warmup, runs=runs)
    _check(load().rfx_channelize_magnitude_host(impl_v, x.ctypes.data, x.size, taps.ctypes.data,
                                                taps.size, channels, mag.ctypes.data,
                                                ctypes.byref(b)))
    return mag.reshape(f, channels), b


def magnitude_host(x, warmup: int = 0, runs: int = 1):
    """|x| on a host NumPy array (complex64). Returns (float32 array, Bench)."""
    import numpy as np

    x = np.ascontiguousarray(x, dtype=np.complex64)
    mag = np.empty(x.shape, dtype=np.float32)
    b = Bench(warmup=warmup, runs=runs)
    _check(load().rfx_magnitude_host(x.ctypes.data, x.size, mag.ctypes.data, ctypes.byref(b)))
    return mag, b


def fir_stream(x, taps, impl="plain", chunk: int = 1 << 20, depth: int = 3,
               memory: str = "copy", out=None, fmt: str = "cf32"):
    """The streamed FIR of a host capture (numpy array or CPU tensor; pinned tensors are used
    in place in "registered" mode). cf32: complex64 samples; ci16 / ci8: the interleaved integer
    components as stored (int16 / int8), converted on the GPU. Returns (y complex64, total_ms,
    chunks)."""
    import numpy as np

    comp = _COMPONENT_BYTES[fmt]
    if hasattr(x, "data_ptr"):
        x_ptr = x.data_ptr()
        n = x.numel() * x.element_size() // (2 * comp)
        if out is not None:
            y = out
        else:
            import torch

            y = torch.empty(n, dtype=torch.complex64, pin_memory=x.is_pinned())
        y_ptr = y.data_ptr()
    else:
        dtype = {"cf32": np.complex64, "ci16": np.dtype("<i2"), "ci8": np.int8}[fmt]
        x = np.ascontiguousarray(x, dtype=dtype)
        x_ptr = x.ctypes.data
        n = x.nbytes // (2 * comp)
        y = out if out is not None else np.empty(n, dtype=np.complex64)
        y_ptr = y.ctypes.data if not hasattr(y, "data_ptr") else y.data_ptr()
    taps = np.ascontiguousarray(taps, dtype=np.float32)
    cfg = StreamConfig(_impl(impl), STREAM_MEMORY[memory], chunk, depth)
    ms = ctypes.c_double()
    chunks = ctypes.c_int()
    _check(load().rfx_fir_stream_format(_format(fmt), x_ptr, n, taps.ctypes.data, taps.size,
                                        ctypes.byref(cfg), y_ptr, ctypes.byref(ms),
                                        ctypes.byref(chunks)))
    return y, ms.value, chunks.value


def autotune_fir(impl, num_taps: int, num_samples: int) -> float:
    ms = ctypes.c_double()
    _check(load().rfx_autotune_fir(_impl(impl), num_taps, num_samples, ctypes.byref(ms)))
    return ms.value


def autotune_channelize(channels: int, num_taps: int, num_samples: int) -> float:
    ms = ctypes.c_double()
    _check(load().rfx_autotune_channelize(channels, num_taps, num_samples, ctypes.byref(ms)))
    return ms.value


def autotune_clear() -> None:
    _check(load().rfx_autotune_clear())


def autotune_save(path) -> None:
    _check(load().rfx_autotune_save(str(path).encode()))


def autotune_load(path) -> None:
    _check(load().rfx_autotune_load(str(path).encode()))
