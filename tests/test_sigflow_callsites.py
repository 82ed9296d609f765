"""The SigFlow compiler's generated CUDA call sites against this library.

The project's compiler (compiler/src/backend_cuda.cpp) emits C++ programs that include
device_ops.hpp and call fir_device / fir_naive_device (:224-236), fir_batched_device /
fir_naive_batched_device for fused FIR groups (:306-340), channelize_device(cufftHandle, ...)
(:272-277) and magnitude_device, inside a sigflow::Runtime's run(). tests/sigflow/callsites.cu
is a program of that shape (both the fir=tiled_const and the fir=naive forms). Here it is
compiled against gpu-rf-pipeline_gb300/host/device_ops.hpp and linked with librfxhost.a (the
C++ layer) and librfx.so — on the CPU, the build alone — and, on the GPU, run on the project's
fixture signals with its outputs compared with the oracle: the FIRs bit for bit against the
float32 chain of the project's kernels, the channelizers within the project's tolerance
(tests/test_pipeline.py:363-364), the magnitudes against |z| of the channelizer output.
"""
from __future__ import annotations

import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import PKG, ROOT
from oracle import rf_oracle as orc
from rfx import signals

HERE = Path(__file__).resolve().parent
SRC = HERE / "sigflow" / "callsites.cu"


def build_program(out: Path, naive: bool) -> Path:
    import __graft_entry__

    __graft_entry__.build()
    from importlib import util

    spec = util.spec_from_file_location("rfx_build", PKG / "build.py")
    b = util.module_from_spec(spec)
    spec.loader.exec_module(b)
    lib = PKG / "lib"
    cmd = [b.nvcc(), *b.ARCH, "-std=c++17", "-O2", "-I", str(ROOT / "include"),
           "-I", str(PKG / "host"), "-I", str(HERE / "sigflow"),
           f"-DSIGFLOW_FIR_NAIVE={int(naive)}", str(SRC), "-o", str(out),
           "-L", str(lib), "-lrfxhost", "-lrfx", "-lcufft", "-cudart", "shared",
           "-Xlinker", f"-rpath,{lib}", "-Xlinker", f"-rpath,{b.cuda_home() / 'lib64'}"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr
    return out


@pytest.mark.parametrize("naive", [False, True])
def test_generated_call_sites_compile(tmp_path: Path, naive: bool) -> None:
    exe = build_program(tmp_path / "callsites", naive)
    assert exe.exists()


@pytest.mark.gpu
@pytest.mark.parametrize("naive", [False, True])
def test_generated_call_sites_run_and_match_the_oracle(tmp_path: Path, naive: bool) -> None:
    exe = build_program(tmp_path / "callsites", naive)
    fx = tmp_path / "fixtures"
    fx.mkdir()
    (tmp_path / "out").mkdir()
    for name in ["tone", "tone_odd"]:
        signals.fixture_signal(name).astype("<c8").tofile(fx / f"{name}.cf32")
    for name in ["lowpass", "lowpass_long", "channelizer_proto"]:
        signals.fixture_taps(name).astype("<f4").tofile(fx / f"{name}.f32")
    proc = subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True,
                          timeout=300)
    assert proc.returncode == 0, proc.stderr
    report = json.loads(proc.stdout)
    assert report["launches"] == {"channelize": 2, "cufft": 2, "fir": 1, "fir_batched": 1,
                                  "magnitude": 1}

    def read(name, dtype="<c8"):
        return np.fromfile(tmp_path / "out" / name, dtype=dtype)

    tone, tone_odd = signals.fixture_signal("tone"), signals.fixture_signal("tone_odd")
    lowpass, long_ = signals.fixture_taps("lowpass"), signals.fixture_taps("lowpass_long")
    proto = signals.fixture_taps("channelizer_proto")
    for got, want in [(read("fir_a.cf32"), orc.fir_f32_seq(tone, lowpass)),
                      (read("fir_b.cf32"), orc.fir_f32_seq(tone_odd, lowpass)),
                      (read("fir_long.cf32"), orc.fir_f32_seq(tone, long_))]:
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    z16 = read("ch16.cf32").reshape(-1, 16)
    np.testing.assert_allclose(z16, orc.channelize_fast(tone, proto, 16), rtol=1e-5, atol=1e-4)
    np.testing.assert_allclose(read("ch16_mag.f32", "<f4").reshape(-1, 16), orc.magnitude(z16),
                               rtol=1e-6, atol=1e-6)
    z64 = read("ch64.cf32").reshape(-1, 64)
    np.testing.assert_allclose(z64, orc.channelize_fast(tone_odd, long_, 64), rtol=1e-5,
                               atol=1e-4)
