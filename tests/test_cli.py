"""The rfgpu command-line tool, tested the way the project tests its own (tests/test_pipeline.py):
the binary runs as a subprocess on fixture files and its output files are compared with the
oracle. Usage errors (exit 2) need no GPU; everything that computes is marked gpu."""
from __future__ import annotations

import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import PKG
from oracle import rf_oracle as orc
from rfx import signals

RFGPU = PKG / "bin" / "rfgpu"
FIR_RTOL = 1e-5          # tests/test_pipeline.py:116-117
FIR_ATOL = 1e-5
CHANNELIZE_RTOL = 1e-5   # tests/test_pipeline.py:363-364
CHANNELIZE_ATOL = 1e-4


@pytest.fixture(scope="session")
def fixtures(tmp_path_factory) -> Path:
    if not RFGPU.exists():
        import __graft_entry__

        __graft_entry__.build()
    d = tmp_path_factory.mktemp("fixtures")
    for name in ["tone", "tone_odd", "short", "zeros"]:
        signals.fixture_signal(name).astype("<c8").tofile(d / f"{name}.cf32")
    for name in ["lowpass", "lowpass_long", "channelizer_proto", "identity"]:
        signals.fixture_taps(name).astype("<f4").tofile(d / f"{name}.f32")
    # SigMF recordings: the project's ci16 fixture, the same signal in ci8, and the converted
    # ci16 samples as a plain .cf32 file for byte comparisons.
    signals.write_sigmf(d / "tone_ci16", signals.tone_ci16(), "ci16_le")
    signals.write_sigmf(d / "tone_ci8", tone_ci8(), "ci8")
    signals.fixture_signal("tone_ci16").astype("<c8").tofile(d / "tone_ci16.cf32")
    orc.decode(tone_ci8(), "ci8").astype("<c8").tofile(d / "tone_ci8.cf32")
    return d


def tone_ci8() -> np.ndarray:
    """The ci16 fixture's signal at 8 bits: components round(v / 256), int8."""
    return np.round(signals.tone_ci16().astype(np.float64) / 256).astype(np.int8)


def rfgpu(*args, check: bool = True) -> subprocess.CompletedProcess:
    proc = subprocess.run([str(RFGPU), *map(str, args)], capture_output=True, text=True,
                          timeout=300)
    if check:
        assert proc.returncode == 0, f"rfgpu {' '.join(map(str, args))}\n{proc.stderr}"
    return proc


def read_cf32(path: Path) -> np.ndarray:
    return np.fromfile(path, dtype="<c8")


# --- usage errors: no GPU needed -------------------------------------------------------------

def test_help_lists_every_implementation() -> None:
    if not RFGPU.exists():
        import __graft_entry__

        __graft_entry__.build()
    proc = rfgpu("--help")
    for name in ["plain", "tc_split", "auto", "naive", "register"]:
        assert f"--impl {name}" in proc.stderr


def test_unknown_impl_is_a_usage_error(fixtures: Path, tmp_path: Path) -> None:
    proc = rfgpu("fir", "--in", fixtures / "tone.cf32", "--taps", fixtures / "lowpass.f32",
                 "--out", tmp_path / "y.cf32", "--impl", "no_such_impl", check=False)
    assert proc.returncode == 2
    assert "no_such_impl" in proc.stderr
    assert not (tmp_path / "y.cf32").exists()


@pytest.mark.parametrize("block", ["0", "48", "2048", "abc"])
def test_bad_block_size_is_a_usage_error(fixtures: Path, tmp_path: Path, block: str) -> None:
    proc = rfgpu("fir", "--in", fixtures / "tone.cf32", "--taps", fixtures / "lowpass.f32",
                 "--out", tmp_path / "y.cf32", "--block", block, check=False)
    assert proc.returncode == 2
    assert "--block" in proc.stderr


@pytest.mark.parametrize("args", [["--channels", "0"], ["--channels", "x"], []])
def test_bad_channel_count_is_a_usage_error(fixtures: Path, tmp_path: Path, args) -> None:
    proc = rfgpu("channelize", "--in", fixtures / "tone.cf32", "--taps",
                 fixtures / "channelizer_proto.f32", "--out", tmp_path / "z.cf32", *args,
                 check=False)
    assert proc.returncode == 2


def test_unknown_option_and_subcommand_are_usage_errors(tmp_path: Path) -> None:
    assert rfgpu("fir", "--nope", "1", check=False).returncode == 2
    assert rfgpu("spectrum_of_everything", check=False).returncode == 2
    assert rfgpu("fir", "--in", "a", "--in", "b", check=False).returncode == 2


# --- numerics: GPU ------------------------------------------------------------------------------

@pytest.fixture(scope="module")
def info() -> dict:
    return json.loads(rfgpu("info").stdout)


@pytest.mark.gpu
def test_info_reports_the_device_and_impls(info: dict) -> None:
    assert info["compute_capability"] == "10.3"
    assert info["impls"]["fir"][0] == "plain"
    assert "tc_split" in info["impls"]["fir"] and "tc_split" in info["impls"]["channelize"]


FIR_IMPLS = ["plain", "tc_split", "auto", "naive", "tiled", "tiled_const", "register"]


@pytest.mark.gpu
@pytest.mark.parametrize("impl", FIR_IMPLS)
@pytest.mark.parametrize("name,taps", [("tone", "lowpass"), ("tone", "lowpass_long"),
                                       ("tone_odd", "lowpass"), ("tone_odd", "lowpass_long"),
                                       ("short", "lowpass"), ("short", "lowpass_long")])
def test_fir_matches_reference(fixtures: Path, tmp_path: Path, impl: str, name: str,
                               taps: str) -> None:
    out = tmp_path / "fir.cf32"
    rfgpu("fir", "--in", fixtures / f"{name}.cf32", "--taps", fixtures / f"{taps}.f32",
          "--out", out, "--impl", impl)
    expected = orc.fir_fast(signals.fixture_signal(name), signals.fixture_taps(taps))
    actual = read_cf32(out)
    assert actual.shape == expected.shape
    np.testing.assert_allclose(actual, expected, rtol=FIR_RTOL, atol=FIR_ATOL)


@pytest.mark.gpu
@pytest.mark.parametrize("impl", FIR_IMPLS)
@pytest.mark.parametrize("block", [32, 96, 1024])
def test_fir_block_size_does_not_change_the_result(fixtures: Path, tmp_path: Path, impl: str,
                                                   block: int) -> None:
    out = tmp_path / "fir.cf32"
    rfgpu("fir", "--in", fixtures / "tone_odd.cf32", "--taps", fixtures / "lowpass_long.f32",
          "--out", out, "--impl", impl, "--block", block)
    expected = orc.fir_fast(signals.fixture_signal("tone_odd"),
                            signals.fixture_taps("lowpass_long"))
    np.testing.assert_allclose(read_cf32(out), expected, rtol=FIR_RTOL, atol=FIR_ATOL)


@pytest.mark.gpu
@pytest.mark.parametrize("impl", FIR_IMPLS)
@pytest.mark.parametrize("name", ["tone", "tone_odd", "short"])
def test_fir_identity_returns_the_input_exactly(fixtures: Path, tmp_path: Path, impl: str,
                                                name: str) -> None:
    out = tmp_path / "fir.cf32"
    rfgpu("fir", "--in", fixtures / f"{name}.cf32", "--taps", fixtures / "identity.f32",
          "--out", out, "--impl", impl)
    assert out.read_bytes() == (fixtures / f"{name}.cf32").read_bytes()


@pytest.mark.gpu
@pytest.mark.parametrize("impl", FIR_IMPLS)
@pytest.mark.parametrize("taps", ["lowpass", "lowpass_long", "identity"])
def test_fir_of_zeros_is_exactly_zero(fixtures: Path, tmp_path: Path, impl: str,
                                      taps: str) -> None:
    out = tmp_path / "fir.cf32"
    rfgpu("fir", "--in", fixtures / "zeros.cf32", "--taps", fixtures / f"{taps}.f32",
          "--out", out, "--impl", impl)
    actual = read_cf32(out)
    assert actual.shape == (4096,) and not np.any(actual)


@pytest.mark.gpu
def test_project_names_give_identical_bytes(fixtures: Path, tmp_path: Path) -> None:
    outs = []
    for impl in ["plain", "naive", "tiled", "tiled_const", "register"]:
        out = tmp_path / f"{impl}.cf32"
        rfgpu("fir", "--in", fixtures / "tone.cf32", "--taps", fixtures / "lowpass_long.f32",
              "--out", out, "--impl", impl)
        outs.append(out.read_bytes())
    assert all(o == outs[0] for o in outs)
    want = orc.fir_f32_seq(signals.fixture_signal("tone"), signals.fixture_taps("lowpass_long"))
    assert outs[0] == want.astype("<c8").tobytes()


@pytest.mark.gpu
def test_bench_reports_each_phase(fixtures: Path, tmp_path: Path, info: dict) -> None:
    proc = rfgpu("fir", "--in", fixtures / "tone.cf32", "--taps", fixtures / "lowpass.f32",
                 "--out", tmp_path / "y.cf32", "--bench", 10, "--warmup", 2)
    report = json.loads(proc.stdout)
    assert report["op"] == "fir" and report["runs"] == 10 and report["warmup"] == 2
    assert report["gpu"] == info["gpu"]
    for phase in ("h2d_ms", "kernel_ms", "d2h_ms"):
        assert report[phase]["mean"] > 0 and report[phase]["std"] >= 0


@pytest.mark.gpu
def test_bench_does_not_change_the_output(fixtures: Path, tmp_path: Path) -> None:
    args = ["--in", fixtures / "tone_odd.cf32", "--taps", fixtures / "lowpass_long.f32",
            "--impl", "tc_split"]
    rfgpu("fir", *args, "--out", tmp_path / "once.cf32")
    rfgpu("fir", *args, "--out", tmp_path / "bench.cf32", "--bench", 10)
    assert (tmp_path / "once.cf32").read_bytes() == (tmp_path / "bench.cf32").read_bytes()


@pytest.mark.gpu
def test_missing_input_file_is_a_runtime_error(fixtures: Path, tmp_path: Path) -> None:
    proc = rfgpu("fir", "--in", tmp_path / "missing.cf32", "--taps", fixtures / "lowpass.f32",
                 "--out", tmp_path / "y.cf32", check=False)
    assert proc.returncode == 1
    assert "missing.cf32" in proc.stderr


@pytest.mark.gpu
def test_truncated_cf32_is_rejected(fixtures: Path, tmp_path: Path) -> None:
    np.zeros(3, dtype="<f4").tofile(tmp_path / "bad.cf32")
    proc = rfgpu("fir", "--in", tmp_path / "bad.cf32", "--taps", fixtures / "lowpass.f32",
                 "--out", tmp_path / "y.cf32", check=False)
    assert proc.returncode == 1
    assert "bad.cf32" in proc.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("impl", ["plain", "auto"])
@pytest.mark.parametrize("name,taps,channels", [
    ("tone", "channelizer_proto", 16),
    ("tone_odd", "channelizer_proto", 16),   # partial last frame
    ("tone", "lowpass_long", 64),            # taps not a multiple of M
    ("short", "lowpass", 4),                 # input shorter than the filter
    ("tone_odd", "identity", 1),             # one channel, one tap: the input itself
])
def test_channelize_matches_reference(fixtures: Path, tmp_path: Path, impl: str, name: str,
                                      taps: str, channels: int) -> None:
    out = tmp_path / "ch.cf32"
    rfgpu("channelize", "--in", fixtures / f"{name}.cf32", "--taps", fixtures / f"{taps}.f32",
          "--channels", channels, "--out", out, "--impl", impl)
    expected = orc.channelize_fast(signals.fixture_signal(name), signals.fixture_taps(taps),
                                   channels).ravel()
    actual = read_cf32(out)
    assert actual.shape == expected.shape
    np.testing.assert_allclose(actual, expected, rtol=CHANNELIZE_RTOL, atol=CHANNELIZE_ATOL)


@pytest.mark.gpu
def test_channelize_tc_on_sixty_four_channels(fixtures: Path, tmp_path: Path) -> None:
    out = tmp_path / "ch.cf32"
    rfgpu("channelize", "--in", fixtures / "tone.cf32", "--taps", fixtures / "lowpass_long.f32",
          "--channels", 64, "--out", out, "--impl", "tc_split")
    expected = orc.channelize_fast(signals.fixture_signal("tone"),
                                   signals.fixture_taps("lowpass_long"), 64).ravel()
    np.testing.assert_allclose(read_cf32(out), expected, rtol=CHANNELIZE_RTOL,
                               atol=CHANNELIZE_ATOL)


@pytest.mark.gpu
@pytest.mark.parametrize("output", ["complex", "magnitude"])
def test_channelize_tc_on_1024_channels(tmp_path: Path, output: str) -> None:
    # The wideband form (branch sums, then the 32 x 32 factored tensor-core DFT) through the CLI.
    w = signals.channelizer1024(1 << 18)
    w.x.astype("<c8").tofile(tmp_path / "x.cf32")
    w.taps.astype("<f4").tofile(tmp_path / "h.f32")
    out = tmp_path / "ch.out"
    rfgpu("channelize", "--in", tmp_path / "x.cf32", "--taps", tmp_path / "h.f32",
          "--channels", 1024, "--out", out, "--impl", "tc_split", "--output", output)
    ref = orc.channelize_fast(w.x, w.taps, 1024)
    if output == "complex":
        assert orc.normwise_error(read_cf32(out).reshape(-1, 1024), ref) <= 2e-6
    else:
        mag = np.fromfile(out, dtype="<f4").reshape(-1, 1024)
        assert orc.normwise_error(mag, np.abs(ref)) <= 2e-6


@pytest.mark.gpu
def test_channelize_puts_a_tone_in_its_channel(fixtures: Path, tmp_path: Path) -> None:
    n = np.arange(16 * 512)
    signals.to_cf32(np.exp(2j * np.pi * 3 * n / 16)).astype("<c8").tofile(tmp_path / "x.cf32")
    rfgpu("channelize", "--in", tmp_path / "x.cf32", "--taps",
          fixtures / "channelizer_proto.f32", "--channels", 16, "--out", tmp_path / "ch.cf32")
    z = read_cf32(tmp_path / "ch.cf32").reshape(-1, 16)[16:]
    power = np.mean(np.abs(z) ** 2, axis=0)
    assert np.argmax(power) == 3
    assert power[3] > 1000 * np.max(np.delete(power, 3))
    np.testing.assert_allclose(np.abs(z[:, 3]), 1.0, atol=0.02)


# --- stream ----------------------------------------------------------------------------------

@pytest.mark.parametrize("args", [["--chunk", "0"], ["--depth", "0"], ["--memory", "disk"]])
def test_bad_stream_options_are_usage_errors(fixtures: Path, tmp_path: Path, args) -> None:
    proc = rfgpu("stream", "--in", fixtures / "tone.cf32", "--taps", fixtures / "lowpass.f32",
                 "--out", tmp_path / "y.cf32", *args, check=False)
    assert proc.returncode == 2


@pytest.mark.gpu
@pytest.mark.parametrize("impl", ["tiled", "tc_split", "auto"])
@pytest.mark.parametrize("chunk,depth", [(1000, 3), (4096, 2), (100000, 1)])
@pytest.mark.parametrize("memory", ["copy", "registered", "zero-copy"])
def test_stream_matches_fir_exactly(fixtures: Path, tmp_path: Path, impl: str, chunk: int,
                                    depth: int, memory: str) -> None:
    rfgpu("fir", "--in", fixtures / "tone.cf32", "--taps", fixtures / "lowpass_long.f32",
          "--out", tmp_path / "fir.cf32", "--impl", impl)
    rfgpu("stream", "--in", fixtures / "tone.cf32", "--taps", fixtures / "lowpass_long.f32",
          "--out", tmp_path / "stream.cf32", "--impl", impl, "--chunk", chunk, "--depth", depth,
          "--memory", memory)
    assert (tmp_path / "fir.cf32").read_bytes() == (tmp_path / "stream.cf32").read_bytes()


@pytest.mark.gpu
def test_stream_of_short_input(fixtures: Path, tmp_path: Path) -> None:
    rfgpu("stream", "--in", fixtures / "short.cf32", "--taps", fixtures / "lowpass.f32",
          "--out", tmp_path / "y.cf32", "--chunk", 3)
    expected = orc.fir_fast(signals.fixture_signal("short"), signals.fixture_taps("lowpass"))
    np.testing.assert_allclose(read_cf32(tmp_path / "y.cf32"), expected, rtol=FIR_RTOL,
                               atol=FIR_ATOL)


@pytest.mark.gpu
def test_stream_bench_reports_throughput_against_the_sample_rate(fixtures: Path,
                                                                  tmp_path: Path) -> None:
    data = tmp_path / "tone.cf32"
    data.write_bytes((fixtures / "tone.cf32").read_bytes())
    (tmp_path / "tone.json").write_text(json.dumps({"sample_rate": 2.4e6}))
    proc = rfgpu("stream", "--in", data, "--taps", fixtures / "lowpass.f32",
                 "--out", tmp_path / "y.cf32", "--chunk", 8192, "--bench", 10)
    report = json.loads(proc.stdout)
    assert report["op"] == "stream" and report["chunks"] == 8 and report["runs"] == 10
    assert report["sample_rate"] == 2.4e6
    assert report["msps"] > 0
    assert report["realtime_factor"] == pytest.approx(report["msps"] * 1e6 / 2.4e6, rel=1e-3)


# --- SigMF recordings (tests/test_pipeline.py:272-307) ------------------------------------------
# Every input may be a SigMF pair named by either file. `fir` uploads integer recordings as
# stored and converts them on the GPU; the result must be the bytes of the FIR of the samples
# converted on the host (the project's read path), for every implementation.

@pytest.mark.parametrize("command", ["fir", "channelize", "stream"])
@pytest.mark.parametrize("meta,message", [
    ({"core:datatype": "cf64_le"}, "cf64_le"),
    ({"core:datatype": "ci16_le", "core:num_channels": 2}, "channels"),
])
def test_unsupported_sigmf_is_a_runtime_error(tmp_path: Path, fixtures: Path, command: str,
                                              meta: dict, message: str) -> None:
    (tmp_path / "rec.sigmf-meta").write_text(json.dumps({"global": meta}))
    (tmp_path / "rec.sigmf-data").write_bytes(bytes(16))
    extra = ["--channels", "4"] if command == "channelize" else []
    proc = rfgpu(command, "--in", tmp_path / "rec.sigmf-meta", "--taps", fixtures / "lowpass.f32",
                 "--out", tmp_path / "y.cf32", *extra, check=False)
    assert proc.returncode == 1
    assert message in proc.stderr


def test_sigmf_with_a_partial_sample_is_a_runtime_error(tmp_path: Path, fixtures: Path) -> None:
    (tmp_path / "rec.sigmf-meta").write_text(json.dumps({"global": {"core:datatype": "ci16_le"}}))
    (tmp_path / "rec.sigmf-data").write_bytes(bytes(6))  # one and a half ci16 samples
    proc = rfgpu("fir", "--in", tmp_path / "rec.sigmf-data", "--taps", fixtures / "lowpass.f32",
                 "--out", tmp_path / "y.cf32", check=False)
    assert proc.returncode == 1
    assert "rec.sigmf-data" in proc.stderr


def test_sigmf_without_its_data_file_is_a_runtime_error(tmp_path: Path, fixtures: Path) -> None:
    (tmp_path / "rec.sigmf-meta").write_text(json.dumps({"global": {"core:datatype": "ci8"}}))
    proc = rfgpu("fir", "--in", tmp_path / "rec.sigmf-meta", "--taps", fixtures / "lowpass.f32",
                 "--out", tmp_path / "y.cf32", check=False)
    assert proc.returncode == 1
    assert "rec.sigmf-data" in proc.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("suffix", [".sigmf-meta", ".sigmf-data"])  # either file of the pair
@pytest.mark.parametrize("impl", ["plain", "tc_split", "auto"])
def test_sigmf_ci16_reads_as_scaled_cf32(fixtures: Path, tmp_path: Path, suffix: str,
                                         impl: str) -> None:
    out = tmp_path / "fir.cf32"
    rfgpu("fir", "--in", fixtures / f"tone_ci16{suffix}", "--taps", fixtures / "identity.f32",
          "--out", out, "--impl", impl)
    raw = signals.tone_ci16().astype(np.float64) / 32768
    np.testing.assert_array_equal(read_cf32(out), raw[0::2] + 1j * raw[1::2])


@pytest.mark.gpu
@pytest.mark.parametrize("rec", ["tone_ci16", "tone_ci8"])
@pytest.mark.parametrize("taps", ["lowpass", "lowpass_long"])
@pytest.mark.parametrize("impl", ["plain", "tc_split", "auto", "register"])
def test_sigmf_fir_is_the_fir_of_the_converted_samples(fixtures: Path, tmp_path: Path, rec: str,
                                                       taps: str, impl: str) -> None:
    rfgpu("fir", "--in", fixtures / f"{rec}.sigmf-meta", "--taps", fixtures / f"{taps}.f32",
          "--out", tmp_path / "sigmf.cf32", "--impl", impl)
    rfgpu("fir", "--in", fixtures / f"{rec}.cf32", "--taps", fixtures / f"{taps}.f32",
          "--out", tmp_path / "cf32.cf32", "--impl", impl)
    assert (tmp_path / "sigmf.cf32").read_bytes() == (tmp_path / "cf32.cf32").read_bytes()
    x = np.fromfile(fixtures / f"{rec}.cf32", dtype="<c8")
    expected = orc.fir(x, signals.fixture_taps(taps))
    np.testing.assert_allclose(read_cf32(tmp_path / "sigmf.cf32"), expected, rtol=FIR_RTOL,
                               atol=FIR_ATOL)


@pytest.mark.gpu
@pytest.mark.parametrize("rec", ["tone_ci16", "tone_ci8"])
@pytest.mark.parametrize("impl", ["tiled", "tc_split"])
@pytest.mark.parametrize("memory", ["copy", "zero-copy"])
def test_sigmf_stream_is_bit_identical_to_fir(fixtures: Path, tmp_path: Path, rec: str, impl: str,
                                              memory: str) -> None:
    rfgpu("fir", "--in", fixtures / f"{rec}.sigmf-meta", "--taps", fixtures / "lowpass_long.f32",
          "--out", tmp_path / "fir.cf32", "--impl", impl)
    rfgpu("stream", "--in", fixtures / f"{rec}.sigmf-data", "--taps",
          fixtures / "lowpass_long.f32", "--out", tmp_path / "stream.cf32", "--impl", impl,
          "--chunk", 3000, "--depth", 3, "--memory", memory)
    assert (tmp_path / "fir.cf32").read_bytes() == (tmp_path / "stream.cf32").read_bytes()


@pytest.mark.gpu
@pytest.mark.parametrize("impl", ["plain", "auto"])
def test_sigmf_channelize_and_stream_read_the_recording(fixtures: Path, tmp_path: Path,
                                                        impl: str) -> None:
    for src, name in [(fixtures / "tone_ci16.sigmf-meta", "a"), (fixtures / "tone_ci16.cf32", "b")]:
        rfgpu("channelize", "--in", src, "--taps", fixtures / "channelizer_proto.f32",
              "--channels", 16, "--out", tmp_path / f"chan_{name}.cf32", "--impl", impl)
        rfgpu("stream", "--in", src, "--taps", fixtures / "lowpass_long.f32",
              "--out", tmp_path / f"stream_{name}.cf32", "--chunk", 4096)
    assert (tmp_path / "chan_a.cf32").read_bytes() == (tmp_path / "chan_b.cf32").read_bytes()
    assert (tmp_path / "stream_a.cf32").read_bytes() == (tmp_path / "stream_b.cf32").read_bytes()


@pytest.mark.gpu
def test_sigmf_sample_rate_comes_from_the_recording(fixtures: Path, tmp_path: Path) -> None:
    proc = rfgpu("stream", "--in", fixtures / "tone_ci16.sigmf-data", "--taps",
                 fixtures / "lowpass.f32", "--out", tmp_path / "y.cf32", "--bench", 3)
    assert json.loads(proc.stdout)["sample_rate"] == signals.SAMPLE_RATE


# --- magnitude (tests/test_pipeline.py:88-110) and channelize --output magnitude -------------

def test_bad_channelize_output_is_a_usage_error(fixtures: Path, tmp_path: Path) -> None:
    proc = rfgpu("channelize", "--in", fixtures / "tone.cf32", "--taps",
                 fixtures / "channelizer_proto.f32", "--channels", 16, "--out",
                 tmp_path / "z.f32", "--output", "power", check=False)
    assert proc.returncode == 2
    assert "--output" in proc.stderr


def test_magnitude_usage_errors(tmp_path: Path) -> None:
    proc = rfgpu("magnitude", "--in", tmp_path / "x.cf32", check=False)
    assert proc.returncode == 2
    proc = rfgpu("magnitude", "--in", tmp_path / "x.cf32", "--out", tmp_path / "m.f32",
                 "--taps", tmp_path / "h.f32", check=False)
    assert proc.returncode == 2


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tone.cf32", "tone_odd.cf32", "short.cf32",
                                  "tone_ci16.sigmf-meta"])
def test_magnitude_matches_reference(fixtures: Path, tmp_path: Path, name: str) -> None:
    out = tmp_path / "magnitude.f32"
    rfgpu("magnitude", "--in", fixtures / name, "--out", out)
    stem = name.split(".")[0]
    expected = orc.magnitude(signals.fixture_signal(stem))
    actual = np.fromfile(out, dtype="<f4")
    assert actual.shape == expected.shape
    np.testing.assert_allclose(actual, expected, rtol=1e-6, atol=1e-6)


@pytest.mark.gpu
def test_magnitude_of_zeros_is_exactly_zero(fixtures: Path, tmp_path: Path) -> None:
    out = tmp_path / "magnitude.f32"
    rfgpu("magnitude", "--in", fixtures / "zeros.cf32", "--out", out)
    actual = np.fromfile(out, dtype="<f4")
    assert actual.shape == (4096,) and not np.any(actual)


@pytest.mark.gpu
@pytest.mark.parametrize("impl,channels,taps", [("plain", 16, "channelizer_proto"),
                                                ("auto", 64, "lowpass_long"),
                                                ("tc_split", 64, "lowpass_long")])
def test_channelize_magnitude_output_is_the_magnitude_of_channelize(
        fixtures: Path, tmp_path: Path, impl: str, channels: int, taps: str) -> None:
    args = ["--in", fixtures / "tone.cf32", "--taps", fixtures / f"{taps}.f32",
            "--channels", channels, "--impl", impl]
    rfgpu("channelize", *args, "--out", tmp_path / "z.cf32")
    rfgpu("magnitude", "--in", tmp_path / "z.cf32", "--out", tmp_path / "mz.f32")
    proc = rfgpu("channelize", *args, "--out", tmp_path / "m.f32", "--output", "magnitude",
                 "--bench", 3)
    assert json.loads(proc.stdout)["num_out"] == 65536
    assert (tmp_path / "m.f32").read_bytes() == (tmp_path / "mz.f32").read_bytes()
