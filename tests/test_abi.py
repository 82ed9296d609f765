"""The C ABI on the CPU: librfx.so builds, loads, exports every function include/rfx.h declares,
and rejects bad arguments before touching the GPU (no compute calls here)."""
from __future__ import annotations

import ctypes
import re

import pytest

from conftest import ROOT

import rfx


@pytest.fixture(scope="module")
def lib():
    if not rfx.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    return rfx.load()


def declared_functions() -> list[str]:
    text = (ROOT / "include" / "rfx.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rfx_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_function_is_exported(lib) -> None:
    names = declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
        assert name in rfx.SIGNATURES, f"{name} missing from the Python binding"


def test_binding_declares_nothing_the_header_does_not() -> None:
    assert set(rfx.SIGNATURES) <= set(declared_functions())


def test_integration_guide_lists_every_entry_point() -> None:
    # The table of INTEGRATION.md maps each C entry point to the project interface it replaces
    # (or says it has none): a function the header adds is listed there too.
    guide = (ROOT / "INTEGRATION.md").read_text()
    missing = [name for name in declared_functions() if f"{name}" not in guide]
    assert not missing, missing


def test_library_targets_sm_103a(lib) -> None:
    assert b"sm_103a" in lib.rfx_version()


def test_impl_names_and_aliases(lib) -> None:
    assert rfx.fir_impl_names() == ["plain", "tc_split", "auto"]
    assert rfx.chan_impl_names() == ["plain", "tc_split", "auto"]
    # The project's --impl names keep working and mean the plain kernel (same results).
    for name in ["naive", "tiled", "tiled_const", "register", "plain"]:
        assert rfx.parse_fir_impl(name) == rfx.FIR_PLAIN
    assert rfx.parse_fir_impl("tc_split") == rfx.FIR_TC
    with pytest.raises(rfx.RfxError) as e:
        rfx.parse_fir_impl("no_such_impl")
    assert e.value.status == 1 and "no_such_impl" in str(e.value)


def test_frames_arithmetic(lib) -> None:
    assert lib.rfx_channelize_frames(0, 16) == 0
    assert lib.rfx_channelize_frames(1, 16) == 1
    assert lib.rfx_channelize_frames(65536, 16) == 4096
    assert lib.rfx_channelize_frames(10007, 16) == 626
    assert lib.rfx_channelize_frames(1 << 26, 1024) == 1 << 16
    assert lib.rfx_channelize_frames(5, 0) == 0


@pytest.mark.parametrize("n,k,status", [(-1, 63, 1), (100, 0, 1), (100, 8193, 2),
                                         (1 << 31, 63, 1)])
def test_fir_argument_errors(lib, n: int, k: int, status: int) -> None:
    buf = ctypes.create_string_buffer(64)
    p = (ctypes.addressof(buf) + 15) & ~15
    rc = lib.rfx_fir_launch(0, p, p, p, n, k, None)
    assert rc == status
    assert lib.rfx_last_error()


def test_fir_alignment_error(lib) -> None:
    buf = ctypes.create_string_buffer(64)
    p = (ctypes.addressof(buf) + 15) & ~15
    assert lib.rfx_fir_launch(0, p + 8, p, p, 10, 3, None) == 3
    assert b"aligned" in lib.rfx_last_error()


def test_zero_samples_is_a_no_op(lib) -> None:
    assert lib.rfx_fir_launch(0, None, None, None, 0, 5, None) == 0


def test_load_const_taps_checks_capacity(lib) -> None:
    buf = ctypes.create_string_buffer(64)
    assert lib.rfx_fir_load_const_taps(ctypes.addressof(buf), 8192, None) == 0
    assert lib.rfx_fir_load_const_taps(ctypes.addressof(buf), 8193, None) == 2
    assert lib.rfx_fir_load_const_taps(ctypes.addressof(buf), 0, None) == 1


def test_batch_argument_errors(lib) -> None:
    assert lib.rfx_fir_batch_launch(0, None, 0, None) == 1
    caps = (rfx.FirCapture * 1)()
    caps[0] = rfx.FirCapture(None, None, None, 10, 5, 0)
    assert lib.rfx_fir_batch_launch(0, caps, 1, None) == 1  # null pointers
    assert lib.rfx_fir_batched_device(0, None, None, None, 0, None, 5, None) == 1


def test_channelizer_plan_argument_errors(lib) -> None:
    handle = ctypes.c_void_p()
    assert lib.rfx_chan_plan_create(0, 0, 100, ctypes.byref(handle)) == 1
    assert lib.rfx_chan_plan_create(7, 16, 100, ctypes.byref(handle)) == 1
    assert lib.rfx_chan_plan_create(0, 16, -5, ctypes.byref(handle)) == 1
    assert lib.rfx_channelize_launch(None, None, None, None, 10, 5, None) == 1
    assert lib.rfx_chan_plan_destroy(None) == 0


def test_host_block_size_is_checked(lib) -> None:
    for block in (0, 48, 2048):
        assert lib.rfx_fir_host(0, None, 0, None, 1, block, None, None) == 1
        assert b"--block" in lib.rfx_last_error()


def test_fir_format_argument_errors(lib) -> None:
    buf = ctypes.create_string_buffer(64)
    p = (ctypes.addressof(buf) + 15) & ~15
    for fmt in (-1, 3, 7):
        assert lib.rfx_fir_launch_format(0, fmt, p, p, p, 10, 3, None) == 1
        assert b"format" in lib.rfx_last_error()
    # The same checks as rfx_fir_launch, before any device work.
    assert lib.rfx_fir_launch_format(0, 1, p + 4, p, p, 10, 3, None) == 3
    assert lib.rfx_fir_launch_format(0, 2, p, p, p, 10, 0, None) == 1
    assert lib.rfx_fir_launch_format(5, 1, p, p, p, 10, 3, None) == 1
    assert lib.rfx_fir_launch_format(0, 1, None, None, None, 0, 3, None) == 0
    assert lib.rfx_fir_host_format(0, 9, None, 0, None, 1, 256, None, None) == 1


def test_magnitude_argument_errors(lib) -> None:
    buf = ctypes.create_string_buffer(64)
    p = (ctypes.addressof(buf) + 15) & ~15
    assert lib.rfx_magnitude_launch(None, None, 0, None) == 0
    assert lib.rfx_magnitude_launch(None, p, 4, None) == 1
    assert lib.rfx_magnitude_launch(p + 8, p, 4, None) == 3
    assert lib.rfx_magnitude_launch(p, p, -1, None) == 1
    assert lib.rfx_channelize_magnitude_launch(None, p, p, p, 10, 5, None) == 1
    assert lib.rfx_magnitude_host(None, 3, None, None) == 1
    assert lib.rfx_channelize_magnitude_host(0, None, 10, None, 5, 0, None, None) == 1


def test_channelize_format_argument_errors(lib) -> None:
    assert lib.rfx_channelize_launch_format(None, 7, 0, None, None, None, 10, 5, None) == 1
    assert lib.rfx_channelize_launch_format(None, 1, 5, None, None, None, 10, 5, None) == 1
    assert lib.rfx_channelize_launch_format(None, 1, 0, None, None, None, 10, 5, None) == 1
    assert lib.rfx_channelize_host_format(0, 4, 0, None, 10, None, 5, 4, None, None) == 1
    assert lib.rfx_channelize_host_format(0, 1, 0, None, 10, None, 5, 0, None, None) == 1
    assert lib.rfx_fir_stream_format(9, None, 10, None, 5, None, None, None, None) == 1


def test_impl_used_reports_the_kernel_that_runs(lib) -> None:
    # tc_split hands calls it cannot take to the plain kernel; the query says so in advance.
    assert rfx.fir_impl_used("tc_split", 1025, 1 << 24) == "tc_split"
    assert rfx.fir_impl_used("tc_split", 1, 1 << 24) == "plain"          # one tap
    assert rfx.fir_impl_used("tc_split", 3458, 1 << 24) == "plain"       # beyond the budget
    assert rfx.fir_impl_used("tc_split", 3457, 1 << 24) == "tc_split"
    assert rfx.fir_impl_used("tc_split", 1025, 127) == "plain"           # under one block
    assert rfx.fir_impl_used("plain", 1025, 1 << 24) == "plain"
    for name in ["naive", "tiled", "tiled_const", "register"]:
        assert rfx.fir_impl_used(name, 1025, 1 << 24) == "plain"
    # auto's built-in rule: the tensor core from 32 taps and 2^16 samples (the resident-window form
    # up to 385 taps); a batch plan puts every filter of two taps or more on a tensor-core phase
    # at any length (its window phase up to 385 taps).
    assert rfx.fir_impl_used("auto", 1025, 1 << 24) == "tc_split"
    assert rfx.fir_impl_used("auto", 63, 1 << 24) == "tc_split"
    assert rfx.fir_impl_used("auto", 32, 1 << 24) == "tc_split"
    assert rfx.fir_impl_used("auto", 31, 1 << 24) == "plain"
    assert rfx.fir_impl_used("auto", 1025, 1 << 12) == "plain"
    assert rfx.fir_impl_used("auto", 63, 1 << 24, batch=True) == "tc_split"
    assert rfx.fir_impl_used("auto", 63, 4096, batch=True) == "tc_split"
    assert rfx.fir_impl_used("auto", 31, 1 << 24, batch=True) == "tc_split"
    assert rfx.fir_impl_used("auto", 1, 1 << 24, batch=True) == "plain"
    assert rfx.fir_impl_used("auto", 386, 1 << 24, batch=True) == "tc_split"
    assert rfx.fir_impl_used("auto", 386, 1 << 12, batch=True) == "tc_split"
    assert rfx.fir_impl_used("auto", 1025, 127, batch=True) == "plain"   # under one block
    with pytest.raises(rfx.RfxError):
        rfx.fir_impl_used("tc_split", 0, 100)
    with pytest.raises(rfx.RfxError):
        rfx.fir_impl_used(7, 10, 100)
