"""The tuned tables behind `auto` (rfx_autotune_*), on the CPU: the text format and the
automatic load of $RFX_TUNE_FILE before the first lookup. Without a GPU the library keys its
entries by the device name "unknown", so a file written for that key applies here."""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

from conftest import PKG, ROOT

PICK = ("import sys; sys.path[:0] = [{root!r}, {pkg!r}]; import rfx; "
        "print(rfx.fir_impl_used('auto', 24, 1 << 24), rfx.fir_impl_used('auto', 1025, 1 << 24))")


def picks(env_file: Path | None) -> list[str]:
    env = dict(os.environ)
    env.pop("RFX_TUNE_FILE", None)
    if env_file is not None:
        env["RFX_TUNE_FILE"] = str(env_file)
    out = subprocess.run([sys.executable, "-c", PICK.format(root=str(ROOT), pkg=str(PKG))],
                         capture_output=True, text=True, env=env, timeout=120)
    assert out.returncode == 0, out.stderr
    return out.stdout.split()


def test_builtin_rule_without_a_table() -> None:
    assert picks(None) == ["plain", "tc_split"]


def test_table_named_by_the_environment_is_loaded_before_the_first_lookup(tmp_path) -> None:
    f = tmp_path / "tune.txt"
    # taps bucket 4 (16-31) and 10 (1024-2047), length bucket 24: swap both choices; a line for
    # another device and a malformed line are skipped.
    f.write_text("fir unknown 4 24 1 48 4 0.100000\n"
                 "fir unknown 10 24 0 0 0 0.200000\n"
                 "fir NVIDIA_Other/1 4 24 0 0 0 0.1\n"
                 "garbage line\n")
    assert picks(f) == ["tc_split", "plain"]


def test_missing_table_file_leaves_the_builtin_rule(tmp_path) -> None:
    assert picks(tmp_path / "absent.txt") == ["plain", "tc_split"]
