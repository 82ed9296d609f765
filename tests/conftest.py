"""Shared test setup: the `gpu` marker, import paths, and the golden vectors."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "gpu-rf-pipeline_gb300"
GOLDEN = ROOT / "tests" / "golden"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config: pytest.Config) -> None:
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


class Golden:
    """tests/golden/reference_outputs.npz: outputs of the project's tools/reference.py."""

    def __init__(self) -> None:
        data = np.load(GOLDEN / "reference_outputs.npz")
        self._data = {k: data[k] for k in data.files}
        self.cases = {c["name"]: c for c in json.loads(str(self._data["__cases__"]))}

    def idx(self, name: str) -> np.ndarray:
        return self._data[f"{name}/idx"]

    def val(self, name: str) -> np.ndarray:
        return self._data[f"{name}/val"]

    def sums(self, name: str) -> np.ndarray:
        return self._data[f"{name}/sum"]


@pytest.fixture(scope="session")
def golden() -> Golden:
    return Golden()
