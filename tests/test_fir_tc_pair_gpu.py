"""The CTA-pair tensor-core FIR (2-SM MMAs, 256-output blocks), forced through a tuning table
in a child process, against the float64 oracle at the tensor-core bar (normwise 2e-6).

Cases cover both ring depths the pair form picks, tap counts around its 256-sample block
(chunks P = 2 .. 9, and P > 12 split groups are out of its shared-memory range), lengths around
its 24576-output tile, the partial last block, and the shortest input it takes (256 samples)."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

TC_NORMWISE = 2e-6
TILE = 96 * 256
CASES = [
    (40000, 2, 6), (40000, 63, 6), (40000, 255, 6), (40000, 256, 6), (40000, 257, 6),
    (40000, 511, 6), (40000, 1025, 6), (40000, 1025, 4), (40000, 1025, 2), (40000, 2049, 6),
    (256, 1025, 6), (257, 63, 6), (TILE - 1, 1025, 6), (TILE, 1025, 6), (TILE + 1, 1025, 6),
    (3 * TILE + 77, 1025, 6), (200001, 255, 4), (1 << 20, 1025, 6),
]


def test_pair_form_matches_oracle() -> None:
    script = Path(__file__).with_name("pair_form_check.py")
    out = subprocess.run([sys.executable, str(script), json.dumps(CASES)], capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    rows = [json.loads(line) for line in out.stdout.splitlines() if line.startswith("{")]
    assert rows[-1] == {"fault": 0}
    results = rows[:-1]
    assert len(results) == len(CASES)
    for r in results:
        assert r["err"] <= TC_NORMWISE, r
