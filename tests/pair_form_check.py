"""Child process of test_fir_tc_pair_gpu.py: forces the CTA-pair tensor-core FIR through a
tuning table, runs each case and prints one JSON line per case (normwise error vs float64).

Run as a separate process so the forced table does not reach other tests."""
from __future__ import annotations

import json
import sys
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path[:0] = [str(ROOT), str(ROOT / "gpu-rf-pipeline_gb300")]

import numpy as np  # noqa: E402
import torch  # noqa: E402

import rfx  # noqa: E402
from oracle import rf_oracle as orc  # noqa: E402
from rfx import signals  # noqa: E402

PAIR_TILE_BLOCKS = 192   # TcConfig.tile_blocks of the pair form
RFX_FIR_TC = 1


def bucket(v: int) -> int:
    return max(int(v).bit_length() - 1, 0)


def main() -> int:
    cases = json.loads(sys.argv[1])
    lib = rfx.load()
    rfx.autotune_fir("tc_split", 63, 4096)       # one entry, to learn this device's key
    with tempfile.TemporaryDirectory() as tmp:
        path = Path(tmp) / "table.txt"
        assert lib.rfx_autotune_save(str(path).encode()) == 0
        key = path.read_text().split()[0]
        lines = {f"{key} {bucket(k)} {bucket(n)} {RFX_FIR_TC} {PAIR_TILE_BLOCKS} {stages} 0.001"
                 for n, k, stages in cases}
        path.write_text("\n".join(sorted(lines)) + "\n")
        assert lib.rfx_autotune_load(str(path).encode()) == 0
    for n, k, stages in cases:
        rng = np.random.default_rng(1000 + n + k)
        x = signals.to_cf32(rng.standard_normal(n) + 1j * rng.standard_normal(n))
        h = (rng.standard_normal(k) / np.sqrt(k)).astype(np.float32)
        xd = torch.from_numpy(x).cuda()
        hd = torch.from_numpy(h).cuda()
        yd = rfx.fir(xd, hd, impl="tc_split")
        torch.cuda.synchronize()
        err = orc.normwise_error(yd.cpu().numpy(), orc.fir_fast(x, h))
        print(json.dumps({"n": n, "k": k, "stages": stages, "err": float(err)}), flush=True)
    print(json.dumps({"fault": rfx.device_fault()}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
