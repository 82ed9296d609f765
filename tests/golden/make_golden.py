#!/usr/bin/env python3
"""Generate the golden vectors that pin the oracle to the gpu-rf-pipeline project's own
float64 reference (tools/reference.py, imported unchanged from a checkout of that project).

Run where the project is checked out (it is not needed anywhere else):

    python tests/golden/make_golden.py --reference PATH/TO/gpu-rf-pipeline

Writes, next to this script:

* ``fixture_sha256.json`` — SHA-256 of the project's fixture files (signals and taps), so the
  tests can check that rfx.signals regenerates them byte for byte;
* ``reference_outputs.npz`` — tools/reference.py's outputs for the FIR and channelizer cases
  that the project's own tests use (tests/test_pipeline.py:120-135 and :367-383,
  tests/test_reference.py:115-121 and :208-223), for a few extra edge cases, and for prefixes
  of three benchmark workloads. Long outputs are stored as every element of a deterministic
  index set (the first 1100 and then every 29th) plus three whole-vector checksums (sum,
  energy and a seeded weighted sum), so the file stays small while every element is pinned.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "gpu-rf-pipeline_gb300"))
from rfx import signals  # noqa: E402

FIXTURE_FILES = ["tone.cf32", "tone_odd.cf32", "short.cf32", "zeros.cf32", "lowpass.f32",
                 "lowpass_long.f32", "channelizer_proto.f32", "identity.f32",
                 "tone_ci16.sigmf-data"]

FULL_LIMIT = 2048  # outputs up to this many elements are stored whole


def sample_index(n: int) -> np.ndarray:
    if n <= FULL_LIMIT:
        return np.arange(n, dtype=np.int64)
    head = np.arange(min(n, 1100), dtype=np.int64)
    tail = np.arange(1100, n, 29, dtype=np.int64)
    return np.concatenate([head, tail, np.array([n - 1], dtype=np.int64)])


def checksum_weights(n: int) -> np.ndarray:
    rng = np.random.default_rng(20261203)
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


def checksums(y: np.ndarray) -> np.ndarray:
    y = np.asarray(y, dtype=np.complex128).ravel()
    w = checksum_weights(y.size)
    return np.array([np.sum(y), np.sum(np.abs(y) ** 2) + 0j, np.sum(w * y)])


def random_complex(seed: int, n: int) -> np.ndarray:
    # The helper the project's oracle tests use (tests/test_reference.py:27-29).
    rng = np.random.default_rng(seed)
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reference", type=Path, required=True,
                    help="checkout of the gpu-rf-pipeline project (holds tools/reference.py)")
    args = ap.parse_args()
    sys.path.insert(0, str(args.reference / "tools"))
    import reference  # noqa: E402  (the project's tools/reference.py, unchanged)

    fixtures = args.reference / "tests" / "fixtures"
    shas = {name: hashlib.sha256((fixtures / name).read_bytes()).hexdigest()
            for name in FIXTURE_FILES}
    (HERE / "fixture_sha256.json").write_text(json.dumps(shas, indent=2, sort_keys=True) + "\n")

    out: dict[str, np.ndarray] = {}
    cases: list[dict] = []

    def record(name: str, y: np.ndarray, spec: dict) -> None:
        y = np.asarray(y, dtype=np.complex128).ravel()
        idx = sample_index(y.size)
        out[f"{name}/idx"] = idx
        out[f"{name}/val"] = y[idx]
        out[f"{name}/sum"] = checksums(y)
        cases.append({"name": name, "size": int(y.size), **spec})

    def fixture_x(name: str) -> np.ndarray:
        return reference.read_cf32(fixtures / f"{name}.cf32")

    def fixture_h(name: str) -> np.ndarray:
        return reference.read_f32(fixtures / f"{name}.f32")

    # FIR on the project's fixtures (tests/test_pipeline.py:120-167).
    for sig in ["tone", "tone_odd", "short", "zeros"]:
        for taps in ["lowpass", "lowpass_long", "identity"]:
            record(f"fir/{sig}/{taps}", reference.fir(fixture_x(sig), fixture_h(taps)),
                   {"op": "fir", "signal": sig, "taps": taps})
    # The SigMF ci16 recording, converted as the project's tests convert it
    # (tests/test_pipeline.py:276-278: components / 32768 in float64, exact), through the FIR
    # (tests/test_pipeline.py:289-295) and the channelizer.
    meta = json.loads((fixtures / "tone_ci16.sigmf-meta").read_text())["global"]
    raw = np.fromfile(fixtures / "tone_ci16.sigmf-data", dtype="<i2").astype(np.float64) / 32768
    x_ci16 = raw[0::2] + 1j * raw[1::2]
    sigmf = {"datatype": meta["core:datatype"], "sample_rate": meta["core:sample_rate"],
             "num_channels": meta["core:num_channels"]}
    for taps in ["lowpass", "lowpass_long", "identity"]:
        record(f"fir/tone_ci16/{taps}", reference.fir(x_ci16, fixture_h(taps)),
               {"op": "fir", "signal": "tone_ci16", "taps": taps, "sigmf": sigmf})
    record("chan/tone_ci16/channelizer_proto/16",
           reference.channelize(x_ci16, fixture_h("channelizer_proto"), 16),
           {"op": "channelize", "signal": "tone_ci16", "taps": "channelizer_proto",
            "channels": 16, "sigmf": sigmf})
    # Channelizer on the project's fixtures (tests/test_pipeline.py:367-373).
    for sig, taps, m in [("tone", "channelizer_proto", 16), ("tone_odd", "channelizer_proto", 16),
                         ("tone", "lowpass_long", 64), ("short", "lowpass", 4),
                         ("tone_odd", "identity", 1), ("tone", "lowpass_long", 16)]:
        record(f"chan/{sig}/{taps}/{m}",
               reference.channelize(fixture_x(sig), fixture_h(taps), m),
               {"op": "channelize", "signal": sig, "taps": taps, "channels": m})
    # The project's brute-force FIR cases (tests/test_reference.py:115-121) plus edge cases
    # around tile sizes: inputs random_complex(3, N), taps default_rng(4) normals.
    for n, k in [(50, 7), (50, 1), (5, 12), (1, 1), (1000, 31), (777, 64), (777, 65),
                 (3000, 1089), (130, 129), (4099, 257)]:
        x = random_complex(3, n)
        h = np.random.default_rng(4).standard_normal(k)
        x32 = signals.to_cf32(x).astype(np.complex128)
        h32 = h.astype(np.float32).astype(np.float64)
        record(f"firrand/{n}/{k}", reference.fir(x32, h32),
               {"op": "fir", "n": n, "k": k, "x_seed": 3, "h_seed": 4})
    # The project's brute-force channelizer cases (tests/test_reference.py:208-216) plus
    # larger channel counts; inputs default_rng(N + K + M).
    for n, k, m in [(100, 37, 4), (64, 16, 16), (7, 63, 4), (33, 1, 1), (50, 24, 8),
                    (5000, 1024, 64), (4100, 4096, 1024), (2048, 256, 128)]:
        rng = np.random.default_rng(n + k + m)
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        h = rng.standard_normal(k)
        x32 = signals.to_cf32(x).astype(np.complex128)
        h32 = h.astype(np.float32).astype(np.float64)
        record(f"chanrand/{n}/{k}/{m}", reference.channelize(x32, h32, m),
               {"op": "channelize", "n": n, "k": k, "channels": m, "seed": n + k + m})
    # Prefixes of the benchmark workloads (their own taps).
    w = signals.long_fir(1 << 15)
    record("bench/fir1025", reference.fir(w.x.astype(np.complex128), w.taps.astype(np.float64)),
           {"op": "fir", "workload": "fir1025", "n": 1 << 15})
    w = signals.channelizer64(1 << 16)
    record("bench/pfb64",
           reference.channelize(w.x.astype(np.complex128), w.taps.astype(np.float64), 64),
           {"op": "channelize", "workload": "pfb64", "n": 1 << 16, "channels": 64})
    w = signals.channelizer1024(40 * 1024)
    record("bench/pfb1024",
           reference.channelize(w.x.astype(np.complex128), w.taps.astype(np.float64), 1024),
           {"op": "channelize", "workload": "pfb1024", "n": 40 * 1024, "channels": 1024})

    out["__cases__"] = np.array(json.dumps(cases))
    np.savez_compressed(HERE / "reference_outputs.npz", **out)
    size = (HERE / "reference_outputs.npz").stat().st_size
    print(f"wrote {len(cases)} cases ({size / 1e3:.0f} kB) and {len(shas)} fixture hashes")


if __name__ == "__main__":
    main()
