"""Generates tests/golden/reference_outputs.json from the reference's own CPU
engine, compiled from its sources by oracle/ref/Makefile (run where the
reference tree is present):

    python tests/golden/make_golden.py

Each case records the request pair, the seeded input recipe and the FNV-1a
hash (tests/numerical_conformance.hpp:193-248 stream) of the reference's
CpuExecutor(CpuPath::scalar) output, so the oracle and the GPU path can be
checked against the real reference on any machine.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import oracle as O  # noqa: E402
import reference as R  # noqa: E402

# (name, horizontal request, vertical request, sample, conversion)
# request tuple: source, destination, active, shift, kernel, taps, b, c, blur,
# border, f64_mode
CASES = [
    ("bicubic-f32", (97, 67, 67.0, 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "symmetric", 0),
     (73, 51, 51.0, 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "symmetric", 0), "f32", None),
    ("bilinear-zero-f32", (81, 64, 63.5, 0.25, "bilinear", 3, 0.0, 0.5, 1.0, "zero", 0),
     (60, 45, 45.0, -0.125, "bilinear", 3, 0.0, 0.5, 1.0, "zero", 0), "f32", None),
    ("lanczos3-repeat-u16", (192, 144, 144.0, 0.0, "lanczos", 3, 0.0, 0.5, 1.0, "repeat", 0),
     (108, 81, 81.0, 0.0, "lanczos", 3, 0.0, 0.5, 1.0, "repeat", 0), "u16",
     (4096.0, 1.0 / 56064.0, 56064.0, 4096.0, 65535)),
    ("lanczos3-chroma-u16", (96, 72, 72.0, 0.0625, "lanczos", 3, 0.0, 0.5, 1.0, "repeat", 0),
     (54, 40, 40.5, 0.0, "lanczos", 3, 0.0, 0.5, 1.0, "repeat", 0), "u16",
     (32768.0, 1.0 / 57344.0, 57344.0, 32768.0, 65535)),
    ("spline36-reflect-u8", (120, 90, 90.0, 0.1, "spline36", 3, 0.0, 0.5, 1.0, "reflect101", 0),
     (64, 50, 50.0, 0.0, "spline36", 3, 0.0, 0.5, 1.0, "reflect101", 0), "u8",
     (16.0, 1.0 / 219.0, 219.0, 16.0, 255)),
    ("spline64-blur-f64", (128, 86, 85.5, 0.0, "spline64", 3, 0.0, 0.5, 1.1, "symmetric", 2),
     (72, 48, 48.0, 0.0, "bicubic", 3, 1.0 / 3.0, 1.0 / 3.0, 1.1, "symmetric", 2), "f32", None),
    ("mitchell-blur-f32", (160, 107, 106.5, 0.0, "bicubic", 3, 1.0 / 3.0, 1.0 / 3.0, 1.1, "mirror", 0),
     (90, 60, 60.0, 0.0, "bicubic", 3, 1.0 / 3.0, 1.0 / 3.0, 1.1, "mirror", 0), "f32", None),
    ("auto-risk-f64-u16", (1080, 980, 978.1, 0.95, "lanczos", 2, 0.0, 0.5, 1.0, "symmetric", 0),
     (24, 16, 16.0, 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "symmetric", 0), "u16",
     (4096.0, 1.0 / 56064.0, 56064.0, 4096.0, 65535)),
    ("lanczos4-wide-f32", (150, 100, 100.0, 0.0, "lanczos", 4, 0.0, 0.5, 1.0, "symmetric", 0),
     (70, 47, 47.0, 0.0, "spline16", 3, 0.0, 0.5, 1.0, "symmetric", 0), "f32", None),
]


def make_input(rows: int, cols: int, sample: str, seed: int) -> np.ndarray:
    """Seeded input shared by the fixtures and the tests: the reference
    tests' xorshift normal generator (tests/numerical_conformance.hpp:178-191)
    mapped to the sample range."""
    v = O.make_normal_input(rows * cols, seed).reshape(rows, cols)
    if sample == "f32":
        return v
    if sample == "u16":
        return ((v.astype(np.float64) + 1.0) * 30000.0 + 2000.0).astype(np.uint16)
    return ((v.astype(np.float64) + 1.0) * 110.0 + 16.0).astype(np.uint8)


def main() -> None:
    if not R.available() and not R.build():
        raise SystemExit("reference sources are not available")
    out = []
    for idx, (name, hq, vq, sample, conv) in enumerate(CASES):
        seed = 0x5EED0000 + idx
        hr, vr = O.make_request(*hq), O.make_request(*vq)
        h, v = R.Plan(hr), R.Plan(vr)
        x = make_input(v.source_size, h.source_size, sample, seed)
        y = R.inverse_2d(h, v, x, conv, path=0)
        out.append({"name": name, "horizontal": list(hq), "vertical": list(vq),
                    "sample": sample, "conversion": list(conv) if conv else None,
                    "seed": seed, "output_hash": O.output_hash(y.astype(np.float32)),
                    "output_sum": float(np.asarray(y, np.float64).sum())})
        print(name, out[-1]["output_hash"])
    with open(os.path.join(HERE, "reference_outputs.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "engine": "reference CpuExecutor(CpuPath::scalar), -O2 -ffp-contract=off",
                   "cases": out}, f, indent=1)


if __name__ == "__main__":
    main()
