"""Shared helpers for the tests (requests, seeded inputs, error metrics)."""
import json
import os

import numpy as np

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Reference tolerances (docs/reference.md:136-145, tests/vs_gpu_concurrency.py:57):
F32_MAX_ABS = 2e-5      # Float32 output vs the CPU scalar route, max-abs
F32_MEAN_ABS = 1e-6     # ... and mean-abs
INT_MAX_CODES = 1       # integer output, codes
F64_MAX_ULP = 1         # Float64 route output, float32 ULPs


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def oracle_request(t):
    return O.make_request(*t)


def product_request(gb, t):
    s, d, a, sh, k, taps, b, c, blur, border, mode = t
    return gb.AxisRequest(s, d, a, sh, k, taps, b, c, blur, border, mode)


def make_input(rows, cols, sample, seed):
    v = O.make_normal_input(rows * cols, seed).reshape(rows, cols)
    if sample == "f32":
        return v
    if sample == "u16":
        return ((v.astype(np.float64) + 1.0) * 30000.0 + 2000.0).astype(np.uint16)
    return ((v.astype(np.float64) + 1.0) * 110.0 + 16.0).astype(np.uint8)


def ordered_bits(x):
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.int64)
    return np.where(b & 0x80000000, 0xFFFFFFFF - b, b | 0x80000000)


def max_ulp(a, b):
    return int(np.max(np.abs(ordered_bits(a) - ordered_bits(b)))) if np.size(a) else 0
