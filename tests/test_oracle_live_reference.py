"""The oracle against the reference's own CPU engine, live (CPU): seeded
random 2D descales (every built-in kernel, border and Float64 mode; Float32,
u8 and u16 samples) through the reference's CpuExecutor(CpuPath::scalar),
built from its sources by oracle/ref, and through the oracle, bit for bit.
The recorded fixtures (tests/golden/reference_outputs.json) pin the oracle
where the reference is absent; this widens the pin where it is built.
Both sides plan from the same request: the oracle's planner and the
reference's."""
import numpy as np
import pytest

import oracle as O
from common import make_input

KERNELS = ["bilinear", "bicubic", "lanczos", "spline16", "spline36", "spline64"]
BORDERS = ["zero", "repeat", "reflect101", "symmetric", "mirror"]
CONVERSIONS = {
    "u8": (16.0, 1.0 / 219.0, 219.0, 16.0, 255),
    "u16": (4096.0, 1.0 / 56064.0, 56064.0, 4096.0, 65535),
}


def _request(rng, src):
    dst = int(rng.integers(max(8, src // 3), src + 1))
    active = float(dst - rng.random() * 1.5) if rng.random() < 0.4 else float(dst)
    return (src, dst, max(active, 1.0), float(rng.uniform(-0.6, 0.6)), KERNELS[rng.integers(6)],
            int(rng.integers(1, 5)), float(rng.random() * 0.5), float(rng.random() * 0.6),
            float(1.0 if rng.random() < 0.6 else rng.uniform(0.8, 1.5)), BORDERS[rng.integers(5)],
            int(rng.integers(0, 3)))


def _cases(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        hq = _request(rng, int(rng.integers(16, 160)))
        vq = _request(rng, int(rng.integers(16, 120)))
        out.append((hq, vq, ("f32", "u8", "u16")[i % 3], 0x11E0000 + i))
    return out


CASES = _cases(120, 2026)


@pytest.fixture(scope="module")
def R():
    import reference
    if not reference.available():
        pytest.skip("the reference engine is not built on this machine")
    return reference


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[2]}-{c[0][4]}-{c[1][4]}-{c[3] & 0xFFFF}")
def test_oracle_equals_reference_engine(R, case):
    hq, vq, sample, seed = case
    hr, vr = O.make_request(*hq), O.make_request(*vq)
    oh, ov = O.Plan(hr), O.Plan(vr)
    rh, rv = R.Plan(hr), R.Plan(vr)
    x = make_input(ov.source_size, oh.source_size, sample, seed)
    conv = CONVERSIONS.get(sample)
    want = R.inverse_2d(rh, rv, x, conv, path=0)
    got = O.inverse_2d(oh, ov, x, conv)
    assert got.dtype == want.dtype and got.shape == want.shape
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
