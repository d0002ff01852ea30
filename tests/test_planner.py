"""The product planner (host C++, through the C ABI) against the reference's
golden plan hashes and, array by array, against the oracle (CPU)."""
import numpy as np
import pytest

import oracle as O
from common import load_golden, oracle_request, product_request

G = load_golden("reference_goldens.json")


@pytest.mark.parametrize("fx", G["axis_fixtures"], ids=lambda f: f["name"])
def test_plan_hashes(gb, fx):
    plan = gb.AxisPlan(product_request(gb, fx["request"]), cached=False)
    f32, complete = plan.hashes()
    assert plan.half_bandwidth == fx["half_bandwidth"]
    assert f32 == fx["f32_plan"]
    assert complete == fx["complete_plan"]


ARRAYS = ["transpose_offsets", "transpose_indices", "transpose_weights", "lower_ld",
          "upper_l", "inverse_diagonal"]
ARRAYS64 = ["transpose_weights_f64", "normal_bands_f64", "ldlt_bands_f64", "inverse_diagonal_f64"]


def _random_requests(n, seed):
    rng = np.random.default_rng(seed)
    kernels = ["bilinear", "bicubic", "lanczos", "spline16", "spline36", "spline64"]
    borders = ["zero", "repeat", "reflect101", "symmetric", "mirror"]
    out = []
    for _ in range(n):
        src = int(rng.integers(9, 400))
        dst = int(rng.integers(8, src + 1))
        active = float(dst - rng.random() * 2.0) if rng.random() < 0.5 else float(dst)
        if active <= 0:
            active = float(dst)
        out.append((src, dst, active, float(rng.normal() * 0.5), kernels[rng.integers(6)],
                    int(rng.integers(1, 6)), float(rng.random() * 0.5), float(rng.random() * 0.6),
                    float(1.0 if rng.random() < 0.6 else 0.8 + rng.random() * 0.8),
                    borders[rng.integers(5)], int(rng.integers(0, 3))))
    return out


@pytest.mark.parametrize("req", _random_requests(60, 7), ids=lambda r: f"{r[4]}-{r[0]}-{r[1]}")
def test_plan_arrays_match_oracle(gb, req):
    p = gb.AxisPlan(product_request(gb, req), cached=False)
    o = O.Plan(oracle_request(req))
    assert (p.source_size, p.destination_size, p.support, p.half_bandwidth) == \
        (o.source_size, o.destination_size, o.support, o.half_bandwidth)
    assert p.normal_rcond == o.normal_rcond
    assert p.requires_float64 == o.requires_float64
    for name in ARRAYS + (ARRAYS64 if o.requires_float64 else []):
        assert np.array_equal(p.array(name), getattr(o, name)), name
    assert p.max_row_entries == int(np.max(np.diff(o.transpose_offsets)))


def test_cache_single_flight_and_stats(gb):
    gb.clear_planner_caches()
    req = product_request(gb, G["axis_fixtures"][6]["request"])
    a = gb.AxisPlan(req)
    s1 = gb.planner_cache_stats()
    b = gb.AxisPlan(req)
    s2 = gb.planner_cache_stats()
    assert s1["plan_entries"] == 1 and s1["plan_resident_bytes"] > 0
    assert s2["plan_hits"] == s1["plan_hits"] + 1
    assert a.hashes() == b.hashes()
    gb.clear_planner_caches()
    assert gb.planner_cache_stats()["plan_entries"] == 0


def test_custom_kernel_matches_builtin(gb):
    # A custom kernel reproducing bilinear yields the bilinear plan arrays.
    req = (50, 40, 40.0, 0.1, "bilinear", 1, 0.0, 0.5, 1.0, "symmetric", 1)
    ref = gb.AxisPlan(product_request(gb, req), cached=False)
    creq = gb.AxisRequest(50, 40, 40.0, 0.1, "custom", 1, 0.0, 0.5, 1.0, "symmetric", 1)
    cust = gb.AxisPlan(creq, custom=lambda x: max(1.0 - x, 0.0), cached=False)
    for name in ARRAYS:
        assert np.array_equal(ref.array(name), cust.array(name))


@pytest.mark.parametrize("bad,exc", [
    ((0, 10, 10.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 0), ValueError),
    ((20, 10, 0.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 0), ValueError),
    ((20, 10, 10.0, float("nan"), "bicubic", 3, 0, 0.5, 1.0, "symmetric", 0), ValueError),
    ((20, 10, 10.0, 0.0, "bicubic", 3, 0, 0.5, -1.0, "symmetric", 0), ValueError),
    ((20, 10, 10.0, 0.0, "lanczos", 0, 0, 0.5, 1.0, "symmetric", 0), ValueError),
    ((20, 10, 10.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, 7, 0), ValueError),
    ((20, 10, 10.0, 0.0, "bicubic", 3, 0, 0.5, 1e300, "symmetric", 0), OverflowError),
])
def test_invalid_requests(gb, bad, exc):
    with pytest.raises(exc):
        gb.AxisPlan(product_request(gb, bad), cached=False)


def test_custom_kernel_nonfinite_is_runtime_error(gb):
    creq = gb.AxisRequest(30, 20, 20.0, 0.0, "custom", 2, 0.0, 0.5, 1.0, "symmetric", 0)
    with pytest.raises(gb.DescaleError):
        gb.AxisPlan(creq, custom=lambda x: float("inf"), cached=False)
