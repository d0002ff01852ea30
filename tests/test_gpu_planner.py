"""The device planner (dsmvc_gb_plan_build_many_device): the normal band,
banded LDL^T factor, condition estimate, Float64 routing and Float32 arrays
of many plans computed on the GPU must give the host planner's plans bit for
bit -- the reference's golden plan hashes (tests/numerical_conformance.hpp:
126-176), every array of 60 seeded random requests (all kernels and padding
modes, forced and automatic Float64, ill-conditioned plans that run the
Hager estimate), and the plan hashes of all 3006 axis plans of the
1920x1080 candidate sweep (heights 500..1000, Debicubic / Debilinear /
Delanczos)."""
import time

import numpy as np
import pytest

from common import load_golden, product_request
from test_planner import ARRAYS, ARRAYS64, _random_requests

pytestmark = pytest.mark.gpu

G = load_golden("reference_goldens.json")


def test_device_plans_match_golden_hashes(gb, executor):
    reqs = [product_request(gb, fx["request"]) for fx in G["axis_fixtures"]]
    plans = gb.build_plans(reqs, device=0)
    for fx, req, p in zip(G["axis_fixtures"], reqs, plans):
        f32, complete = p.hashes()
        assert (f32, complete) == (fx["f32_plan"], fx["complete_plan"]), fx["name"]
        assert p.half_bandwidth == fx["half_bandwidth"]


ILL = [(1080, 980, 978.1, 0.95, "lanczos", 2, 0, 0.5, 1.0, "symmetric", 0),
       (1920, 1734, 1732.0888888888887, 0.9555555555556339, "bilinear", 3, 0, 0.5, 1.0, "symmetric", 0),
       (384, 256, 256.0, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 2),
       (120, 70, 70.0, 0.0, "lanczos", 6, 0, 0.5, 1.0, "mirror", 1)]


def test_device_plans_equal_host_plans_array_by_array(gb, executor):
    tuples = _random_requests(60, 7) + ILL
    reqs = [product_request(gb, t) for t in tuples]
    host = gb.build_plans(reqs, threads=4)
    dev = gb.build_plans(reqs, device=0)
    assert any(p.requires_float64 for p in host) and any(p.normal_rcond < 1e-4 for p in host)
    for t, h, d in zip(tuples, host, dev):
        assert (d.support, d.half_bandwidth, d.max_row_entries) == (h.support, h.half_bandwidth, h.max_row_entries)
        assert d.normal_rcond == h.normal_rcond, t
        assert d.normal_inf_norm == h.normal_inf_norm, t
        assert d.requires_float64 == h.requires_float64, t
        for name in ARRAYS + (ARRAYS64 if h.requires_float64 else []):
            assert np.array_equal(d.array(name), h.array(name)), (t, name)
        assert d.hashes() == h.hashes()


def test_device_plans_of_the_candidate_sweep(gb, executor):
    from dsmvc_gb300 import synthetic
    cands = synthetic.native_resolution_candidates(1920, 1080, range(500, 1001))
    reqs = [r for c in cands for r in (c[3], c[4])]
    assert len(reqs) == 3006
    t0 = time.perf_counter()
    host = gb.build_plans(reqs, threads=0)
    t1 = time.perf_counter()
    dev = gb.build_plans(reqs, device=0)
    t2 = time.perf_counter()
    print(f"3006 plans: host threads {t1 - t0:.3f} s, device {t2 - t1:.3f} s")
    for h, d in zip(host, dev):
        assert d.hashes() == h.hashes()


def test_device_planner_refuses_custom_kernels(gb, executor):
    req = gb.AxisRequest(64, 48, 48.0, 0.0, "custom", 3)
    with pytest.raises(ValueError, match="custom"):
        gb.build_plans([req], device=0)


def test_prepare_many_matches_single_prepares(gb, executor):
    """dsmvc_gb_prepare_many (one upload for many plans, device-planned
    here) serves calls exactly like plans prepared one at a time."""
    from common import make_input
    reqs = [gb.AxisRequest(480, 320, 320.0, 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "symmetric", 0),
            gb.AxisRequest(270, 180, 180.0, 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "symmetric", 0),
            gb.AxisRequest(300, 200, 200.0, 0.0, "spline36", 3, 0.0, 0.5, 1.0, "reflect101", 2),
            gb.AxisRequest(170, 113, 113.0, 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "symmetric", 2)]
    plans = gb.build_plans(reqs, device=0)
    single = gb.Executor(0)
    many = gb.Executor(0)
    for p in plans:
        single.prepare(p)
    many.prepare_many(plans + plans[:1])          # repeats are prepared once
    for h, v, sample in ((plans[0], plans[1], "f32"), (plans[0], plans[1], "u16"), (plans[2], plans[3], "f32")):
        x = make_input(v.source_size, h.source_size, sample, 5)
        conv = gb.integer_conversion(16, False, False) if sample == "u16" else None
        assert np.array_equal(single.inverse_2d(h, v, x, conv), many.inverse_2d(h, v, x, conv))
    assert many.stats()["plan_uploads"] == 4
    single.close()
    many.close()
