"""dsmvc_gb_plan_build_many: plans built on several host threads equal the
plans built one at a time (plan hashes), and a failing request names its
index without returning any plan."""
import pytest

from common import product_request


def test_parallel_plans_equal_serial(gb):
    from dsmvc_gb300 import synthetic
    cands = synthetic.native_resolution_candidates(1920, 1080, range(500, 1001, 50))
    reqs = [r for c in cands for r in (c[3], c[4])]
    many = gb.build_plans(reqs, threads=8)
    assert len(many) == len(reqs)
    for req, p in zip(reqs, many):
        one = gb.AxisPlan(req, cached=False)
        assert p.hashes() == one.hashes()
        assert (p.source_size, p.destination_size) == (req.source_size, req.destination_size)


def test_failing_request_names_index(gb):
    good = product_request(gb, (100, 60, 60.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "mirror", 0))
    bad = product_request(gb, (100, 0, 60.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "mirror", 0))
    with pytest.raises(ValueError, match="plan 1"):
        gb.build_plans([good, bad, good], threads=2)
