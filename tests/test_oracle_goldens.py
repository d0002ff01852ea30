"""The oracle against the reference's own golden vectors (CPU)."""
import numpy as np
import pytest

import oracle as O
from common import load_golden, oracle_request

G = load_golden("reference_goldens.json")


@pytest.mark.parametrize("fx", G["axis_fixtures"], ids=lambda f: f["name"])
def test_axis_fixture_hashes(fx):
    # tests/numerical_contract_tests.cpp:37-79 evaluate_fixture
    plan = O.Plan(oracle_request(fx["request"]))
    assert plan.half_bandwidth == fx["half_bandwidth"]
    assert plan.f32_hash() == fx["f32_plan"]
    assert plan.complete_hash() == fx["complete_plan"]
    x = O.make_normal_input(plan.source_size, fx["seed"])
    assert O.output_hash(plan.inverse_axis_f32(x)) == fx["production"]
    if plan.requires_float64:
        ordered = plan.inverse_axis_f64_ordered(x.astype(np.float64)).astype(np.float32)
    else:
        ordered = plan.inverse_axis_f32_ordered(x)
    assert O.output_hash(ordered) == fx["ordered"]


def test_fixture_conditioning_classes():
    rc = [O.Plan(oracle_request(f["request"])).normal_rcond for f in G["axis_fixtures"]]
    assert all(r >= 1e-4 for r in rc[:4]) and rc[5] >= 1e-4
    assert rc[4] < 1e-4 and rc[6] < 1e-4


def test_mixed_2d_hash():
    # tests/numerical_contract_tests.cpp:330-420 evaluate_f64_2d (safe x risky)
    m = G["mixed_2d"]
    h, v = O.Plan(oracle_request(m["horizontal"])), O.Plan(oracle_request(m["vertical"]))
    assert not h.requires_float64 and v.requires_float64
    packed = O.make_normal_input(v.source_size * h.source_size, m["seed"])
    x = np.full((v.source_size, h.source_size + m["input_pad"]), 7.0, np.float32)
    x[:, :h.source_size] = packed.reshape(v.source_size, h.source_size)
    y = O.inverse_2d(h, v, np.ascontiguousarray(x[:, :h.source_size]))
    assert O.output_hash(y) == m["production"]


def test_qr_anchor():
    a = G["qr_anchor"]
    plan = O.Plan(oracle_request(a["request"]))
    state = a["seed"]
    xs = []
    for _ in range(plan.source_size):
        state ^= (state << 13) & 0xFFFFFFFF
        state ^= state >> 17
        state ^= (state << 5) & 0xFFFFFFFF
        xs.append(float(np.float32(state & 0xFFFF) / np.float32(65535.0)))
    y = plan.inverse_axis_f64_ordered(np.array(xs))
    err = max(abs(y[0] - a["first"]), abs(y[-1] - a["last"]))
    bound = 4 * np.finfo(np.float64).eps / plan.normal_rcond * max(1.0, abs(a["first"]), abs(a["last"]))
    assert err <= bound


def test_bilinear_sixty_digit_anchor():
    a = G["bilinear_anchor"]
    plan = O.Plan(oracle_request(a["request"]))
    assert plan.requires_float64
    assert a["rcond_range"][0] < plan.normal_rcond < a["rcond_range"][1]
    state = a["seed"]
    xs = np.empty(plan.source_size, np.float32)
    for i in range(plan.source_size):
        state ^= (state << 13) & 0xFFFFFFFF
        state ^= state >> 17
        state ^= (state << 5) & 0xFFFFFFFF
        xs[i] = np.float32(state & 0xFFFF) / np.float32(65535.0)
    y = plan.inverse_axis_f32(xs)
    assert max(abs(float(y[0]) - a["first"]), abs(float(y[-1]) - a["last"])) < 3e-6


def test_padding_index_modes():
    # detail::padding_index, src/axis_plan.cpp:1024-1066
    pi = O.lib().orc_padding_index
    assert [pi(i, 4, 0) for i in (-1, 0, 3, 4)] == [-1, 0, 3, -1]
    assert [pi(i, 4, 1) for i in (-3, 5)] == [0, 3]
    assert [pi(i, 4, 2) for i in (-1, -2, 4, 5)] == [1, 2, 2, 1]
    assert [pi(i, 4, 3) for i in (-1, -2, 4, 5)] == [0, 1, 3, 2]
    assert [pi(i, 4, 4) for i in (-1, -4, -5, 8)] == [0, 3, -1, -1]
