"""Optional Float64 residual refinement (DSMVC_GB_F64_REFINE=1): after each
pass of the Float64 2D route, r = A^T b - G x is evaluated with the plan's
Float64 weights and unfactored normal band, G d = r is solved with the
LDL^T factor and x += d.

Bars (written into each test):
  * the refined route keeps the Float64 contract: <= 1 float32 ULP (1 code)
    of the CPU scalar Float64 route;
  * on an ill-conditioned plan (Lanczos2 1080 -> 980, rcond 3.95e-6, which
    automatic mode sends to Float64) it moves the output to the exact
    solution of the plan's Float64 system (its weights and stored normal
    band), computed here in extended precision (numpy longdouble): at most
    3 samples differ from the correctly rounded exact result, no more than
    without refinement, none by more than 1 ULP.
"""
import numpy as np
import pytest

import oracle as O
from common import F64_MAX_ULP, INT_MAX_CODES, make_input, max_ulp, oracle_request, product_request

pytestmark = pytest.mark.gpu

ILL_H = (1080, 980, 978.1, 0.95, "lanczos", 2, 0, 0.5, 1.0, "symmetric", 0)
FORCED_V = (160, 120, 120.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 2)
FORCED_H = (300, 200, 200.0, 0.0, "spline36", 3, 0, 0.5, 1.0, "reflect101", 2)


@pytest.fixture(scope="module")
def refine_executor(gb):
    from conftest import _executor_with
    ex = _executor_with(gb, "DSMVC_GB_F64_REFINE", "1")
    yield ex
    ex.close()


def _axis_exact(plan, data):
    """Extended-precision solve of the plan's Float64 system for every row of
    `data` (rows x source): G^-1 A^T b with the plan's Float64 weights and
    its stored normal band G (the system the refinement targets), the right
    side accumulated and G factored and solved in numpy longdouble."""
    L = np.longdouble
    n, hb = plan.destination_size, plan.half_bandwidth
    off = plan.array("transpose_offsets").astype(np.int64)
    idx = plan.array("transpose_indices").astype(np.int64)
    w = plan.array("transpose_weights_f64").astype(L)
    g = plan.array("normal_bands_f64").reshape(hb + 1, n).astype(L)
    x = data.astype(L)
    rhs = np.stack([(x[:, idx[off[i]:off[i + 1]]] * w[off[i]:off[i + 1]]).sum(axis=1) for i in range(n)], axis=1)
    # Banded LDL^T (unit L) in longdouble.
    f = g.copy()
    for i in range(n):
        end = min(hb + 1, n - i)
        for dd in range(1, end):
            m = f[dd, i] / f[0, i]
            for o in range(end - dd):
                f[o, i + dd] -= m * f[dd + o, i]
        for dd in range(1, end):
            f[dd, i] /= f[0, i]
    y = rhs.copy()
    for i in range(n):
        for dd in range(1, min(hb, i) + 1):
            y[:, i] -= f[dd, i - dd] * y[:, i - dd]
    y /= f[0]
    for i in range(n - 2, -1, -1):
        for dd in range(1, min(hb, n - 1 - i) + 1):
            y[:, i] -= f[dd, i] * y[:, i + dd]
    return y


def test_refined_route_keeps_the_contract(gb, refine_executor):
    for hq, vq in ((FORCED_H, FORCED_V), (ILL_H, FORCED_V)):
        h = gb.AxisPlan(product_request(gb, hq), cached=False)
        v = gb.AxisPlan(product_request(gb, vq), cached=False)
        assert h.requires_float64 and v.requires_float64
        oh, ov = O.Plan(oracle_request(hq)), O.Plan(oracle_request(vq))
        x = make_input(v.source_size, h.source_size, "f32", 41)
        refine_executor.profile(True)
        got = refine_executor.inverse_2d(h, v, x)
        names = {k["name"] for k in refine_executor.kernel_times()}
        refine_executor.profile(False)
        assert {"refine_f64/rows", "refine_f64/columns"} <= {n.rsplit("/hb", 1)[0] for n in names}, names
        assert max_ulp(got, O.inverse_2d(oh, ov, x)) <= F64_MAX_ULP
        xi = make_input(v.source_size, h.source_size, "u16", 42)
        conv = gb.integer_conversion(16, False, False)
        goti = refine_executor.inverse_2d(h, v, xi, conv)
        wanti = O.inverse_2d(oh, ov, xi, conv)
        assert np.max(np.abs(goti.astype(np.int64) - wanti.astype(np.int64))) <= INT_MAX_CODES


def test_refinement_moves_towards_the_exact_solution(gb, executor, refine_executor):
    h = gb.AxisPlan(product_request(gb, ILL_H), cached=False)
    v = gb.AxisPlan(product_request(gb, FORCED_V), cached=False)
    assert h.normal_rcond < 1e-4 and h.requires_float64
    rng = np.random.default_rng(9)
    x = rng.random((v.source_size, h.source_size), dtype=np.float32)
    exact = _axis_exact(v, _axis_exact(h, x).T).T.astype(np.float32)
    plain = executor.inverse_2d(h, v, x)
    refined = refine_executor.inverse_2d(h, v, x)
    miss_plain = int(np.count_nonzero(plain != exact))
    miss_refined = int(np.count_nonzero(refined != exact))
    print(f"samples differing from the rounded exact solution: direct {miss_plain}, refined {miss_refined}")
    assert miss_refined <= miss_plain and miss_refined <= 3
    assert max_ulp(refined, exact) <= 1
