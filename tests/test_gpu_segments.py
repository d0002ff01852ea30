"""Segments of the chunk-delayed transposing passes: a plane's vectors split
into ranges of whole chunks served by different warps, each range's
forward substitution started one chunk early from a zero history.

Bars: against whole vectors, Float32 samples within 4e-7 of the largest
output magnitude and integer samples within 1 code; against the CPU scalar
route, the reference tolerance (max-abs 2e-5, mean-abs 1e-6; 1 code)."""
import numpy as np
import pytest

import oracle as O
from common import F32_MAX_ABS, F32_MEAN_ABS, INT_MAX_CODES, make_input, max_ulp, oracle_request, product_request
from conftest import _executor_with

pytestmark = pytest.mark.gpu

GEOMS = [
    ("c1-luma-u16", (1920, 1440, 1440.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0),
     (1080, 810, 810.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0), "u16"),
    ("c0-bicubic-f32", (1920, 1280, 1280.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1),
     (1080, 720, 720.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1), "f32"),
    ("odd-bilinear-u8", (333, 217, 216.5, 0.25, "bilinear", 3, 0, 0.5, 1.0, "zero", 0),
     (301, 200, 199.75, -0.3, "bilinear", 3, 0, 0.5, 1.0, "mirror", 0), "u8"),
    ("spline36-tail-f32", (600, 449, 449.0, 0.1, "spline36", 3, 0, 0.5, 1.0, "reflect101", 0),
     (500, 417, 417.0, 0.0, "spline36", 3, 0, 0.5, 1.0, "symmetric", 0), "f32"),
]


@pytest.fixture(scope="module", params=[2, 3, 7])
def forced(gb, request):
    ex = _executor_with(gb, "DSMVC_GB_SEGMENTS", str(request.param))
    yield ex
    ex.close()


@pytest.mark.parametrize("name,hq,vq,sample", GEOMS, ids=[g[0] for g in GEOMS])
def test_segments_match_whole_vectors(gb, forced, whole_executor, name, hq, vq, sample):
    h = gb.AxisPlan(product_request(gb, hq), cached=False)
    v = gb.AxisPlan(product_request(gb, vq), cached=False)
    assert h.stream_info()["segmentable"] and v.stream_info()["segmentable"]
    x = make_input(v.source_size, h.source_size, sample, 77)
    conv = gb.integer_conversion(8 if sample == "u8" else 16, False, False) if sample != "f32" else None
    got = forced.inverse_2d(h, v, x, conv)
    whole = whole_executor.inverse_2d(h, v, x, conv)
    scalar = O.inverse_2d(O.Plan(oracle_request(hq)), O.Plan(oracle_request(vq)), x, conv)
    if sample == "f32":
        assert np.abs(got - whole).max() <= 4e-7 * max(1.0, float(np.abs(whole).max()))
        err = np.abs(got.astype(np.float64) - scalar)
        assert err.max() <= F32_MAX_ABS and err.mean() <= F32_MEAN_ABS
    else:
        assert np.abs(got.astype(np.int64) - whole.astype(np.int64)).max() <= 1
        assert np.abs(got.astype(np.int64) - scalar.astype(np.int64)).max() <= INT_MAX_CODES


def test_segments_are_launched(gb, forced, whole_executor):
    """The forced split multiplies the chunk-delayed jobs (the job table
    grows); the automatic one splits a lone plane and keeps a large batch
    whole."""
    torch = pytest.importorskip("torch")
    _name, hq, vq, _s = GEOMS[1]
    h = gb.AxisPlan(product_request(gb, hq), cached=False)
    v = gb.AxisPlan(product_request(gb, vq), cached=False)
    dx = torch.zeros((v.source_size, h.source_size), dtype=torch.float32, device="cuda")
    dy = torch.zeros((v.destination_size, h.destination_size), dtype=torch.float32, device="cuda")
    task = gb.PlaneTask(h, v, dx.data_ptr(), h.source_size, dy.data_ptr(), h.destination_size, 0, 0, None)
    sizes = {}
    for label, ex in (("forced", forced), ("whole", whole_executor)):
        b = ex.prepare_batch([task])
        sizes[label] = b.info()["table_bytes"]
        b.close()
    assert sizes["forced"] > sizes["whole"]


F64_GEOMS = [
    ("bicubic-forced", (960, 640, 640.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "mirror", 2),
     (540, 360, 360.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "mirror", 2)),
    ("spline64-blur-forced", (1280, 853, 853.0, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 2),
     (720, 480, 480.0, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 2)),
]


@pytest.mark.parametrize("sample", ["f32", "u16"])
@pytest.mark.parametrize("name,hq,vq", F64_GEOMS, ids=[g[0] for g in F64_GEOMS])
def test_float64_segments(gb, forced, whole_executor, name, hq, vq, sample):
    """Float64 two-pass kernels in segments (forward and backward margins of
    2-4 chunks, admitted below 2^-60): within the <= 1 float ULP / 1 code
    contract of the CPU scalar Float64 route and of whole vectors."""
    h = gb.AxisPlan(product_request(gb, hq), cached=False)
    v = gb.AxisPlan(product_request(gb, vq), cached=False)
    assert h.stream_info()["f64_segmentable"]
    x = make_input(v.source_size, h.source_size, sample, 91)
    conv = gb.integer_conversion(16, False, False) if sample == "u16" else None
    got = forced.inverse_2d(h, v, x, conv)
    whole = whole_executor.inverse_2d(h, v, x, conv)
    want = O.inverse_2d(O.Plan(oracle_request(hq)), O.Plan(oracle_request(vq)), x, conv)
    if sample == "u16":
        assert np.abs(got.astype(np.int64) - want.astype(np.int64)).max() <= 1
        assert np.abs(got.astype(np.int64) - whole.astype(np.int64)).max() <= 1
    else:
        assert max_ulp(got, want) <= 1 and max_ulp(got, whole) <= 1


def test_float64_segments_are_launched(gb, forced, whole_executor):
    torch = pytest.importorskip("torch")
    _name, hq, vq = F64_GEOMS[0]
    h = gb.AxisPlan(product_request(gb, hq), cached=False)
    v = gb.AxisPlan(product_request(gb, vq), cached=False)
    dx = torch.zeros((v.source_size, h.source_size), dtype=torch.float32, device="cuda")
    dy = torch.zeros((v.destination_size, h.destination_size), dtype=torch.float32, device="cuda")
    task = gb.PlaneTask(h, v, dx.data_ptr(), h.source_size, dy.data_ptr(), h.destination_size, 0, 0, None)
    sizes = {}
    for label, ex in (("forced", forced), ("whole", whole_executor)):
        b = ex.prepare_batch([task])
        sizes[label] = (b.info()["table_bytes"], b.info()["scratch_bytes"])
        b.close()
    assert sizes["forced"][0] > sizes["whole"][0] and sizes["forced"][1] > sizes["whole"][1]


TWO_PASS_GEOMS = [
    ("spline64-blur-hb9", (768, 512, 512.0, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 0),
     (432, 288, 288.0, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 0), "f32"),
    ("c1-luma-exact-u16", (1920, 1440, 1440.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0),
     (1080, 810, 810.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0), "u16"),
]


@pytest.fixture(scope="module", params=[2, 5])
def forced_exact(gb, request):
    ex = _executor_with(gb, "DSMVC_GB_EXACT", "1", DSMVC_GB_SEGMENTS=str(request.param))
    yield ex
    ex.close()


@pytest.mark.parametrize("name,hq,vq,sample", TWO_PASS_GEOMS, ids=[g[0] for g in TWO_PASS_GEOMS])
def test_two_pass_segments(gb, forced_exact, exact_executor, name, hq, vq, sample):
    """Two-pass Float32 kernels in segments (margins of 1-4 chunks admitted
    below 2^-26): within 4e-7 of the largest magnitude (1 code) of whole
    vectors, which follow the reference CUDA order bit for bit, and within
    the reference tolerance of the CPU scalar route."""
    h = gb.AxisPlan(product_request(gb, hq), cached=False)
    v = gb.AxisPlan(product_request(gb, vq), cached=False)
    assert h.stream_info()["exact_margin"] and v.stream_info()["exact_margin"]
    x = make_input(v.source_size, h.source_size, sample, 93)
    conv = gb.integer_conversion(16, False, False) if sample != "f32" else None
    forced_exact.profile(True)
    got = forced_exact.inverse_2d(h, v, x, conv)
    names = {k["name"] for k in forced_exact.kernel_times()}
    forced_exact.profile(False)
    assert any(n.startswith("tsolve_f32") for n in names), names
    whole = exact_executor.inverse_2d(h, v, x, conv)
    scalar = O.inverse_2d(O.Plan(oracle_request(hq)), O.Plan(oracle_request(vq)), x, conv)
    if sample == "f32":
        assert np.abs(got - whole).max() <= 4e-7 * max(1.0, float(np.abs(whole).max()))
        err = np.abs(got.astype(np.float64) - scalar)
        assert err.max() <= F32_MAX_ABS and err.mean() <= F32_MEAN_ABS
    else:
        assert np.abs(got.astype(np.int64) - whole.astype(np.int64)).max() <= 1
        assert np.abs(got.astype(np.int64) - scalar.astype(np.int64)).max() <= INT_MAX_CODES
