"""GPU parity: the CUDA path through the C ABI against the oracle.

Bars (written into each test):
  * sequential kernels, Float32: bit-exact against the oracle's statement of
    the reference CUDA operation order (fmaf chains), and within the
    reference's Float32 tolerance of the CPU scalar route (max-abs 2e-5,
    mean-abs 1e-6, tests/vs_gpu_concurrency.py:57);
  * streaming kernels (chunk-delayed backward pass), Float32: within
    STREAM_REL (4e-7) of the largest output magnitude of that same CUDA-order
    result, and within the reference tolerance of the CPU scalar route;
  * integer output: within 1 code of the CPU scalar route;
  * Float64 route: within 1 float32 ULP (1 code) of the CPU scalar Float64
    route, the contract, with the default fused two-pass kernels; equal to it
    bit for bit with the kernels that reproduce its operation order
    (DSMVC_GB_F64_EXACT=1) and with the sequential Float64 kernels.
"""
import numpy as np
import pytest

import oracle as O
from common import (F32_MAX_ABS, F32_MEAN_ABS, F64_MAX_ULP, INT_MAX_CODES, load_golden, make_input,
                    max_ulp, oracle_request, product_request)

pytestmark = pytest.mark.gpu

STREAM_REL = 4e-7   # streaming vs sequential CUDA order, relative to max |x|


def plans(gb, executor, req, prepare=True):
    p = gb.AxisPlan(product_request(gb, req), cached=False)
    if prepare:
        executor.prepare(p)
    return p, O.Plan(oracle_request(req))


def image(rows, cols, seed):
    rng = np.random.default_rng(seed)
    return rng.random((rows, cols), dtype=np.float32)


HB_CASES = [
    ("bilinear", (90, 61, 61.0, 0.0, "bilinear", 3, 0, 0.5, 1.0, "symmetric", 1)),
    ("bicubic", (90, 61, 61.0, 0.3, "bicubic", 3, 0, 0.5, 1.0, "reflect101", 1)),
    ("lanczos3", (90, 61, 60.5, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 1)),
    ("spline64", (90, 61, 61.0, -0.2, "spline64", 3, 0, 0.5, 1.0, "zero", 1)),
    ("spline64-blur-hb9", (90, 61, 61.0, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 1)),
    ("lanczos6-hb11", (120, 70, 70.0, 0.0, "lanczos", 6, 0, 0.5, 1.0, "mirror", 1)),
    ("lanczos7-generic-hb13", (120, 70, 70.0, 0.0, "lanczos", 7, 0, 0.5, 1.0, "symmetric", 1)),
    ("dest-1-hb0", (9, 1, 1.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1)),
]


@pytest.mark.parametrize("name,req", HB_CASES, ids=[c[0] for c in HB_CASES])
def test_rows_and_columns_bit_exact(gb, seq_executor, name, req):
    executor = seq_executor
    p, o = plans(gb, executor, req)
    x = image(37, p.source_size, 1)
    got = executor.inverse_rows(p, x)
    assert np.array_equal(got, O.inverse_rows_gpu_order(o, x))
    scalar = O.inverse_rows(o, x)
    assert np.max(np.abs(got - scalar)) <= F32_MAX_ABS * max(1.0, np.max(np.abs(scalar)))
    xc = image(p.source_size, 29, 2)
    gotc = executor.inverse_columns(p, xc)
    assert np.array_equal(gotc, O.inverse_columns_gpu_order(o, xc))


CASES_2D = [
    ("c0-shape-small", (240, 160, 160.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1),
     (135, 90, 90.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1)),
    ("lanczos3-repeat", (192, 144, 144.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0),
     (108, 81, 81.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0)),
    ("mitchell-blur-odd", (161, 107, 106.5, 0.2, "bicubic", 3, 1 / 3, 1 / 3, 1.1, "mirror", 0),
     (93, 61, 61.0, -0.1, "bicubic", 3, 1 / 3, 1 / 3, 1.1, "mirror", 0)),
    ("spline36-x-bilinear", (100, 77, 77.0, 0.0, "spline36", 3, 0, 0.5, 1.0, "zero", 0),
     (64, 49, 49.0, 0.0, "bilinear", 3, 0, 0.5, 1.0, "zero", 0)),
]


@pytest.mark.parametrize("name,hq,vq", CASES_2D, ids=[c[0] for c in CASES_2D])
def test_2d_float32(gb, executor, seq_executor, name, hq, vq):
    h, oh = plans(gb, seq_executor, hq)
    v, ov = plans(gb, seq_executor, vq)
    executor.prepare(h)
    executor.prepare(v)
    x = image(v.source_size, h.source_size, 3)
    exact = O.inverse_2d_gpu_order(oh, ov, x)
    scalar = O.inverse_2d(oh, ov, x)
    seq = seq_executor.inverse_2d(h, v, x)
    assert np.array_equal(seq, exact)
    got = executor.inverse_2d(h, v, x)
    assert np.max(np.abs(got - exact)) <= STREAM_REL * np.max(np.abs(exact))
    for y in (seq, got):
        err = np.abs(y.astype(np.float64) - scalar)
        assert err.max() <= F32_MAX_ABS and err.mean() <= F32_MEAN_ABS


def _random_geometries(count, seed):
    """Seeded 2D geometries over every kernel family, border and ratios
    1.0-2.4: gather windows of 4 to 16 samples, partial last chunks and
    half-bandwidths 1 to 7 (the Debilinear 192x108 -> 112x63 shape among
    them)."""
    rng = np.random.default_rng(seed)
    kernels = [("bilinear", 3, 0, 0.5), ("bicubic", 3, 0, 0.5), ("bicubic", 3, 1 / 3, 1 / 3),
               ("lanczos", 3, 0, 0.5), ("lanczos", 4, 0, 0.5), ("spline16", 3, 0, 0.5),
               ("spline36", 3, 0, 0.5)]
    borders = ["zero", "repeat", "reflect101", "symmetric", "mirror"]
    out = [((192, 112, 112.0, 0.0, "bilinear", 3, 0, 0.5, 1.0, "mirror", 0),
            (108, 63, 63.0, 0.0, "bilinear", 3, 0, 0.5, 1.0, "mirror", 0))]
    for i in range(count):
        k, taps, b, c = kernels[i % len(kernels)]
        border = borders[int(rng.integers(len(borders)))]
        axes = []
        for src in (int(rng.integers(40, 420)), int(rng.integers(24, 260))):
            dst = max(8, min(src, int(round(src / rng.uniform(1.0, 2.4)))))
            axes.append((src, dst, float(dst), 0.0, k, taps, b, c, 1.0, border, 0))
        out.append(tuple(axes))
    return out


RANDOM_2D = _random_geometries(28, 99)


@pytest.mark.parametrize("hq,vq", RANDOM_2D, ids=[f"g{i}" for i in range(len(RANDOM_2D))])
def test_2d_random_geometries(gb, executor, whole_executor, paired_executor, hq, vq):
    """Random geometries: the default executor (which splits a lone plane's
    vectors into segments where admitted) within the reference tolerance of
    the CPU scalar route; whole vectors on the unpaired and the paired
    kernels bit for bit alike."""
    h, oh = plans(gb, executor, hq)
    v, ov = plans(gb, executor, vq)
    x = image(v.source_size, h.source_size, 11)
    scalar = O.inverse_2d(oh, ov, x)
    got = executor.inverse_2d(h, v, x)
    assert np.array_equal(whole_executor.inverse_2d(h, v, x), paired_executor.inverse_2d(h, v, x))
    err = np.abs(got.astype(np.float64) - scalar)
    assert err.max() <= F32_MAX_ABS and err.mean() <= F32_MEAN_ABS, (hq, vq, err.max())
    xi = make_input(v.source_size, h.source_size, "u16", 12)
    conv = gb.integer_conversion(16, False, False)
    goti = executor.inverse_2d(h, v, xi, conv)
    wanti = O.inverse_2d(oh, ov, xi, conv)
    assert np.abs(goti.astype(np.int64) - wanti.astype(np.int64)).max() <= INT_MAX_CODES


def _varied_requests(count, seed):
    """Seeded 2D requests away from the defaults: shifts, active lengths
    below the destination size, blur, every built-in kernel family with
    Lanczos 2 to 5 and Spline64, f64mode automatic or forced."""
    rng = np.random.default_rng(seed)
    kernels = [("bilinear", 3, 0, 0.5), ("bicubic", 3, 0, 0.5), ("bicubic", 3, 1 / 3, 1 / 3),
               ("lanczos", 2, 0, 0.5), ("lanczos", 3, 0, 0.5), ("lanczos", 5, 0, 0.5),
               ("spline16", 3, 0, 0.5), ("spline36", 3, 0, 0.5), ("spline64", 3, 0, 0.5)]
    borders = ["zero", "repeat", "reflect101", "symmetric", "mirror"]
    out = []
    for i in range(count):
        k, taps, b, c = kernels[i % len(kernels)]
        border = borders[int(rng.integers(len(borders)))]
        mode = (0, 0, 2)[i % 3]
        axes = []
        for src in (int(rng.integers(32, 300)), int(rng.integers(24, 200))):
            dst = max(8, min(src, int(round(src / rng.uniform(1.0, 2.2)))))
            active = float(dst) if rng.random() < 0.5 else float(dst) - float(rng.uniform(0.0, 1.0))
            blur = 1.0 if rng.random() < 0.6 else float(rng.uniform(0.9, 1.3))
            axes.append((src, dst, active, float(rng.uniform(-0.5, 0.5)), k, taps, b, c, blur, border, mode))
        out.append(tuple(axes))
    return out


REQUESTS_2D = _varied_requests(27, 404)


@pytest.mark.parametrize("hq,vq", REQUESTS_2D, ids=[f"r{i}" for i in range(len(REQUESTS_2D))])
def test_2d_random_requests(gb, executor, hq, vq):
    """Random requests with shifts, blur and forced Float64: the Float32
    route within the reference tolerance of the CPU scalar route, the
    Float64 route within 1 float32 ULP of it, integer output within 1 code."""
    h, oh = plans(gb, executor, hq)
    v, ov = plans(gb, executor, vq)
    x = image(v.source_size, h.source_size, 21)
    got = executor.inverse_2d(h, v, x)
    want = O.inverse_2d(oh, ov, x)
    if h.requires_float64 or v.requires_float64:
        assert max_ulp(got, want) <= F64_MAX_ULP, (hq, vq)
    else:
        err = np.abs(got.astype(np.float64) - want)
        assert err.max() <= F32_MAX_ABS and err.mean() <= F32_MEAN_ABS, (hq, vq, err.max())
    for bits, sample in ((8, "u8"), (16, "u16")):
        xi = make_input(v.source_size, h.source_size, sample, 22)
        conv = gb.integer_conversion(bits, False, False)
        goti = executor.inverse_2d(h, v, xi, conv)
        wanti = O.inverse_2d(oh, ov, xi, conv)
        assert np.abs(goti.astype(np.int64) - wanti.astype(np.int64)).max() <= INT_MAX_CODES, (hq, vq, sample)


@pytest.mark.parametrize("sample", ["u8", "u16"])
@pytest.mark.parametrize("name,hq,vq", CASES_2D[:3], ids=[c[0] for c in CASES_2D[:3]])
def test_2d_integer(gb, executor, seq_executor, sample, name, hq, vq):
    h, oh = plans(gb, seq_executor, hq)
    v, ov = plans(gb, seq_executor, vq)
    executor.prepare(h)
    executor.prepare(v)
    x = make_input(v.source_size, h.source_size, sample, 11)
    bits = 8 if sample == "u8" else 16
    conv = gb.integer_conversion(bits, chroma=False, full_range=False)
    exact = O.inverse_2d_gpu_order(oh, ov, x, conv)
    assert np.array_equal(seq_executor.inverse_2d(h, v, x, conv), exact)
    got = executor.inverse_2d(h, v, x, conv)
    assert np.max(np.abs(got.astype(np.int64) - exact.astype(np.int64))) <= INT_MAX_CODES
    scalar = O.inverse_2d(oh, ov, x, conv)
    assert np.max(np.abs(got.astype(np.int64) - scalar.astype(np.int64))) <= INT_MAX_CODES


F64_CASES = [
    ("forced-both", (97, 67, 67.0, 0.1, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 2),
     (73, 51, 51.0, 0.0, "spline36", 3, 0, 0.5, 1.0, "reflect101", 2)),
    ("auto-risk-horizontal", (1080, 980, 978.1, 0.95, "lanczos", 2, 0, 0.5, 1.0, "symmetric", 0),
     (40, 30, 30.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 0)),
    ("auto-risk-vertical", (40, 30, 30.0, 0.0, "bilinear", 3, 0, 0.5, 1.0, "symmetric", 0),
     (1920, 1734, 1732.0888888888887, 0.9555555555556339, "bilinear", 3, 0, 0.5, 1.0, "symmetric", 0)),
    ("forced-spline64-blur-hb9", (128, 86, 85.5, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 2),
     (72, 48, 48.0, 0.0, "lanczos", 7, 0, 0.5, 1.0, "symmetric", 2)),
]


@pytest.mark.parametrize("order", ["fused", "exact"])
@pytest.mark.parametrize("name,hq,vq", F64_CASES, ids=[c[0] for c in F64_CASES])
def test_2d_float64_route(gb, executor, f64_exact_executor, name, hq, vq, order):
    ex = executor if order == "fused" else f64_exact_executor
    h, oh = plans(gb, ex, hq)
    v, ov = plans(gb, ex, vq)
    assert h.requires_float64 or v.requires_float64
    x = image(v.source_size, h.source_size, 5)
    got = ex.inverse_2d(h, v, x)
    want = O.inverse_2d(oh, ov, x)
    xi = make_input(v.source_size, h.source_size, "u16", 6)
    conv = gb.integer_conversion(16, chroma=True, full_range=False)
    goti = ex.inverse_2d(h, v, xi, conv)
    wanti = O.inverse_2d(oh, ov, xi, conv)
    if order == "exact":
        assert max_ulp(got, want) == 0
        assert np.array_equal(goti, wanti)
    else:
        assert max_ulp(got, want) <= F64_MAX_ULP
        assert np.max(np.abs(goti.astype(np.int64) - wanti.astype(np.int64))) <= INT_MAX_CODES


def test_float64_rows_and_columns(gb, executor):
    req = (73, 61, 60.5, 0.125, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 2)
    p, o = plans(gb, executor, req)
    x = image(19, p.source_size, 8)
    assert max_ulp(executor.inverse_rows(p, x), O.inverse_rows(o, x)) == 0
    xc = image(p.source_size, 23, 9)
    assert max_ulp(executor.inverse_columns(p, xc), O.inverse_columns(o, xc)) == 0


@pytest.mark.parametrize("case", load_golden("reference_outputs.json")["cases"],
                         ids=lambda c: c["name"])
def test_against_reference_engine_outputs(gb, executor, f64_exact_executor, case):
    h, oh = plans(gb, executor, case["horizontal"])
    v, ov = plans(gb, executor, case["vertical"])
    x = make_input(v.source_size, h.source_size, case["sample"], case["seed"])
    got = executor.inverse_2d(h, v, x, case["conversion"])
    if h.requires_float64 or v.requires_float64:
        # The Float64 route in the CPU's operation order reproduces the
        # reference CPU output bit for bit; the fused one is within the
        # contract of it.
        exact = f64_exact_executor.inverse_2d(h, v, x, case["conversion"])
        assert O.output_hash(exact.astype(np.float32)) == case["output_hash"]
        if case["sample"] == "f32":
            assert max_ulp(got, exact) <= F64_MAX_ULP
        else:
            assert np.max(np.abs(got.astype(np.int64) - exact.astype(np.int64))) <= INT_MAX_CODES
    else:
        want = O.inverse_2d(oh, ov, x, case["conversion"])
        assert O.output_hash(want.astype(np.float32)) == case["output_hash"]
        if case["sample"] == "f32":
            scale = max(1.0, float(np.max(np.abs(want))))
            assert np.max(np.abs(got - want)) <= F32_MAX_ABS * scale
        else:
            assert np.max(np.abs(got.astype(np.int64) - want.astype(np.int64))) <= INT_MAX_CODES


def test_strides_and_padding_are_respected(gb, executor):
    # include/dsmvc/engine.hpp:231-235: row padding is neither read nor written.
    hq, vq = CASES_2D[0][1], CASES_2D[0][2]
    h, oh = plans(gb, executor, hq)
    v, ov = plans(gb, executor, vq)
    x = image(v.source_size, h.source_size, 12)
    xin = np.full((v.source_size, h.source_size + 5), np.nan, np.float32)
    xin[:, :h.source_size] = x
    out = np.full((v.destination_size, h.destination_size + 3), -777.0, np.float32)
    executor.inverse_2d(h, v, xin[:, :h.source_size], out=out[:, :h.destination_size])
    assert np.all(out[:, h.destination_size:] == -777.0)
    # The same samples as a call on contiguous planes, within tolerance of
    # the CPU scalar route.
    assert np.array_equal(out[:, :h.destination_size], executor.inverse_2d(h, v, x))
    err = np.abs(out[:, :h.destination_size].astype(np.float64) - O.inverse_2d(oh, ov, x))
    assert err.max() <= F32_MAX_ABS and err.mean() <= F32_MEAN_ABS


def test_strides_and_padding_streaming(gb, executor):
    hq, vq = CASES_2D[1][1], CASES_2D[1][2]
    h, oh = plans(gb, executor, hq)
    v, ov = plans(gb, executor, vq)
    x = make_input(v.source_size, h.source_size, "u16", 31)
    conv = gb.integer_conversion(16, chroma=False, full_range=False)
    xin = np.full((v.source_size, h.source_size + 8), 0xFFFF, np.uint16)
    xin[:, :h.source_size] = x
    out = np.full((v.destination_size, h.destination_size + 5), 0xBEEF, np.uint16)
    executor.inverse_2d(h, v, xin[:, :h.source_size], conv, out=out[:, :h.destination_size])
    assert np.all(out[:, h.destination_size:] == 0xBEEF)
    scalar = O.inverse_2d(oh, ov, x, conv)
    assert np.max(np.abs(out[:, :h.destination_size].astype(np.int64) - scalar)) <= INT_MAX_CODES


FULL = [
    ("c1-luma-lanczos3-u16", (1920, 1440, 1440.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0),
     (1080, 810, 810.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0), "u16"),
    ("c1-chroma-lanczos3-u16", (960, 720, 720.0, 0.25 - 0.25 * 1440 / 1920, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0),
     (540, 405, 405.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0), "u16"),
    ("c0-bicubic-f32", (1920, 1280, 1280.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1),
     (1080, 720, 720.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1), "f32"),
]


@pytest.mark.parametrize("name,hq,vq,sample", FULL, ids=[c[0] for c in FULL])
def test_full_size_frames_use_streaming_kernels(gb, executor, whole_executor, paired_executor, name, hq, vq,
                                                sample):
    """Full-size frames of the benchmark configurations: the paired
    streaming kernels run (profiled kernel names), give the same samples as
    the unpaired ones on whole vectors, and the default executor (segments)
    agrees with the CPU scalar route within the reference tolerance."""
    h, oh = plans(gb, executor, hq)
    v, ov = plans(gb, executor, vq)
    assert h.stream_info()["eligible"] and v.stream_info()["eligible"]
    x = make_input(v.source_size, h.source_size, sample, 41) if sample != "f32" else \
        image(v.source_size, h.source_size, 41)
    conv = gb.integer_conversion(16, chroma="chroma" in name, full_range=False) if sample != "f32" else None
    executor.profile(True)
    got = executor.inverse_2d(h, v, x, conv)
    names = {k["name"] for k in executor.kernel_times()}
    executor.profile(False)
    assert any(n.startswith("tstream_f32/rows") for n in names), names
    assert any(n.startswith("tstream_f32/columns") for n in names), names
    paired_executor.profile(True)
    paired = paired_executor.inverse_2d(h, v, x, conv)
    names = {k["name"] for k in paired_executor.kernel_times()}
    paired_executor.profile(False)
    assert any(n.startswith("tstream2_f32/rows") for n in names), names
    assert any(n.startswith("tstream2_f32/columns") for n in names), names
    assert np.array_equal(whole_executor.inverse_2d(h, v, x, conv), paired)
    scalar = O.inverse_2d(oh, ov, x, conv)
    if sample == "f32":
        err = np.abs(got.astype(np.float64) - scalar)
        assert err.max() <= F32_MAX_ABS and err.mean() <= F32_MEAN_ABS
    else:
        assert np.max(np.abs(got.astype(np.int64) - scalar.astype(np.int64))) <= INT_MAX_CODES


ROW_COL_STREAM = [
    ("lanczos3-rows", (400, 300, 300.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0)),
    ("bicubic-odd", (333, 217, 216.5, 0.25, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1)),
    ("bilinear-zero", (250, 200, 200.0, 0.0, "bilinear", 3, 0, 0.5, 1.0, "zero", 0)),
]


@pytest.mark.parametrize("name,req", ROW_COL_STREAM, ids=[c[0] for c in ROW_COL_STREAM])
def test_rows_and_columns_streaming(gb, executor, name, req):
    """One-axis calls on the streaming kernels (rows: adjacent samples,
    columns: strided), several chunks long."""
    p, o = plans(gb, executor, req)
    assert p.stream_info()["eligible"]
    x = image(45, p.source_size, 51)
    want = O.inverse_rows_gpu_order(o, x)
    got = executor.inverse_rows(p, x)
    assert np.max(np.abs(got - want)) <= STREAM_REL * np.max(np.abs(want))
    xc = image(p.source_size, 47, 52)
    wantc = O.inverse_columns_gpu_order(o, xc)
    gotc = executor.inverse_columns(p, xc)
    assert np.max(np.abs(gotc - wantc)) <= STREAM_REL * np.max(np.abs(wantc))


def test_unprepared_plans_still_run(gb, executor):
    req = (50, 40, 40.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1)
    p, o = plans(gb, executor, req, prepare=False)
    x = image(5, 50, 13)
    assert np.array_equal(executor.inverse_rows(p, x), O.inverse_rows_gpu_order(o, x))


def test_float64_nonfinite_input_raises(gb, executor):
    req = (40, 30, 30.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 2)
    p, _ = plans(gb, executor, req)
    x = image(30 + 10, 40, 14)
    x[3, 7] = np.inf
    with pytest.raises(gb.DescaleError):
        executor.inverse_2d(p, p, x[:40, :40])
    # The executor stays usable after the error.
    y = executor.inverse_2d(p, p, image(40, 40, 15))
    assert np.all(np.isfinite(y))


def test_device_batch_matches_host_calls(gb, whole_executor):
    """Whole vectors: a device batch gives the host calls' samples bit for
    bit (with segments, the split depends on the launch's size)."""
    executor = whole_executor
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    tasks, expect, keep = [], [], []
    geoms = [(CASES_2D[0][1], CASES_2D[0][2], "f32"), (CASES_2D[1][1], CASES_2D[1][2], "u16"),
             (CASES_2D[2][1], CASES_2D[2][2], "f32"), (F64_CASES[0][1], F64_CASES[0][2], "u8")]
    for i, (hq, vq, sample) in enumerate(geoms * 2):
        h, oh = plans(gb, executor, hq)
        v, ov = plans(gb, executor, vq)
        x = make_input(v.source_size, h.source_size, sample, 100 + i)
        conv = gb.integer_conversion(8 if sample == "u8" else 16, False, False) if sample != "f32" else None
        # uint16 planes travel as int16 tensors (same bytes).
        dx = torch.from_numpy(x.view(np.int16) if sample == "u16" else x).cuda()
        dy = torch.empty((v.destination_size, h.destination_size), dtype=dx.dtype, device="cuda")
        keep += [dx, dy, h, v]
        tasks.append(gb.PlaneTask(h, v, dx.data_ptr(), h.source_size, dy.data_ptr(),
                                  h.destination_size, {"f32": 0, "u8": 1, "u16": 2}[sample], 0, conv))
        expect.append((dy, executor.inverse_2d(h, v, x, conv), sample))
    executor.run_batch(tasks, stream=torch.cuda.current_stream().cuda_stream, synchronize=True)
    for dy, want, sample in expect:
        got = dy.cpu().numpy()
        if sample == "u16":
            got = got.view(np.uint16)
        assert np.array_equal(got, want)


WIDE_2D = [
    ("spline64-blur-hb9", (384, 256, 256.0, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 0),
     (216, 144, 144.0, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 0)),
    ("lanczos4-blur-hb9", (300, 197, 197.0, 0.1, "lanczos", 4, 0, 0.5, 1.1, "mirror", 0),
     (170, 121, 121.0, 0.0, "lanczos", 4, 0, 0.5, 1.1, "mirror", 0)),
    ("lanczos6-hb11", (240, 200, 200.0, 0.0, "lanczos", 6, 0, 0.5, 1.0, "symmetric", 0),
     (135, 112, 112.0, 0.0, "lanczos", 6, 0, 0.5, 1.0, "symmetric", 0)),
]


@pytest.mark.parametrize("name,hq,vq", CASES_2D + WIDE_2D, ids=[c[0] for c in CASES_2D + WIDE_2D])
def test_two_pass_kernels_are_bit_exact(gb, exact_executor, name, hq, vq):
    """The two-pass transposing kernels run the reference CUDA operation
    order without approximation: Float32 output equals the oracle's CUDA
    order bit for bit, integer output too; the kernels run (profiled names)
    whenever the plans are not Float64."""
    h, oh = plans(gb, exact_executor, hq)
    v, ov = plans(gb, exact_executor, vq)
    x = image(v.source_size, h.source_size, 61)
    exact_executor.profile(True)
    got = exact_executor.inverse_2d(h, v, x)
    names = {k["name"] for k in exact_executor.kernel_times()}
    exact_executor.profile(False)
    if not (h.requires_float64 or v.requires_float64):
        assert any(n.startswith("tsolve_f32/rows") for n in names), names
        assert any(n.startswith("tsolve_f32/columns") for n in names), names
        assert np.array_equal(got, O.inverse_2d_gpu_order(oh, ov, x))
        xi = make_input(v.source_size, h.source_size, "u16", 62)
        conv = gb.integer_conversion(16, False, False)
        goti = exact_executor.inverse_2d(h, v, xi, conv)
        assert np.array_equal(goti, O.inverse_2d_gpu_order(oh, ov, xi, conv))


@pytest.mark.parametrize("name,hq,vq", WIDE_2D, ids=[c[0] for c in WIDE_2D])
def test_wide_bands_use_two_pass_kernels(gb, executor, name, hq, vq):
    """Half-bandwidths 9 and 11 (no chunk-delayed kernel, or factors that
    decay too slowly for it) run on the two-pass kernels by default."""
    h, oh = plans(gb, executor, hq)
    v, ov = plans(gb, executor, vq)
    x = image(v.source_size, h.source_size, 63)
    executor.profile(True)
    got = executor.inverse_2d(h, v, x)
    names = {k["name"] for k in executor.kernel_times()}
    executor.profile(False)
    assert any(n.startswith("tsolve_f32") for n in names), names
    scalar = O.inverse_2d(oh, ov, x)
    err = np.abs(got.astype(np.float64) - scalar)
    assert err.max() <= F32_MAX_ABS and err.mean() <= F32_MEAN_ABS


F64_TRANSPOSED = [
    ("bicubic-forced", (300, 200, 200.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 2),
     (170, 113, 113.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 2)),
    ("lanczos3-forced-repeat", (257, 190, 190.0, 0.3, "lanczos", 3, 0, 0.5, 1.0, "repeat", 2),
     (143, 101, 101.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 2)),
    ("spline64-blur-hb9-forced", (384, 256, 256.0, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 2),
     (216, 144, 144.0, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 2)),
]


@pytest.mark.parametrize("order", ["fused", "exact"])
@pytest.mark.parametrize("sample", ["f32", "u16"])
@pytest.mark.parametrize("name,hq,vq", F64_TRANSPOSED, ids=[c[0] for c in F64_TRANSPOSED])
def test_float64_transposing_kernels(gb, executor, f64_exact_executor, sample, name, hq, vq, order):
    """Both axes retaining Float64: the Float64 two-pass transposing kernels
    run (profiled names); in the CPU scalar route's operation order they give
    its output bit for bit, fused they stay within the contract (<= 1 float
    ULP, <= 1 code)."""
    executor = executor if order == "fused" else f64_exact_executor
    h, oh = plans(gb, executor, hq)
    v, ov = plans(gb, executor, vq)
    assert h.requires_float64 and v.requires_float64
    x = make_input(v.source_size, h.source_size, sample, 71)
    conv = gb.integer_conversion(16, False, False) if sample == "u16" else None
    executor.profile(True)
    got = executor.inverse_2d(h, v, x, conv)
    names = {k["name"] for k in executor.kernel_times()}
    executor.profile(False)
    assert any(n.startswith("tsolve_f64/rows") for n in names), names
    assert any(n.startswith("tsolve_f64/columns") for n in names), names
    want = O.inverse_2d(oh, ov, x, conv)
    if order == "exact":
        if sample == "u16":
            assert np.array_equal(got, want)
        else:
            assert max_ulp(got, want) == 0
    elif sample == "u16":
        assert np.max(np.abs(got.astype(np.int64) - want.astype(np.int64))) <= INT_MAX_CODES
    else:
        assert max_ulp(got, want) <= F64_MAX_ULP
