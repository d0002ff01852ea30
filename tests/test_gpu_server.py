"""Request loop (dsmvc_gb_server_*): continuous batching of mixed requests.

Bars:
  * every request's output is bit-identical alone and in the mix (requests
    submitted together, batched with others, on several workers);
  * outputs match the oracle's CPU scalar route within the parity bars
    (Float32 max-abs 2e-5; integer 1 code; Float64 route 1 float ULP);
  * a small memory budget still serves everything (smaller batches), a
    request larger than the budget is refused, and a Float64 request with
    non-finite input fails alone while the requests batched with it succeed.
"""
import numpy as np
import pytest

import oracle as O
from common import F32_MAX_ABS, INT_MAX_CODES, make_input, max_ulp

pytestmark = pytest.mark.gpu

KERNELS = [("bilinear", 3, 0.0, 0.5), ("bicubic", 3, 0.0, 0.5), ("lanczos", 3, 0.0, 0.5),
           ("spline36", 3, 0.0, 0.5)]
SIZES = [(320, 180), (480, 270), (640, 360)]


def _request_specs(count, seed):
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        w, h = SIZES[int(rng.integers(len(SIZES)))]
        ratio = float(rng.choice([0.5, 0.6, 0.67, 0.75, 0.9]))
        k = KERNELS[int(rng.integers(len(KERNELS)))]
        f64 = 2 if rng.random() < 0.2 else 0
        yuv = bool(rng.random() < 0.5)
        specs.append((w, h, ratio, k, f64, yuv, 1000 + i))
    return specs


def _even(v):
    v = int(round(v))
    return v + (v & 1)


def _build(gb, spec, plans):
    """Planes of one request: (h, v, input, conversion, oracle plans)."""
    w, h, ratio, (k, taps, b, c), f64, yuv, seed = spec
    dw, dh = _even(w * ratio), _even(h * ratio)
    shapes = [(w, h, dw, dh)] + ([(w // 2, h // 2, dw // 2, dh // 2)] * 2 if yuv else [])
    planes = []
    for idx, (sw, sh, ow, oh) in enumerate(shapes):
        key = (sw, sh, ow, oh, k, taps, f64)
        if key not in plans:
            hr = gb.AxisRequest(sw, ow, float(ow), 0.0, k, taps, b, c, 1.0, "mirror", f64)
            vr = gb.AxisRequest(sh, oh, float(oh), 0.0, k, taps, b, c, 1.0, "mirror", f64)
            plans[key] = (gb.AxisPlan(hr, cached=False), gb.AxisPlan(vr, cached=False),
                          O.Plan(O.make_request(sw, ow, float(ow), 0.0, k, taps, b, c, 1.0, "mirror", f64)),
                          O.Plan(O.make_request(sh, oh, float(oh), 0.0, k, taps, b, c, 1.0, "mirror", f64)))
        ph, pv, oph, opv = plans[key]
        sample = "u16" if yuv else "f32"
        x = make_input(sh, sw, sample, seed * 7 + idx)
        conv = gb.integer_conversion(16, idx > 0, False) if yuv else None
        planes.append((ph, pv, x, conv, oph, opv))
    return planes


def _submit(server, planes):
    outs = [np.zeros((pv.destination_size, ph.destination_size), x.dtype) for ph, pv, x, _c, _a, _b in planes]
    ticket = server.submit([(ph, pv, x, o, conv) for (ph, pv, x, conv, _a, _b), o in zip(planes, outs)])
    return ticket, outs


@pytest.fixture(scope="module")
def requests(gb):
    plans = {}
    return [_build(gb, s, plans) for s in _request_specs(36, 5)]


@pytest.mark.parametrize("mode", ["whole", "segments"])
def test_alone_and_in_the_mix_are_identical(gb, executor, whole_executor, requests, mode):
    """Each request's result alone equals its result in the mix: bit for bit
    on whole vectors; with segments (the default, whose split depends on
    the batch's size) within 1 code for integer samples, 4e-7 of the largest
    magnitude for Float32 samples, and bit for bit for Float64 plans."""
    ex = whole_executor if mode == "whole" else executor
    server = gb.Server(ex, memory_budget=1 << 30, streams=4, max_batch=16)
    alone = []
    for planes in requests:
        t, outs = _submit(server, planes)
        server.wait(t)
        alone.append(outs)
    submitted = [_submit(server, planes) for planes in requests]
    for t, _outs in submitted:
        server.wait(t)
    stats = server.stats()
    server.close()
    for planes, a, (_t, m) in zip(requests, alone, submitted):
        for (ph, pv, *_rest), x, y in zip(planes, a, m):
            if mode == "whole" or ph.requires_float64 or pv.requires_float64:
                assert np.array_equal(x, y)
            elif x.dtype == np.uint16:
                assert np.abs(x.astype(np.int64) - y.astype(np.int64)).max() <= 1
            else:
                assert np.abs(x - y).max() <= 4e-7 * max(1.0, float(np.abs(x).max()))
    assert stats["completed"] == 2 * len(requests) and stats["failed"] == 0
    assert stats["batches"] < stats["completed"]           # the mix was batched
    assert 0 < stats["latency_p50_ms"] <= stats["latency_p99_ms"] <= stats["latency_max_ms"]
    # Against the oracle.
    for planes, outs in zip(requests[:12], alone[:12]):
        for (ph, pv, x, conv, oph, opv), got in zip(planes, outs):
            want = O.inverse_2d(oph, opv, x, conv)
            if x.dtype == np.uint16:
                assert np.abs(got.astype(np.int64) - want.astype(np.int64)).max() <= INT_MAX_CODES
            elif ph.requires_float64 or pv.requires_float64:
                assert max_ulp(got, want) <= 1
            else:
                assert np.abs(got.astype(np.float64) - want).max() <= F32_MAX_ABS


def test_small_budget_and_oversized_request(gb, executor, requests):
    server = gb.Server(executor, memory_budget=24 << 20, streams=2, max_batch=64)
    tickets = [_submit(server, planes) for planes in requests[:10]]
    for t, _ in tickets:
        server.wait(t)
    s = server.stats()
    assert s["completed"] == 10 and s["failed"] == 0
    assert s["peak_device_bytes"] <= 24 << 20
    big = gb.AxisPlan(gb.AxisRequest(3840, 2560, 2560.0, 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "mirror", 0),
                      cached=False)
    bigv = gb.AxisPlan(gb.AxisRequest(2160, 1440, 1440.0, 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "mirror", 0),
                       cached=False)
    x = np.zeros((2160, 3840), np.float32)
    out = np.zeros((1440, 2560), np.float32)
    with pytest.raises(OverflowError):
        server.submit([(big, bigv, x, out)])
    server.close()


def test_float64_failure_is_isolated(gb, executor):
    server = gb.Server(executor, memory_budget=1 << 30, streams=1, max_batch=8)
    h = gb.AxisPlan(gb.AxisRequest(96, 64, 64.0, 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "mirror", 2), cached=False)
    v = gb.AxisPlan(gb.AxisRequest(54, 36, 36.0, 0.0, "bicubic", 3, 0.0, 0.5, 1.0, "mirror", 2), cached=False)
    good = [make_input(54, 96, "f32", s) for s in range(4)]
    bad = make_input(54, 96, "f32", 9)
    bad[5, 5] = np.nan
    outs = [np.zeros((36, 64), np.float32) for _ in range(5)]
    # Hold the single worker with a first request so the next five share a batch.
    tickets = [server.submit([(h, v, x, o)]) for x, o in zip(good[:2] + [bad] + good[2:], outs)]
    results = []
    for t in tickets:
        try:
            server.wait(t)
            results.append(True)
        except gb.DescaleError:
            results.append(False)
    assert results == [True, True, False, True, True]
    ref = executor.inverse_2d(h, v, good[0])
    assert np.array_equal(outs[0], ref)
    server.close()
