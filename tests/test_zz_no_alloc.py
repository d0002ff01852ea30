"""The allocation-free 2D entry point (dsmvc_gb_inverse_2d_noalloc), for
callers that cannot allocate device memory: called through the C ABI on
device buffers, twice in a row, and checked against the executor's 2D entry
point within the parity tolerances of the other GPU tests.  This file is
collected last so that a run stopping at the first failure has already run
every other test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from common import INT_MAX_CODES, make_input, product_request

pytestmark = pytest.mark.gpu

STREAM_REL = 4e-7   # the executor may use the streaming kernels

CASES = [
    ("bicubic-f32", (480, 320, 320.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1),
     (270, 180, 180.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1), "f32"),
    ("lanczos3-u16", (1920, 1440, 1440.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0),
     (1080, 810, 810.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0), "u16"),
    ("spline36-u8", (300, 225, 225.0, 0.1, "spline36", 3, 0, 0.5, 1.0, "reflect101", 0),
     (200, 150, 150.0, 0.0, "spline36", 3, 0, 0.5, 1.0, "reflect101", 0), "u8"),
]


def _device(torch, arr):
    if arr.dtype == np.uint16:
        return torch.from_numpy(arr.view(np.int16)).cuda()
    return torch.from_numpy(arr).cuda()


def _host(t, dtype):
    a = t.cpu().numpy()
    return a.view(np.uint16) if dtype == np.uint16 else a


@pytest.mark.parametrize("name,hq,vq,sample", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_executor_twice(gb, executor, name, hq, vq, sample):
    torch = pytest.importorskip("torch")
    h = gb.AxisPlan(product_request(gb, hq))
    v = gb.AxisPlan(product_request(gb, vq))
    x = make_input(v.source_size, h.source_size, sample, 77) if sample != "f32" else \
        np.random.default_rng(77).random((v.source_size, h.source_size), dtype=np.float32)
    conv = gb.integer_conversion(8 if sample == "u8" else 16, False, False) if sample != "f32" else None
    want = executor.inverse_2d(h, v, x, conv)
    kind = {"f32": 0, "u8": 1, "u16": 2}[sample]
    dx = _device(torch, x)
    stream = torch.cuda.Stream()
    for _ in range(2):
        dy = torch.full((v.destination_size, h.destination_size), 0, dtype=dx.dtype, device="cuda")
        torch.cuda.synchronize()
        gb.inverse_2d_noalloc(h, v, kind, dx.data_ptr(), h.source_size, dy.data_ptr(),
                              h.destination_size, conv, stream.cuda_stream)
        stream.synchronize()
        got = _host(dy, x.dtype)
        if sample == "f32":
            assert np.max(np.abs(got - want)) <= STREAM_REL * np.max(np.abs(want))
        else:
            assert np.max(np.abs(got.astype(np.int64) - want.astype(np.int64))) <= INT_MAX_CODES


def test_noalloc_rejects_oversized_frames_and_float64(gb):
    big_h = gb.AxisPlan(product_request(gb, (7680, 5120, 5120.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1)))
    big_v = gb.AxisPlan(product_request(gb, (4320, 2880, 2880.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1)))
    assert 4 * big_v.source_size * big_h.destination_size > gb.NOALLOC_SCRATCH_BYTES
    with pytest.raises(ValueError, match="scratch"):
        gb.inverse_2d_noalloc(big_h, big_v, 0, 1 << 20, big_h.source_size, 1 << 21,
                              big_h.destination_size)
    f64 = gb.AxisPlan(product_request(gb, (64, 48, 48.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 2)))
    with pytest.raises(ValueError, match="Float64"):
        gb.inverse_2d_noalloc(f64, f64, 0, 1 << 20, 64, 1 << 21, 48)
