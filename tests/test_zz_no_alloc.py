"""The allocation-free 2D entry point (dsmvc_gb_inverse_2d_noalloc), for
callers that cannot allocate device memory -- code running inside another
framework's memory pool, or a real-time loop that must never call into the
allocator.  It is called through the C ABI on device buffers, twice in a row,
and checked bit for bit against the oracle's statement of the sequential
kernels' operation order and against the executor's 2D entry point within
the parity tolerances of the other GPU tests.  The second call must leave the
device's free memory unchanged.  Its plan uploads come from pageable host
memory, so it refuses a stream that is being captured.  This file is
collected last so that a run stopping at the first failure has already run
every other test; it also passes alone in a fresh process."""
import numpy as np
import pytest

import oracle as O
from common import INT_MAX_CODES, make_input, oracle_request, product_request

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
def test_noalloc_matches_oracle_and_executor_twice(gb, executor, name, hq, vq, sample):
    torch = pytest.importorskip("torch")
    h = gb.AxisPlan(product_request(gb, hq))
    v = gb.AxisPlan(product_request(gb, vq))
    x = make_input(v.source_size, h.source_size, sample, 77) if sample != "f32" else \
        np.random.default_rng(77).random((v.source_size, h.source_size), dtype=np.float32)
    conv = gb.integer_conversion(8 if sample == "u8" else 16, False, False) if sample != "f32" else None
    want = executor.inverse_2d(h, v, x, conv)
    # The sequential kernels follow the reference CUDA operation order.
    order = O.inverse_2d_gpu_order(O.Plan(oracle_request(hq)), O.Plan(oracle_request(vq)), x, conv)
    kind = {"f32": 0, "u8": 1, "u16": 2}[sample]
    dx = _device(torch, x)
    outs = [torch.full((v.destination_size, h.destination_size), 0, dtype=dx.dtype, device="cuda")
            for _ in range(2)]
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    free = []
    for dy in outs:
        gb.inverse_2d_noalloc(h, v, kind, dx.data_ptr(), h.source_size, dy.data_ptr(),
                              h.destination_size, conv, stream.cuda_stream)
        stream.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        got = _host(dy, x.dtype)
        assert np.array_equal(got, order)
        if sample == "f32":
            assert np.max(np.abs(got - want)) <= STREAM_REL * np.max(np.abs(want))
        else:
            assert np.max(np.abs(got.astype(np.int64) - want.astype(np.int64))) <= INT_MAX_CODES
    # The first call has loaded the kernels and located the scratch array;
    # the second allocates nothing.
    assert free[1] == free[0]


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


def test_noalloc_integer_output_counts_the_forward_plane(gb):
    """A frame whose intermediate fits the scratch array with room to spare
    but not together with the forward plane that u16 output needs: accepted
    for Float32 sizes on paper, rejected for u16."""
    h = gb.AxisPlan(product_request(gb, (4096, 2048, 2048.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 0)))
    v = gb.AxisPlan(product_request(gb, (3000, 1500, 1500.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 0)))
    mid = 4 * v.source_size * h.destination_size
    fwd = 4 * v.destination_size * h.destination_size
    plans = h.storage_bytes + v.storage_bytes
    assert mid + plans < gb.NOALLOC_SCRATCH_BYTES < mid + fwd
    conv = gb.integer_conversion(16, False, False)
    with pytest.raises(ValueError, match="scratch"):
        gb.inverse_2d_noalloc(h, v, 2, 1 << 20, h.source_size, 1 << 21, h.destination_size, conv)


def test_noalloc_refuses_a_capturing_stream(gb, executor):
    torch = pytest.importorskip("torch")
    h = gb.AxisPlan(product_request(gb, CASES[0][1]))
    v = gb.AxisPlan(product_request(gb, CASES[0][2]))
    dx = torch.zeros((v.source_size, h.source_size), dtype=torch.float32, device="cuda")
    dy = torch.zeros((v.destination_size, h.destination_size), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        graph.capture_begin()
        try:
            with pytest.raises(ValueError, match="captured"):
                gb.inverse_2d_noalloc(h, v, 0, dx.data_ptr(), h.source_size, dy.data_ptr(),
                                      h.destination_size, None, stream.cuda_stream)
        finally:
            graph.capture_end()
    torch.cuda.synchronize()
