"""Prepared batches (dsmvc_gb_batch_*): packed once, launched many times,
captured into a CUDA graph.  Bar: every launch writes exactly the bytes that
dsmvc_gb_run_batch writes for the same task list (same routing, same
kernels), and those match the oracle within the parity bars of
test_gpu_parity.py."""
import numpy as np
import pytest

import oracle as O
from common import INT_MAX_CODES, make_input, oracle_request, product_request

pytestmark = pytest.mark.gpu

# Luma and chroma axes of the 1080p -> 810p Lanczos-3 descale, at full size
# (streaming kernels) and a small bicubic pair (sequential kernels).
LUMA_H = (1920, 1440, 1440.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "symmetric", 1)
LUMA_V = (1080, 810, 810.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "symmetric", 1)
CHROMA_H = (960, 720, 720.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "symmetric", 1)
CHROMA_V = (540, 405, 405.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "symmetric", 1)
SMALL_H = (240, 160, 160.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1)
SMALL_V = (135, 90, 90.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1)


def _plan(gb, executor, req):
    p = gb.AxisPlan(product_request(gb, req), cached=False)
    executor.prepare(p)
    return p


def _tasks(gb, executor, torch, copies=2):
    geoms = [(LUMA_H, LUMA_V, "u16"), (CHROMA_H, CHROMA_V, "u16"), (SMALL_H, SMALL_V, "f32")]
    plans = {}
    tasks, inputs, outputs, meta = [], [], [], []
    for i, (hq, vq, sample) in enumerate(geoms * copies):
        h = plans.setdefault(hq, _plan(gb, executor, hq))
        v = plans.setdefault(vq, _plan(gb, executor, vq))
        x = make_input(v.source_size, h.source_size, sample, 300 + i)
        conv = gb.integer_conversion(16, i % 3 == 1, False) if sample == "u16" else None
        dx = torch.from_numpy(x.view(np.int16) if sample == "u16" else x).cuda()
        dy = torch.zeros((v.destination_size, h.destination_size), dtype=dx.dtype, device="cuda")
        inputs.append(dx)
        outputs.append(dy)
        meta.append((hq, vq, x, conv, sample))
        tasks.append(gb.PlaneTask(h, v, dx.data_ptr(), h.source_size, dy.data_ptr(),
                                  h.destination_size, 2 if sample == "u16" else 0, 0, conv))
    return tasks, inputs, outputs, meta


def _snapshot(outputs):
    return [y.cpu().numpy().copy() for y in outputs]


def test_prepared_batch_matches_run_batch(gb, executor):
    torch = pytest.importorskip("torch")
    tasks, _inputs, outputs, meta = _tasks(gb, executor, torch)
    sid = torch.cuda.current_stream().cuda_stream
    executor.run_batch(tasks, stream=sid, synchronize=True)
    want = _snapshot(outputs)
    batch = executor.prepare_batch(tasks)
    info = batch.info()
    assert info["kernel_launches"] >= 2 and info["scratch_bytes"] > 0 and info["table_bytes"] > 0
    for _ in range(3):
        for y in outputs:
            y.zero_()
        batch.launch(sid)
        batch.check(sid)
        for got, exp in zip(_snapshot(outputs), want):
            assert np.array_equal(got, exp)
    # One plane of each kind against the oracle's CPU scalar route.
    for (hq, vq, x, conv, sample), got in list(zip(meta, want))[:3]:
        oh, ov = O.Plan(oracle_request(hq)), O.Plan(oracle_request(vq))
        ref = O.inverse_2d(oh, ov, x, conv)
        if sample == "u16":
            diff = np.abs(got.view(np.uint16).astype(np.int64) - ref.astype(np.int64))
            assert diff.max() <= INT_MAX_CODES
        else:
            assert np.abs(got - ref).max() <= 2e-5


def test_prepared_batch_graph_replay(gb, executor):
    torch = pytest.importorskip("torch")
    tasks, _inputs, outputs, _meta = _tasks(gb, executor, torch, copies=1)
    batch = executor.prepare_batch(tasks)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        batch.launch(side.cuda_stream)       # warm launch outside the capture
    torch.cuda.synchronize()
    want = _snapshot(outputs)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        batch.launch(side.cuda_stream)
    for _ in range(2):
        for y in outputs:
            y.zero_()
        torch.cuda.synchronize()
        graph.replay()
        torch.cuda.synchronize()
        for got, exp in zip(_snapshot(outputs), want):
            assert np.array_equal(got, exp)
    batch.check(side.cuda_stream)


def test_prepared_batch_float64_status(gb, executor):
    torch = pytest.importorskip("torch")
    req = (40, 30, 30.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 2)
    p = _plan(gb, executor, req)
    x = np.random.default_rng(5).random((40, 40), dtype=np.float32)
    x[3, 7] = np.inf
    dx = torch.from_numpy(x).cuda()
    dy = torch.empty((30, 30), dtype=torch.float32, device="cuda")
    batch = executor.prepare_batch([gb.PlaneTask(p, p, dx.data_ptr(), 40, dy.data_ptr(), 30, 0, 0, None)])
    sid = torch.cuda.current_stream().cuda_stream
    batch.launch(sid)
    with pytest.raises(gb.DescaleError):
        batch.check(sid)
    # The status is cleared by the check; finite input then passes.
    dx.copy_(torch.from_numpy(np.random.default_rng(6).random((40, 40), dtype=np.float32)))
    batch.launch(sid)
    batch.check(sid)
    assert torch.isfinite(dy).all()


def test_unprepared_plans_use_the_device_plan_cache(gb):
    ex = gb.Executor(0)
    h = gb.AxisPlan(product_request(gb, SMALL_H), cached=False)
    v = gb.AxisPlan(product_request(gb, SMALL_V), cached=False)
    x = make_input(v.source_size, h.source_size, "f32", 41)
    first = ex.inverse_2d(h, v, x)
    s1 = ex.stats()
    second = ex.inverse_2d(h, v, x)
    s2 = ex.stats()
    assert np.array_equal(first, second)
    assert s1["plan_cache_misses"] == 2 and s2["plan_cache_misses"] == 2
    assert s2["plan_uploads"] == s1["plan_uploads"]
    # The repeated call reuses its slot's compiled launches (which hold the
    # cached plans); a different task list looks the plans up in the cache.
    assert s2["compile_reuses"] == s1["compile_reuses"] + 1
    assert s2["plan_cache_hits"] == s1["plan_cache_hits"]
    torch = pytest.importorskip("torch")
    dx = torch.from_numpy(x).cuda()
    dy = torch.zeros((v.destination_size, h.destination_size), dtype=torch.float32, device="cuda")
    side = torch.cuda.Stream()
    ex.run_batch([gb.PlaneTask(h, v, dx.data_ptr(), h.source_size, dy.data_ptr(), h.destination_size, 0, 0,
                               None)], stream=side.cuda_stream, synchronize=True)
    s3 = ex.stats()
    assert s3["plan_cache_hits"] == s2["plan_cache_hits"] + 2 and s3["plan_uploads"] == s1["plan_uploads"]
    assert np.array_equal(dy.cpu().numpy(), first)
    assert s2["plan_cache_bytes"] > 0
    ex.close()


def test_pipelined_host_planes_equal_single_calls(gb):
    """dsmvc_gb_inverse_2d_planes: many host planes pipelined in groups (1 MiB
    groups here, so most planes are in different groups) give exactly the
    per-plane calls' samples; a repeated call reuses its groups' compiled
    launches and device job tables with the same samples, and a call that
    fails on non-finite Float64 data leaves the next call correct."""
    from conftest import _executor_with
    # Whole vectors (no segments), so that groups and single calls run the
    # same arithmetic.
    ex = _executor_with(gb, "DSMVC_GB_PIPELINE_MB", "1", DSMVC_GB_SEGMENTS="1")
    geoms = [(CHROMA_H, CHROMA_V, "u16"), (SMALL_H, SMALL_V, "f32"),
             ((97, 67, 67.0, 0.1, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 2),
              (73, 51, 51.0, 0.0, "spline36", 3, 0, 0.5, 1.0, "reflect101", 2), "f32")]
    planes, want = [], []
    for i, (hq, vq, sample) in enumerate(geoms * 4):
        h = gb.AxisPlan(product_request(gb, hq), cached=False)
        v = gb.AxisPlan(product_request(gb, vq), cached=False)
        x = make_input(v.source_size, h.source_size, sample, 500 + i)
        conv = gb.integer_conversion(16, True, False) if sample == "u16" else None
        out = np.zeros((v.destination_size, h.destination_size), x.dtype)
        planes.append((h, v, x, out, conv))
        want.append(ex.inverse_2d(h, v, x, conv))
    ex.inverse_2d_planes(planes)
    for (_h, _v, _x, out, _c), w in zip(planes, want):
        assert np.array_equal(out, w)
    reuses = ex.stats()["compile_reuses"]
    for _h, _v, _x, out, _c in planes:
        out[...] = 0
    ex.inverse_2d_planes(planes)
    assert ex.stats()["compile_reuses"] > reuses
    for (_h, _v, _x, out, _c), w in zip(planes, want):
        assert np.array_equal(out, w)
    # Non-finite data in a Float64 plane fails the call.
    h, v, x, out, _ = planes[2]
    bad = x.copy()
    bad[1, 1] = np.inf
    with pytest.raises(gb.DescaleError):
        ex.inverse_2d_planes(planes[:2] + [(h, v, bad, out)])
    for _h, _v, _x, out, _c in planes:
        out[...] = 0
    ex.inverse_2d_planes(planes)
    for (_h, _v, _x, out, _c), w in zip(planes, want):
        assert np.array_equal(out, w)
    ex.close()


@pytest.mark.gpu
def test_pipelined_planes_in_one_ring(gb, whole_executor):
    """Planes packed back to back in one host buffer per direction travel in
    merged copies; a pitched plane (row padding on the host) in the middle
    and planes of odd byte sizes break the runs.  Every output equals the
    per-plane call, and the ring's bytes between planes stay untouched."""
    geoms = [(CHROMA_H, CHROMA_V), (SMALL_H, SMALL_V),
             ((97, 67, 67.0, 0.1, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 0),
              (73, 51, 51.0, 0.0, "spline36", 3, 0, 0.5, 1.0, "reflect101", 0))]
    plans = [(gb.AxisPlan(product_request(gb, hq), cached=False),
              gb.AxisPlan(product_request(gb, vq), cached=False)) for hq, vq in geoms]
    order = [0, 1, 2, 0, 0, 2, 1, 1, 0, 2]
    pitched = 4
    conv = gb.integer_conversion(16, True, False)
    sizes_in = [plans[k][1].source_size * plans[k][0].source_size for k in order]
    sizes_out = [plans[k][1].destination_size * plans[k][0].destination_size for k in order]
    ring_in = np.zeros(sum(sizes_in) + 64, np.uint16)
    ring_out = np.full(sum(sizes_out) + 64, 0xABCD, np.uint16)
    executor = whole_executor
    planes, want = [], []
    at_in = at_out = 0
    for i, k in enumerate(order):
        h, v = plans[k]
        x = make_input(v.source_size, h.source_size, "u16", 900 + i)
        if i == pitched:
            # Row padding on both sides: a pitched copy between the runs.
            xin = np.zeros((v.source_size, h.source_size + 5), np.uint16)[:, :h.source_size]
            xout = np.zeros((v.destination_size, h.destination_size + 3), np.uint16)[:, :h.destination_size]
            xin[...] = x
        else:
            xin = ring_in[at_in:at_in + x.size].reshape(x.shape)
            xin[...] = x
            xout = ring_out[at_out:at_out + sizes_out[i]].reshape(v.destination_size, h.destination_size)
            at_in += x.size
            at_out += sizes_out[i]
        planes.append((h, v, xin, xout, conv))
        want.append(executor.inverse_2d(h, v, x, conv))
    executor.inverse_2d_planes(planes)
    for (_h, _v, _x, out, _c), w in zip(planes, want):
        assert np.array_equal(out, w)
    assert np.all(ring_out[at_out:] == 0xABCD)


@pytest.mark.gpu
def test_pipelined_planes_direct_host_access(gb, whole_executor):
    """DSMVC_GB_HOST_DIRECT=1: page-locked planes are read and written by the
    kernels in place (no staging copies); pageable planes in the same call
    still travel by copies.  Every output equals the copying executor's."""
    torch = pytest.importorskip("torch")
    from conftest import _executor_with
    direct = _executor_with(gb, "DSMVC_GB_HOST_DIRECT", "1", DSMVC_GB_SEGMENTS="1")
    conv = gb.integer_conversion(16, True, False)
    h = gb.AxisPlan(product_request(gb, CHROMA_H), cached=False)
    v = gb.AxisPlan(product_request(gb, CHROMA_V), cached=False)
    planes, want = [], []
    for i in range(6):
        x = make_input(v.source_size, h.source_size, "u16", 700 + i)
        if i % 3 != 2:
            xin = torch.empty(x.shape, dtype=torch.int16, pin_memory=True).numpy().view(np.uint16)
            out = torch.zeros((v.destination_size, h.destination_size), dtype=torch.int16,
                              pin_memory=True).numpy().view(np.uint16)
        else:
            xin = np.empty_like(x)
            out = np.zeros((v.destination_size, h.destination_size), np.uint16)
        xin[...] = x
        planes.append((h, v, xin, out, conv))
        want.append(whole_executor.inverse_2d(h, v, x, conv))
    direct.inverse_2d_planes(planes)
    for (_h, _v, _x, out, _c), w in zip(planes, want):
        assert np.array_equal(out, w)
    direct.close()


def test_two_part_batch_matches_one_part(gb, whole_executor):
    """A batch of eight or more tasks that owns its scratch is split into two
    parts launched on a forked stream; on whole vectors (results independent
    of launch composition) both splits write the same bytes, directly and
    replayed from a CUDA graph."""
    torch = pytest.importorskip("torch")
    tasks, _inputs, outputs, _meta = _tasks(gb, whole_executor, torch, copies=3)
    assert len(tasks) >= 8
    sid = torch.cuda.current_stream().cuda_stream
    one = whole_executor.prepare_batch(tasks, parts=1)
    assert one.info()["parts"] == 1
    one.launch(sid)
    one.check(sid)
    want = _snapshot(outputs)
    auto = whole_executor.prepare_batch(tasks)
    two = whole_executor.prepare_batch(tasks, parts=2)
    assert auto.info()["parts"] == 2 and two.info()["parts"] == 2
    assert two.info()["kernel_launches"] >= one.info()["kernel_launches"]
    for batch in (auto, two):
        for y in outputs:
            y.zero_()
        batch.launch(sid)
        batch.check(sid)
        for got, exp in zip(_snapshot(outputs), want):
            assert np.array_equal(got, exp)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        two.launch(side.cuda_stream)
    for _ in range(2):
        for y in outputs:
            y.zero_()
        torch.cuda.synchronize()
        graph.replay()
        torch.cuda.synchronize()
        for got, exp in zip(_snapshot(outputs), want):
            assert np.array_equal(got, exp)
    two.check(sid)
