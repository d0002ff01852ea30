"""Ring residency of the streaming kernels, replayed on the CPU.

For every plan the host admits to a streaming kernel, the kernel's ring
feeder is replayed sample by sample from the packed records exactly as the
kernel runs it, and every nonzero gather weight must find its source sample
resident in the ring when its destination is computed:

  * 1D kernels (stream_impl.cuh): one refill per destination up to that
    destination's window end, in granules of 4 (f32 rows and all column
    loads), 8 (u16 rows) or 16 (u8 rows) samples, single samples at the tail;
  * 2D transposing kernels (tstream_impl.cuh): one refill per group of four
    destinations up to max(window start of the group's first record, window
    start of its last record) + window, in blocks of 16, single samples at
    the tail; padding records past the last destination take part.

A plan whose group refill looked only at a padding record's start once read
two unloaded samples (Debilinear 108 -> 63); this test covers that shape.
"""
import numpy as np
import pytest

RING = 32
CHUNK = 32


def _records(p):
    info = p.stream_info(records=True)
    if not info["eligible"]:
        return None, info
    starts = info["forward"][:, 0].copy().view(np.int32).astype(int)
    return (starts, info["forward"][:, 4:4 + info["window"]]), info


def _replay_1d(starts, weights, n, m, kw, granule):
    ring = {}
    have = 0
    misses = []
    for j in range(n):
        s0 = starts[j]
        while have < s0 + kw:
            step = granule if have + granule <= m else 1
            for s in range(have, have + step):
                ring[s % RING] = s
            have += step
        for k in range(kw):
            if weights[j, k] != 0 and ring.get((s0 + k) % RING) != s0 + k:
                misses.append((j, s0 + k))
    return misses


def _replay_2d(starts, weights, n, m, kw):
    ring = {}
    have = 0
    misses = []
    padded = len(starts)
    for j in range(padded):
        if j % 4 == 0:
            need = min(max(starts[j], starts[j + 3]) + kw, m)
            while have < need:
                step = 16 if have + 16 <= m else 1
                for s in range(have, have + step):
                    ring[s % RING] = s
                have += step
        if j >= n:
            continue
        s0 = starts[j]
        for k in range(kw):
            if weights[j, k] != 0 and ring.get((s0 + k) % RING) != s0 + k:
                misses.append((j, s0 + k))
    return misses


def _plans(gb):
    rng = np.random.default_rng(4321)
    kernels = [("bilinear", 3), ("bicubic", 3), ("lanczos", 3), ("lanczos", 2), ("spline16", 3),
               ("spline36", 3)]
    borders = ["zero", "repeat", "reflect101", "symmetric", "mirror"]
    reqs = []
    for i in range(160):
        src = int(rng.integers(16, 400))
        ratio = float(rng.uniform(1.0, 2.4))
        dst = max(8, min(src, int(round(src / ratio))))
        k, taps = kernels[i % len(kernels)]
        reqs.append(gb.AxisRequest(src, dst, float(dst), 0.0, k, taps, 0.0, 0.5, 1.0,
                                   borders[i % len(borders)], 0))
    # The Debilinear shape that exposed the padding-record refill.
    reqs.append(gb.AxisRequest(108, 63, 63.0, 0.0, "bilinear", 3, 0.0, 0.5, 1.0, "mirror", 0))
    reqs.append(gb.AxisRequest(192, 112, 112.0, 0.0, "bilinear", 3, 0.0, 0.5, 1.0, "mirror", 0))
    return [gb.AxisPlan(r, cached=False) for r in reqs]


def test_streaming_rings_hold_every_window(gb):
    checked_1d = checked_2d = 0
    for p in _plans(gb):
        rec, info = _records(p)
        if rec is None:
            continue
        starts, weights = rec
        n, m, kw = p.destination_size, p.source_size, info["window"]
        assert len(starts) % CHUNK == 0 and len(starts) >= n
        assert all(starts[j] <= starts[j + 1] for j in range(len(starts) - 1))
        assert starts[n - 1] + kw <= m
        for granule, ok in ((4, True), (8, info["ring_ok_u16"]), (16, info["ring_ok_u8"])):
            if ok:
                assert _replay_1d(starts, weights, n, m, kw, granule) == [], (p.request, granule)
                checked_1d += 1
        if info["ring_ok_transposed"]:
            assert _replay_2d(starts, weights, n, m, kw) == [], p.request
            checked_2d += 1
    assert checked_1d > 100 and checked_2d > 50


def test_padding_records_repeat_the_last_window_start(gb):
    p = gb.AxisPlan(gb.AxisRequest(108, 63, 63.0, 0.0, "bilinear", 3, 0.0, 0.5, 1.0, "mirror", 0),
                    cached=False)
    (starts, _w), info = _records(p)
    assert info["eligible"] and len(starts) == 64
    assert starts[63] == starts[62]
