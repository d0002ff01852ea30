"""Host logic of the streaming kernels (CPU): eligibility, record layout, and
a numpy emulation of the kernel's algorithm on the packed records (exact
forward pass, chunk-delayed backward pass with a zero-carry warm-up) checked
against the oracle's reference CUDA operation order."""
import numpy as np
import pytest

import oracle as O
from common import oracle_request, product_request


def fma32(a, b, c):
    return (np.float64(a) * np.float64(b) + np.float64(c)).astype(np.float32)


def emulate(info, plan, x):
    """x: (vectors, m) float32 -> (vectors, n) float32, kernel algorithm."""
    fwd, bwd = info["forward"], info["backward"]
    K, hb, n, LC = info["window"], plan.half_bandwidth, plan.destination_size, info["chunk"]
    V = x.shape[0]
    y = np.zeros((V, n), np.float32)
    for j in range(n):
        rec = fwd[j]
        s0 = int(rec[:1].view(np.int32)[0])
        s = np.zeros(V, np.float32)
        for k in range(K):
            s = fma32(rec[4 + k], x[:, s0 + k], s)
        for q in range(hb):
            d = hb - q
            prev = y[:, j - d] if j - d >= 0 else np.zeros(V, np.float32)
            s = fma32(rec[4 + K + q], prev, s)
        y[:, j] = s * rec[1]

    def back(lo, hi, carry, yv):
        """Backward over [lo, hi) from carry (x_{hi..hi+hb-1}); returns x."""
        xs = {hi + e: carry[e] for e in range(hb)}
        out = {}
        for j in range(hi - 1, lo - 1, -1):
            s = np.zeros(V, np.float32)
            if j < n:
                for q in range(hb):
                    d = q + 1 if hb == 3 else hb - q
                    s = fma32(bwd[j, q], xs.get(j + d, np.zeros(V, np.float32)), s)
                v = (yv[:, j] - s).astype(np.float32)
            else:
                v = np.zeros(V, np.float32)
            xs[j] = v
            out[j] = v
        return out

    chunks = (n + LC - 1) // LC
    zero = [np.zeros(V, np.float32)] * hb
    res = np.zeros((V, n), np.float32)
    for c in range(chunks):
        lo, hi = c * LC, (c + 1) * LC
        if c == chunks - 1:
            carry = zero
        elif c + 1 == chunks - 1:
            nxt = back(hi, hi + LC, zero, y)
            carry = [nxt[hi + e] if hi + e < n else np.zeros(V, np.float32) for e in range(hb)]
        else:
            warm = back(hi, hi + LC, zero, y)
            carry = [warm[hi + e] for e in range(hb)]
        xs = back(lo, hi, carry, y)
        for j in range(lo, min(hi, n)):
            res[:, j] = xs[j]
    return res


CASES = [
    ("lanczos3-1920-1440", (1920, 1440, 1440.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0), True),
    ("lanczos3-chroma-v", (540, 405, 405.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "repeat", 0), True),
    ("bicubic-1080-720", (1080, 720, 720.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 1), True),
    ("bilinear-odd", (201, 150, 149.5, 0.3, "bilinear", 3, 0, 0.5, 1.0, "zero", 0), True),
    ("spline64-hb7", (300, 200, 200.0, -0.2, "spline64", 3, 0, 0.5, 1.0, "reflect101", 0), True),
    ("short-single-chunk", (40, 30, 30.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "mirror", 0), True),
    ("spline64-blur-hb9", (300, 200, 200.0, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 0), False),
    ("f64-forced", (100, 70, 70.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "symmetric", 2), False),
]


@pytest.mark.parametrize("name,req,eligible", CASES, ids=[c[0] for c in CASES])
def test_stream_eligibility_and_emulation(gb, name, req, eligible):
    p = gb.AxisPlan(product_request(gb, req), cached=False)
    info = p.stream_info(records=True)
    assert bool(info["eligible"]) == eligible, info["reason"]
    if not eligible:
        assert info["reason"]
        return
    assert info["backward_transfer"] <= 2.0 ** -26
    o = O.Plan(oracle_request(req))
    rng = np.random.default_rng(3)
    x = rng.random((6, p.source_size), dtype=np.float32)
    got = emulate(info, o, x)
    want = np.stack([o.inverse_axis_f32_gpu(r) for r in x])
    scale = float(np.max(np.abs(want)))
    assert np.max(np.abs(got - want)) <= 4e-7 * scale
    # The forward pass is exact: the last chunk's outputs equal the oracle's.
    last = (p.destination_size - 1) // info["chunk"] * info["chunk"]
    assert np.max(np.abs(got[:, last:] - want[:, last:])) <= 2e-7 * scale


def test_record_layout(gb):
    req = (47, 39, 39.0, -0.3125, "bicubic", 3, 0, 0.5, 1.0, "reflect101", 1)
    p = gb.AxisPlan(product_request(gb, req), cached=False)
    info = p.stream_info(records=True)
    assert info["eligible"] and info["window"] % 4 == 0
    off = p.array("transpose_offsets")
    idx = p.array("transpose_indices")
    w = p.array("transpose_weights")
    lower = p.array("lower_ld").reshape(p.half_bandwidth, -1)
    upper = p.array("upper_l").reshape(p.half_bandwidth, -1)
    K, hb = info["window"], p.half_bandwidth
    prev = 0
    for j in range(p.destination_size):
        rec = info["forward"][j]
        s0 = int(rec[:1].view(np.int32)[0])
        assert s0 >= prev and 0 <= s0 <= p.source_size - K
        prev = s0
        dense = np.zeros(K, np.float32)
        dense[idx[off[j]:off[j + 1]] - s0] = w[off[j]:off[j + 1]]
        assert np.array_equal(rec[4:4 + K], dense)
        assert rec[1] == p.array("inverse_diagonal")[j]
        for q in range(hb):
            d = hb - q
            assert rec[4 + K + q] == (-lower[d - 1, j] if d <= j else 0.0)
            du = q + 1  # half-bandwidth 3: ascending
            assert info["backward"][j, q] == (upper[du - 1, j] if du <= min(hb, p.destination_size - j - 1) else 0.0)


def forward_transfer(p, chunk):
    """Largest state left by a unit history pushed through one chunk's
    homogeneous forward recurrence (chunks 1 .. chunks-2), in float64."""
    n, hb = p.destination_size, p.half_bandwidth
    lower = p.array("lower_ld").astype(np.float64).reshape(hb, n)
    inv = p.array("inverse_diagonal").astype(np.float64)
    chunks = (n + chunk - 1) // chunk
    worst = 0.0
    for k in range(1, chunks - 1):
        lo = k * chunk
        for e in range(hb):
            y = {lo - 1 - e: 1.0}
            for t in range(lo, lo + chunk):
                y[t] = -inv[t] * sum(lower[d - 1, t] * y.get(t - d, 0.0) for d in range(1, min(hb, t) + 1))
            worst = max(worst, max(abs(y[lo + chunk - 1 - q]) for q in range(hb)))
    return worst


def emulate_segment(info, plan, x, ca, cb):
    """Chunks [ca, cb) of the kernel's segment algorithm: forward from chunk
    ca - 1 with a zero history, stored backward passes over [ca, cb) with the
    warm-up of chunk cb (or the exact end of the vector)."""
    fwd, bwd = info["forward"], info["backward"]
    K, hb, n, LC = info["window"], plan.half_bandwidth, plan.destination_size, info["chunk"]
    chunks = (n + LC - 1) // LC
    V = x.shape[0]
    c0 = max(ca - 1, 0)
    ce = cb if cb < chunks else chunks - 1
    y = {}
    for j in range(c0 * LC, min((ce + 1) * LC, n)):
        rec = fwd[j]
        s0 = int(rec[:1].view(np.int32)[0])
        s = np.zeros(V, np.float32)
        for k in range(K):
            s = fma32(rec[4 + k], x[:, s0 + k], s)
        for q in range(hb):
            d = hb - q
            s = fma32(rec[4 + K + q], y.get(j - d, np.zeros(V, np.float32)), s)
        y[j] = s * rec[1]

    def back(lo, hi, carry):
        xs = {hi + e: carry[e] for e in range(hb)}
        for j in range(hi - 1, lo - 1, -1):
            if j >= n:
                xs[j] = np.zeros(V, np.float32)
                continue
            s = np.zeros(V, np.float32)
            for q in range(hb):
                d = q + 1 if hb == 3 else hb - q
                s = fma32(bwd[j, q], xs.get(j + d, np.zeros(V, np.float32)), s)
            xs[j] = (y[j] - s).astype(np.float32)
        return xs

    zero = [np.zeros(V, np.float32)] * hb
    res = {}
    for c in range(ca, cb):
        lo, hi = c * LC, (c + 1) * LC
        if c + 1 == chunks:
            carry = zero
        else:
            nxt = back(hi, hi + LC, zero)
            carry = [nxt[hi + e] for e in range(hb)]
        xs = back(lo, hi, carry)
        for j in range(lo, min(hi, n)):
            res[j] = xs[j]
    return res


@pytest.mark.parametrize("name,req,eligible", CASES[:6], ids=[c[0] for c in CASES[:6]])
def test_segment_admission_and_emulation(gb, name, req, eligible):
    """The forward warm-up check equals a float64 restatement, and segments
    computed as the kernels do (zero history one chunk early, stored
    backward passes over whole chunks) agree with the oracle like the
    unsegmented passes."""
    p = gb.AxisPlan(product_request(gb, req), cached=False)
    info = p.stream_info(records=True)
    want_ft = forward_transfer(p, info["chunk"])
    assert info["forward_transfer"] == pytest.approx(want_ft, rel=1e-9, abs=1e-300)
    assert bool(info["segmentable"]) == bool(info["eligible"] and info["ring_ok_transposed"]
                                             and want_ft <= 2.0 ** -26)
    chunks = (p.destination_size + info["chunk"] - 1) // info["chunk"]
    if not info["segmentable"] or chunks < 4:
        return
    o = O.Plan(oracle_request(req))
    rng = np.random.default_rng(4)
    x = rng.random((3, p.source_size), dtype=np.float32)
    want = np.stack([o.inverse_axis_f32_gpu(r) for r in x])
    scale = float(np.max(np.abs(want)))
    whole = emulate(info, o, x)
    bounds = [0, 1, chunks // 2, chunks - 1, chunks]
    for ca, cb in zip(bounds, bounds[1:]):
        seg = emulate_segment(info, o, x, ca, cb)
        for j, v in seg.items():
            assert np.max(np.abs(v - want[:, j])) <= 4e-7 * scale
            assert np.max(np.abs(v - whole[:, j])) <= 2e-7 * scale


# 4K Debicubic(1/3, 1/3) with blur 1.1: seven taps 1.5 samples apart, so the
# groups of four need the 16-sample union (the cases above take 12 or none).
GROUPED_16 = [
    ("bicubic-blur-3840-2560", (3840, 2560, 2560.0, 0.0, "bicubic", 3, 1 / 3, 1 / 3, 1.1, "symmetric", 0), True),
    ("bicubic-blur-2160-1440", (2160, 1440, 1440.0, 0.0, "bicubic", 3, 1 / 3, 1 / 3, 1.1, "symmetric", 0), True),
]


@pytest.mark.parametrize("name,req,eligible", CASES[:6] + GROUPED_16, ids=[c[0] for c in CASES[:6] + GROUPED_16])
def test_grouped_records(gb, name, req, eligible):
    """Grouped records of the 2D chunk-delayed kernels restate the
    per-destination records: each group of four destinations carries the
    first window start, its ring offset and the union's refill target, the
    four inverse diagonals, the four windows laid over the union (zeros
    elsewhere) and the four records' lower factors."""
    p = gb.AxisPlan(product_request(gb, req), cached=False)
    info = p.stream_info(records=True)
    if not (info["eligible"] and info["ring_ok_transposed"]):
        assert info["group_union"] == 0
        return
    fwd, K, hb = info["forward"], info["window"], p.half_bandwidth
    starts = fwd[:, 0].copy().view(np.int32)
    span = max(int(starts[g + 3]) + K - int(starts[g]) for g in range(0, len(starts), 4))
    want_u = 12 if span <= 12 else 16 if span <= 16 else 0
    assert info["group_union"] == want_u
    if any(name == c[0] for c in GROUPED_16):
        assert want_u == 16
    if not want_u:
        return
    U = want_u
    groups = info["groups"]
    assert groups.shape == (len(starts) // 4, 8 + 4 * U + -(-4 * hb // 4) * 4)
    assert info["group_stride"] == groups.shape[1]
    for gi, grp in enumerate(groups):
        g = 4 * gi
        hdr = grp[:4].copy().view(np.int32)
        base = int(starts[g])
        assert hdr[0] == base and hdr[1] == (base % 32) * 34 and hdr[2] == int(starts[g + 3]) + K
        for q in range(4):
            rec = fwd[g + q]
            assert grp[4 + q] == rec[1]
            dense = np.zeros(U, np.float32)
            at = int(starts[g + q]) - base
            dense[at:at + K] = rec[4:4 + K]
            assert np.array_equal(grp[8 + q * U:8 + (q + 1) * U], dense)
            assert np.array_equal(grp[8 + 4 * U + q * hb:8 + 4 * U + (q + 1) * hb], rec[4 + K:4 + K + hb])


def f64_margin_transfer(p, chunk, margin):
    """Influence left by a unit history (forward, undivided values) or carry
    (backward) after `margin` chunks from every chunk boundary, in float64,
    from the plan's Float64 LDL^T bands (band d at i: L(i + d, i))."""
    n, hb = p.destination_size, p.half_bandwidth
    bands = p.array("ldlt_bands_f64").reshape(hb + 1, n)
    chunks = (n + chunk - 1) // chunk
    span = margin * chunk
    worst = 0.0
    for k in range(1, chunks):
        a = k * chunk
        if a + span <= n:
            for e in range(hb):
                z = {a - 1 - e: 1.0}
                for i in range(a, a + span):
                    z[i] = -sum(bands[d, i - d] * z.get(i - d, 0.0) for d in range(1, min(hb, i) + 1))
                worst = max(worst, max(abs(z[a + span - 1 - q]) for q in range(hb)))
            for e in range(hb):
                x = {a + span + e: 1.0}
                for i in range(a + span - 1, a - 1, -1):
                    x[i] = -sum(bands[d, i] * x.get(i + d, 0.0) for d in range(1, min(hb, n - i - 1) + 1))
                worst = max(worst, max(abs(x[a + q]) for q in range(hb)))
    return worst


@pytest.mark.parametrize("req", [
    (600, 400, 400.0, 0.0, "bicubic", 3, 0, 0.5, 1.0, "mirror", 2),
    (500, 333, 333.0, 0.1, "spline64", 3, 0, 0.5, 1.1, "symmetric", 2),
])
def test_float64_segment_margins(gb, req):
    """The Float64 segment margin: the smallest of 2..4 chunks leaving less
    than 2^-60, its transfer equal to a float64 restatement."""
    p = gb.AxisPlan(product_request(gb, req), cached=False)
    info = p.stream_info()
    assert info["f64_eligible"]
    chunks = -(-p.destination_size // info["chunk"])
    want = 0
    for margin in (2, 3, 4):
        t = f64_margin_transfer(p, info["chunk"], margin)
        if chunks >= 2 * margin and t <= 2.0 ** -60:
            want = margin
            break
    assert info["f64_margin"] == want and bool(info["f64_segmentable"]) == (want > 0)
    assert info["f64_margin_transfer"] == pytest.approx(t, rel=1e-9, abs=1e-300)


def exact_margin_transfer(info, p, margin):
    """Influence left by a unit history (forward) or carry (backward) after
    `margin` chunks of the packed Float32 records, in float64."""
    fwd, bwd, K, hb = info["forward"], info["backward"], info["window"], p.half_bandwidth
    n, chunk = p.destination_size, info["chunk"]
    chunks = -(-n // chunk)
    span = margin * chunk
    worst = 0.0
    for k in range(1, chunks):
        a = k * chunk
        if a + span > n:
            break
        for e in range(hb):
            z = {a - 1 - e: 1.0}
            for i in range(a, a + span):
                z[i] = float(fwd[i, 1]) * sum(float(fwd[i, 4 + K + q]) * z.get(i - (hb - q), 0.0) for q in range(hb))
            worst = max(worst, max(abs(z[a + span - 1 - q]) for q in range(hb)))
            x = {a + span + e: 1.0}
            for i in range(a + span - 1, a - 1, -1):
                x[i] = -sum(float(bwd[i, q]) * x.get(i + (q + 1 if hb == 3 else hb - q), 0.0) for q in range(hb))
            worst = max(worst, max(abs(x[a + q]) for q in range(hb)))
    return worst


@pytest.mark.parametrize("req", [
    (300, 200, 200.0, 0.0, "spline64", 3, 0, 0.5, 1.1, "symmetric", 0),
    (500, 470, 470.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "mirror", 0),
])
def test_two_pass_segment_margins(gb, req):
    """The two-pass kernels' segment margin: the smallest of 1..4 chunks
    leaving less than 2^-26, its transfer equal to a float64 restatement on
    the packed records."""
    p = gb.AxisPlan(product_request(gb, req), cached=False)
    info = p.stream_info(records=True)
    assert info["exact"]
    chunks = -(-p.destination_size // info["chunk"])
    want, t = 0, None
    for margin in (1, 2, 3, 4):
        t = exact_margin_transfer(info, p, margin)
        if chunks >= 2 * margin + 1 and t <= 2.0 ** -26:
            want = margin
            break
    assert info["exact_margin"] == want
    assert info["exact_margin_transfer"] == pytest.approx(t, rel=1e-6, abs=1e-300)
