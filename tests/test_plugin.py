"""The plugin-shaped mirror (dsmvc_gb300/plugin.py) against the reference's
plugin surface (src/vs_plugin.cpp): argument validation and its messages,
per-plane requests with the chroma placement, range detection, the no-op
return and the absence of a CPU fallback; on the GPU, every plane of GRAYS,
YUV420P16 and YUV420P8 frames through the plugin against the oracle, and
many filters requested concurrently against the same filters run one frame
at a time (the fan-out of tests/vs_gpu_concurrency.py).

Bars: Float32 output within max-abs 2e-5 and mean-abs 1e-6 of the CPU scalar
route; integer output within 1 code; concurrent results bit-identical to
sequential ones.
"""
import hashlib
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle as O
from common import F32_MAX_ABS, F32_MEAN_ABS, INT_MAX_CODES


@pytest.fixture(scope="module")
def P(gb):
    return gb.plugin


def gray(w, h, seed=1):
    from dsmvc_gb300.plugin import Frame, GRAYS
    rng = np.random.default_rng(seed)
    return Frame([(0.25 + 0.5 * rng.random((h, w), dtype=np.float32))], GRAYS)


def yuv420(w, h, bits, seed=2, props=None):
    from dsmvc_gb300.plugin import Frame, YUV420P8, YUV420P16
    fmt = YUV420P16 if bits == 16 else YUV420P8
    rng = np.random.default_rng(seed)
    top = (1 << bits) - 1
    planes = [rng.integers(top // 4, 3 * top // 4, (h >> (1 if i else 0), w >> (1 if i else 0)),
                           dtype=fmt.dtype) for i in range(3)]
    return Frame(planes, fmt, dict(props or {}))


_ARGS = ["kernel", "taps", "support", "b", "c", "blur", "src_left", "src_top", "src_width",
         "src_height", "border_handling", "padding", "force", "force_h", "force_v", "opt",
         "backend", "f64mode", "custom", "custom_kernel"]


def parsed(P, src, fixed_mode, width, height, process=True, **kw):
    """The plugin's parsed arguments (unset ones None), both axes processed."""
    a = P._parse(src, fixed_mode, width, height, **{n: kw.get(n) for n in _ARGS})
    a["process_h"] = process or width != src.width
    a["process_v"] = process or height != src.height
    return a


# ---------------------------------------------------------------- validation

@pytest.mark.parametrize("kwargs,message", [
    # src/vs_plugin.cpp:500-502
    (dict(width=64, height=6), "height must be at least 8"),
    (dict(width=200, height=40), "output dimensions must not exceed input dimensions"),
    # src/vs_plugin.cpp:376-393
    (dict(width=64, height=40, padding=4), "padding must be 0, 1, 2, or 3"),
    (dict(width=64, height=40, padding=1, border_handling=1),
     "specify either padding or border_handling, not both"),
    (dict(width=64, height=40, f64mode=3), "f64mode must be 0, 1, or 2"),
    # src/vs_plugin.cpp:458
    (dict(width=64, height=40, blur=0.0), "blur must be finite and greater than zero"),
    (dict(width=64, height=40, blur=float("inf")), "blur must be finite and greater than zero"),
    (dict(width=64, height=40, backend="vulkan"), "is not provided"),
])
def test_fixed_kernel_validation(P, kwargs, message):
    with pytest.raises(ValueError, match=message):
        P.Debicubic(gray(96, 54), **kwargs)


def test_descale_kernel_arguments(P):
    src = gray(96, 54)
    with pytest.raises(ValueError, match="kernel or custom kernel is required"):
        P.Descale(src, 64, 40)
    # src/vs_plugin.cpp:444
    with pytest.raises(ValueError, match="specify either kernel or custom kernel, not both"):
        P.Descale(src, 64, 40, kernel="bicubic", custom_kernel=lambda x: 1.0 - abs(x))
    with pytest.raises(ValueError, match="unsupported kernel"):
        P.Descale(src, 64, 40, kernel="gauss")
    with pytest.raises(ValueError, match="custom kernels require taps or support"):
        P.Descale(src, 64, 40, custom_kernel=lambda x: 1.0 - abs(x))
    # src/vs_plugin.cpp:481
    with pytest.raises(ValueError, match="taps must be greater than zero"):
        P.Descale(src, 64, 40, kernel="lanczos", taps=0)


def test_subsampled_output_sizes(P):
    # src/vs_plugin.cpp:1791-1794
    with pytest.raises(ValueError, match="output width is incompatible with subsampling"):
        P.Debicubic(yuv420(96, 54, 8), 63, 40)
    with pytest.raises(ValueError, match="output height is incompatible with subsampling"):
        P.Debicubic(yuv420(96, 54, 8), 64, 41)


def test_unchanged_geometry_returns_the_source(P):
    # Neither axis processed (src/vs_plugin.cpp:1797-1810): the clip itself.
    src = gray(96, 54)
    assert P.Debicubic(src, 96, 54) is src
    assert P.Descale(src, 96, 54, kernel="lanczos") is src


def test_no_cpu_fallback(P, gb):
    # An explicit CUDA backend never falls back (src/backend.cpp:53-58).
    if gb.cuda_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(RuntimeError, match="requires an available CUDA device"):
        P.Debicubic(gray(96, 54), 64, 40)


def test_chroma_requests_follow_the_reference_placement(P):
    # prepare_filter_requests, src/vs_plugin.cpp:656-705.
    src = yuv420(1920, 1080, 16)
    a = parsed(P, src, 3, 1440, 810, taps=3, src_left=0.5, src_top=-0.25, src_width=1439.0,
               src_height=809.5)
    (h0, h1), (v0, v1) = P._requests(a, src)
    assert (h0.source_size, h0.destination_size, h0.active_length, h0.shift) == (1920, 1440, 1439.0, 0.5)
    assert (v0.source_size, v0.destination_size, v0.active_length, v0.shift) == (1080, 810, 809.5, -0.25)
    assert (h1.source_size, h1.destination_size) == (960, 720)
    assert h1.shift == 0.25 - 0.25 * 1440.0 / 1920.0 + 0.5 * 960.0 / 1920.0
    assert h1.active_length == 1439.0 * 960.0 / 1920.0
    assert (v1.source_size, v1.destination_size) == (540, 405)
    assert v1.shift == -0.25 * 540.0 / 1080.0
    assert v1.active_length == 809.5 * 540.0 / 1080.0
    assert h0.kernel == "lanczos" and h0.taps == 3 and h0.border == 3
    # GRAY frames plan one request per axis.
    g = gray(96, 54)
    (h0, h1), (v0, v1) = P._requests(parsed(P, g, 2, 64, 40, padding=1), g)
    assert h1 is None and v1 is None and h0.border == 1


def test_range_detection(P):
    # frame_range, src/vs_plugin.cpp:750-759.
    from dsmvc_gb300.plugin import Frame, VideoFormat
    assert P._range(yuv420(96, 54, 8)) == 0
    assert P._range(yuv420(96, 54, 8, props={"_Range": 1})) == 1
    assert P._range(yuv420(96, 54, 8, props={"_ColorRange": 0})) == 0
    rgb = Frame([np.zeros((8, 8), np.uint8)] * 3, VideoFormat("RGB", "integer", 8))
    assert P._range(rgb) == 1


# ---------------------------------------------------------------- GPU parity

def _oplan(r):
    return O.Plan(O.make_request(r.source_size, r.destination_size, r.active_length, r.shift,
                                 r.kernel, r.taps, r.b, r.c, r.blur, r.border, r.f64_mode))


def _expected(P, gb, src, width, height, **kw):
    """The oracle's planes for the plugin call: the same requests, the CPU
    scalar route, the integer conversion of the plugin's route."""
    fixed = {"Debicubic": 2, "Debilinear": 1, "Delanczos": 3}[kw.pop("fn")]
    hreq, vreq = P._requests(parsed(P, src, fixed, width, height, process=False, **kw), src)
    fmt = src.format
    out = []
    for i, plane in enumerate(src.planes):
        k = 1 if i and fmt.color_family == "YUV" else 0
        h = _oplan(hreq[k]) if hreq[k] else None
        v = _oplan(vreq[k]) if vreq[k] else None
        if fmt.sample_type == "integer":
            conv = gb.integer_conversion(fmt.bits_per_sample, i > 0, False)
            if h and v:
                out.append(O.inverse_2d(h, v, plane, conv))
                continue
            x = (plane.astype(np.float32) - np.float32(conv[0])) * np.float32(conv[1])
        else:
            x = plane
        y = O.inverse_2d(h, v, x) if h and v else O.inverse_rows(h, x) if h else O.inverse_columns(v, x)
        if fmt.sample_type == "integer":
            y = np.rint(np.clip(y * np.float32(conv[2]) + np.float32(conv[3]), 0, conv[4])).astype(fmt.dtype)
        out.append(y)
    return out


FILTERS = [
    ("Debicubic", 640, 360, {}),
    ("Debicubic", 640, 360, dict(b=1 / 3, c=1 / 3)),
    ("Delanczos", 640, 360, dict(taps=3)),
    ("Debilinear", 800, 450, {}),
    ("Debicubic", 640, 540, {}),     # rows only
    ("Debicubic", 960, 360, {}),     # columns only
]


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", ["GRAYS", "YUV420P16", "YUV420P8"])
def test_plugin_planes_match_the_oracle(P, gb, executor, fmt):
    src = gray(960, 540) if fmt == "GRAYS" else yuv420(960, 540, 16 if fmt == "YUV420P16" else 8)
    filters = FILTERS + ([("Debicubic", 640, 360, dict(f64mode=2))] if fmt == "GRAYS" else [])
    for name, w, h, kw in filters:
        got = getattr(P, name)(src, w, h, executor=executor, **kw)
        want = _expected(P, gb, src, w, h, fn=name, **kw)
        assert len(got.planes) == len(want)
        for g, e in zip(got.planes, want):
            assert g.shape == e.shape and g.dtype == e.dtype, (name, w, h, kw)
            if fmt == "GRAYS":
                err = np.abs(g.astype(np.float64) - e)
                assert err.max() <= F32_MAX_ABS and err.mean() <= F32_MEAN_ABS, (name, w, h, kw)
            else:
                codes = np.abs(g.astype(np.int64) - e.astype(np.int64)).max()
                assert codes <= INT_MAX_CODES, (name, w, h, kw, codes)


def _digest(frame):
    d = hashlib.sha1()
    for p in frame.planes:
        d.update(np.ascontiguousarray(p).tobytes())
    return d.hexdigest()


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", ["GRAYS", "YUV420P16", "YUV420P8"])
def test_concurrent_requests_match_sequential(P, executor, fmt):
    frames = [gray(960, 540, seed=10 + n) if fmt == "GRAYS"
              else yuv420(960, 540, 16 if fmt == "YUV420P16" else 8, seed=10 + n) for n in range(8)]
    filters = FILTERS + ([("Debicubic", 640, 360, dict(f64mode=2))] if fmt == "GRAYS" else [])
    work = [(f, n) for f in range(len(filters)) for n in range(len(frames))]

    def run(item):
        f, n = item
        name, w, h, kw = filters[f]
        return _digest(getattr(P, name)(frames[n], w, h, executor=executor, **kw))

    sequential = [run(item) for item in work]
    with ThreadPoolExecutor(max_workers=16) as pool:
        concurrent = list(pool.map(run, work[::-1]))[::-1]
    for item, a, b in zip(work, sequential, concurrent):
        assert a == b, f"{fmt}: filter {item[0]} frame {item[1]} differs between concurrent and sequential"
