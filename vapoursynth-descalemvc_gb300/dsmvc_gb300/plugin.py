"""Python mirror of the reference's VapourSynth plugin surface for the CUDA
path: ``Descale``, ``Debilinear``, ``Debicubic``, ``Delanczos``,
``Despline16/36/64`` with the reference's argument names, defaults,
validation and per-plane routing (src/vs_plugin.cpp:362-510 arguments,
:656-705 per-plane requests, :750-782 integer ranges, :1774-1983 creation,
:1425-1758 the frame loop, :1985-2068 registration).

Frames are host planes (numpy arrays); every descale runs on the GPU through
the C ABI.  Errors carry the reference's messages, prefixed like
``vsapi->setFilterError`` ("dsmvc: ...").
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence, Union

import numpy as np

_EXECUTOR = None


@dataclass(frozen=True)
class VideoFormat:
    color_family: str = "GRAY"        # GRAY, YUV, RGB
    sample_type: str = "float"        # float, integer
    bits_per_sample: int = 32
    subsampling_w: int = 0
    subsampling_h: int = 0

    @property
    def num_planes(self) -> int:
        return 1 if self.color_family == "GRAY" else 3

    @property
    def dtype(self):
        if self.sample_type == "float":
            if self.bits_per_sample != 32:
                raise ValueError("only 32-bit float samples are supported")
            return np.dtype(np.float32)
        return np.dtype(np.uint8 if self.bits_per_sample <= 8 else np.uint16)


GRAYS = VideoFormat("GRAY", "float", 32)
YUV420P16 = VideoFormat("YUV", "integer", 16, 1, 1)
YUV420P8 = VideoFormat("YUV", "integer", 8, 1, 1)


@dataclass
class Frame:
    planes: List[np.ndarray]
    format: VideoFormat = GRAYS
    props: dict = field(default_factory=dict)

    @property
    def width(self) -> int:
        return self.planes[0].shape[1]

    @property
    def height(self) -> int:
        return self.planes[0].shape[0]


def _executor():
    global _EXECUTOR
    if _EXECUTOR is None:
        from . import Executor
        _EXECUTOR = Executor()
    return _EXECUTOR


_FIXED = {1: "bilinear", 2: "bicubic", 3: "lanczos", 4: "spline16", 5: "spline36",
          6: "spline64"}
_NAMES = {"bilinear": "Debilinear", "bicubic": "Debicubic", "lanczos": "Delanczos",
          "spline16": "Despline16", "spline36": "Despline36", "spline64": "Despline64",
          "custom": "Descale"}


def _parse(src: Frame, fixed_mode: int, width, height, kernel, taps, support, b, c, blur,
           src_left, src_top, src_width, src_height, border_handling, padding, force,
           force_h, force_v, opt, backend, f64mode, custom, custom_kernel):
    """parse_arguments, src/vs_plugin.cpp:362-510."""
    if width is None or height is None:
        raise ValueError("width and height are required")
    width, height = int(width), int(height)
    src_width = float(width) if src_width is None else float(src_width)
    src_height = float(height) if src_height is None else float(src_height)
    if padding is not None and border_handling is not None:
        raise ValueError("specify either padding or border_handling, not both")
    if padding is not None:
        if padding < 0 or padding > 3:
            raise ValueError("padding must be 0, 1, 2, or 3")
        border = int(padding)
    elif border_handling is not None:
        border = 0 if border_handling == 1 else 1 if border_handling == 2 else 4
    else:
        border = 3
    f64mode = 0 if f64mode is None else int(f64mode)
    if f64mode < 0 or f64mode > 2:
        raise ValueError("f64mode must be 0, 1, or 2")
    force = int(force or 0)
    force_h = force if force_h is None else int(force_h)
    force_v = force if force_v is None else int(force_v)
    backend = "auto" if backend is None else str(backend).lower()
    if backend not in ("auto", "cuda"):
        raise ValueError(f"backend '{backend}' is not provided by the GB300 executor")
    if fixed_mode:
        kind = _FIXED[fixed_mode]
        fn = custom_kernel or custom
        if fn is not None:
            raise ValueError("custom kernels are only accepted by Descale")
    else:
        fn = custom if custom is not None else custom_kernel
        if kernel is not None and fn is not None:
            raise ValueError("specify either kernel or custom kernel, not both")
        if kernel is None and fn is None:
            raise ValueError("kernel or custom kernel is required")
        kind = "custom" if fn is not None else str(kernel).lower()
        if kind not in _NAMES:
            raise ValueError(f"unsupported kernel: {kernel}")
    blur = 1.0 if blur is None else float(blur)
    if not (blur > 0.0) or not math.isfinite(blur):
        raise ValueError("blur must be finite and greater than zero")
    fmt = src.format
    extent = min(src.width, src.height)
    if fmt.num_planes > 1:
        extent = min(extent, src.width >> fmt.subsampling_w, src.height >> fmt.subsampling_h)
    if blur >= extent:
        raise ValueError("blur exceeds the supported source-plane extent")
    taps_v = int(taps) if taps is not None else int(support) if support is not None else 3
    if kind in ("lanczos", "custom") and taps_v < 1:
        raise ValueError("taps must be greater than zero")
    if kind == "custom" and taps is None and support is None:
        raise ValueError("custom kernels require taps or support")
    if width < 1:
        raise ValueError("width must be greater than zero")
    if height < 8:
        raise ValueError("height must be at least 8")
    if width > src.width or height > src.height:
        raise ValueError("output dimensions must not exceed input dimensions")
    if not (src_width > 0.0) or not (src_height > 0.0):
        raise ValueError("src_width and src_height must be positive")
    return dict(width=width, height=height, kind=kind, taps=taps_v, b=float(b or 0.0),
                c=0.5 if c is None else float(c), blur=blur, src_left=float(src_left or 0.0),
                src_top=float(src_top or 0.0), src_width=src_width, src_height=src_height,
                border=border, f64mode=f64mode, force_h=force_h, force_v=force_v,
                custom=fn, name=_NAMES[kind])


def _requests(a, src: Frame):
    """prepare_filter_requests, src/vs_plugin.cpp:656-705."""
    from . import AxisRequest
    fmt = src.format
    sw, sh, dw, dh = src.width, src.height, a["width"], a["height"]
    base = dict(kernel=a["kind"], taps=a["taps"], b=a["b"], c=a["c"], blur=a["blur"],
                border=a["border"], f64_mode=a["f64mode"])
    hreq = [None, None]
    vreq = [None, None]
    if a["process_h"]:
        hreq[0] = AxisRequest(sw, dw, a["src_width"], a["src_left"], **base)
        if fmt.num_planes > 1 and fmt.subsampling_w > 0:
            cs = sw >> fmt.subsampling_w
            shift = 0.25 - 0.25 * dw / sw + a["src_left"] * cs / sw
            hreq[1] = AxisRequest(cs, dw >> fmt.subsampling_w, a["src_width"] * cs / sw, shift, **base)
    if a["process_v"]:
        vreq[0] = AxisRequest(sh, dh, a["src_height"], a["src_top"], **base)
        if fmt.num_planes > 1 and fmt.subsampling_h > 0:
            cs = sh >> fmt.subsampling_h
            vreq[1] = AxisRequest(cs, dh >> fmt.subsampling_h, a["src_height"] * cs / sh,
                                  a["src_top"] * cs / sh, **base)
    return hreq, vreq


def _range(frame: Frame) -> int:
    """frame_range, src/vs_plugin.cpp:750-759."""
    for key in ("_Range", "_ColorRange"):
        if key in frame.props:
            return 1 if frame.props[key] == 1 else 0
    return 1 if frame.format.color_family == "RGB" else 0


def _descale(fixed_mode: int, src: Union[Frame, Sequence[Frame]], width=None, height=None,
             kernel=None, taps=None, b=None, c=None, blur=None, src_left=None, src_top=None,
             src_width=None, src_height=None, border_handling=None, force=None, force_h=None,
             force_v=None, opt=None, backend=None, padding=None, f64mode=None, custom=None,
             support=None, custom_kernel=None, executor=None):
    if isinstance(src, (list, tuple)):
        return [_descale(fixed_mode, f, width, height, kernel, taps, b, c, blur, src_left,
                         src_top, src_width, src_height, border_handling, force, force_h,
                         force_v, opt, backend, padding, f64mode, custom, support,
                         custom_kernel, executor) for f in src]
    from . import AxisPlan, integer_conversion
    a = _parse(src, fixed_mode, width, height, kernel, taps, support, b, c, blur, src_left,
               src_top, src_width, src_height, border_handling, padding, force, force_h,
               force_v, opt, backend, f64mode, custom, custom_kernel)
    fmt = src.format
    if a["width"] % (1 << fmt.subsampling_w):
        raise ValueError("output width is incompatible with subsampling")
    if a["height"] % (1 << fmt.subsampling_h):
        raise ValueError("output height is incompatible with subsampling")
    # src/vs_plugin.cpp:1797-1810
    a["process_h"] = (a["width"] != src.width or a["src_left"] != 0.0
                      or a["src_width"] != float(a["width"]) or a["force_h"] != 0)
    a["process_v"] = (a["height"] != src.height or a["src_top"] != 0.0
                      or a["src_height"] != float(a["height"]) or a["force_v"] != 0)
    if not a["process_h"] and not a["process_v"]:
        return src
    integer = fmt.sample_type == "integer"
    if integer and not (8 <= fmt.bits_per_sample <= 16):
        raise ValueError("only 8-16 bit integer clips are supported")
    fused = integer and a["process_h"] and a["process_v"]
    from . import cuda_available
    if executor is None and not cuda_available():
        # An explicit CUDA backend never falls back (src/backend.cpp:53-58).
        raise RuntimeError("backend 'cuda' requires an available CUDA device")
    hreq, vreq = _requests(a, src)
    fn = a["custom"]
    cached = fn is None
    hplans = [AxisPlan(r, fn, cached) if r else None for r in hreq]
    vplans = [AxisPlan(r, fn, cached) if r else None for r in vreq]
    ex = executor or _executor()
    for p in hplans + vplans:
        if p is not None:
            ex.prepare(p)
    rng = _range(src)
    out_planes = []
    try:
        for plane_index, plane in enumerate(src.planes):
            hi = 1 if plane_index and fmt.subsampling_w > 0 else 0
            vi = 1 if plane_index and fmt.subsampling_h > 0 else 0
            chroma = fmt.color_family == "YUV" and plane_index != 0
            if integer:
                conv = integer_conversion(fmt.bits_per_sample, chroma, rng == 1)
            if fused:
                out_planes.append(ex.inverse_2d(hplans[hi], vplans[vi], plane, conv))
                continue
            x = plane
            if integer:
                # The reference converts through resize.Point to float and back
                # (src/vs_plugin.cpp:570-626); the normalisation used here is
                # the same integer range mapping as the fused route.
                x = ((plane.astype(np.float32) - np.float32(conv[0])) * np.float32(conv[1]))
            if a["process_h"] and a["process_v"]:
                y = ex.inverse_2d(hplans[hi], vplans[vi], x)
            elif a["process_h"]:
                y = ex.inverse_rows(hplans[hi], x)
            else:
                y = ex.inverse_columns(vplans[vi], x)
            if integer:
                s = np.clip(y * np.float32(conv[2]) + np.float32(conv[3]), 0, conv[4])
                y = np.rint(s).astype(fmt.dtype)
            out_planes.append(y)
    except (ValueError, RuntimeError, OverflowError, MemoryError) as e:
        raise type(e)(f"dsmvc: frame processing failed: {e}") from e
    return Frame(out_planes, fmt, dict(src.props))


def Descale(src, width=None, height=None, kernel=None, taps=None, b=None, c=None, blur=None,
            src_left=None, src_top=None, src_width=None, src_height=None,
            border_handling=None, force=None, force_h=None, force_v=None, opt=None,
            custom=None, support=None, custom_kernel: Optional[Callable[[float], float]] = None,
            backend=None, padding=None, f64mode=None, executor=None):
    return _descale(0, src, width, height, kernel, taps, b, c, blur, src_left, src_top,
                    src_width, src_height, border_handling, force, force_h, force_v, opt,
                    backend, padding, f64mode, custom, support, custom_kernel, executor)


def _fixed(mode):
    def fn(src, width=None, height=None, *, b=None, c=None, taps=None, blur=None,
           src_left=None, src_top=None, src_width=None, src_height=None,
           border_handling=None, force=None, force_h=None, force_v=None, opt=None,
           backend=None, padding=None, f64mode=None, executor=None):
        return _descale(mode, src, width, height, None, taps, b, c, blur, src_left, src_top,
                        src_width, src_height, border_handling, force, force_h, force_v, opt,
                        backend, padding, f64mode, None, None, None, executor)
    fn.__name__ = _NAMES[_FIXED[mode]]
    return fn


Debilinear = _fixed(1)
Debicubic = _fixed(2)
Delanczos = _fixed(3)
Despline16 = _fixed(4)
Despline36 = _fixed(5)
Despline64 = _fixed(6)
