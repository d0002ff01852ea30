"""Seeded synthetic frames and candidate lists for benchmarks and tests.

Frames follow the construction of the reference's benchmark inputs: a
seeded uniform [0, 1] field at the base (descaled) size, a Gaussian blur of
sigma 1.5, a bicubic (b=0, c=0.5) upscale to the source size, and N(0, 1e-3)
noise; integer planes are then quantised at limited range.  The upscale is
the forward operator A of a descale plan (the transpose of its stored CSR),
so a frame is exactly representable at its base size up to the noise.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np

from . import AxisPlan, AxisRequest

SWEEP_KERNELS = {
    # name: (kernel, taps, b, c)
    "bicubic": ("bicubic", 3, 0.0, 0.5),
    "bilinear": ("bilinear", 3, 0.0, 0.5),
    "lanczos3": ("lanczos", 3, 0.0, 0.5),
}


def upscale_matrix(src: int, dst: int, kernel: str = "bicubic", border: str = "symmetric"):
    """Sparse A (src x dst) of the descale plan src -> dst."""
    import scipy.sparse as sp
    k, taps, b, c = SWEEP_KERNELS[kernel]
    p = AxisPlan(AxisRequest(src, dst, float(dst), 0.0, k, taps, b, c, 1.0, border, 1), cached=False)
    at = sp.csr_matrix((p.array("transpose_weights").astype(np.float64),
                        p.array("transpose_indices"), p.array("transpose_offsets")),
                       shape=(dst, src))
    return at.T.tocsr()


def gray_frame(width: int, height: int, base_width: int, base_height: int, seed: int) -> np.ndarray:
    """Float32 GRAYS frame (height x width) upscaled from a base field."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    ah = upscale_matrix(width, base_width)
    av = upscale_matrix(height, base_height)
    base = gaussian_filter(rng.random((base_height, base_width)), 1.5)
    up = av @ (ah @ base.T).T
    up = up + rng.normal(0.0, 1e-3, up.shape)
    return np.ascontiguousarray(up, dtype=np.float32)


def sweep_width(height: int, width_per_height: float = 16.0 / 9.0) -> int:
    """Candidate width for a candidate height: round(h * 16 / 9), made even."""
    w = int(round(height * width_per_height))
    return w + (w & 1)


def native_resolution_candidates(width: int, height: int, heights: Sequence[int],
                                 kernels: Sequence[str] = ("bicubic", "bilinear", "lanczos3"),
                                 border: str = "symmetric", f64_mode: int = 0
                                 ) -> List[Tuple[str, int, int, AxisRequest, AxisRequest]]:
    """(kernel, w, h, horizontal request, vertical request) per candidate,
    heights outer, kernels inner; default arguments of the plugin's filters
    (no shift, active size = destination size)."""
    out = []
    for h in heights:
        w = sweep_width(h, width / height)
        for name in kernels:
            k, taps, b, c = SWEEP_KERNELS[name]
            out.append((name, w, h,
                        AxisRequest(width, w, float(w), 0.0, k, taps, b, c, 1.0, border, f64_mode),
                        AxisRequest(height, h, float(h), 0.0, k, taps, b, c, 1.0, border, f64_mode)))
    return out
