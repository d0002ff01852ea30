"""Python binding of the GB300 descale executor's C ABI (include/dsmvc_gb300.h).

The shared library ``libdsmvc_gb300.so`` (built in-tree by ``build.py``)
holds the host planner and the CUDA executor; this module only marshals
arguments.  There is no CPU fallback: executor calls raise when the library
or a CUDA device is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from dataclasses import dataclass
from typing import Callable, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdsmvc_gb300.so")

KERNELS = {"bilinear": 0, "bicubic": 1, "lanczos": 2, "spline16": 3,
           "spline36": 4, "spline64": 5, "custom": 6}
BORDERS = {"zero": 0, "repeat": 1, "reflect101": 2, "symmetric": 3, "mirror": 4}
SAMPLES = {np.dtype(np.float32): 0, np.dtype(np.uint8): 1, np.dtype(np.uint16): 2}

OK, INVALID_ARGUMENT, RUNTIME_ERROR, LENGTH_ERROR, CUDA_ERROR, OUT_OF_MEMORY, UNAVAILABLE = range(7)


class DescaleError(RuntimeError):
    """Error raised by the executor; ``code`` is the C status."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


_EXC = {INVALID_ARGUMENT: ValueError, LENGTH_ERROR: OverflowError,
        OUT_OF_MEMORY: MemoryError}


class AxisRequestC(C.Structure):
    _fields_ = [("source_size", C.c_int32), ("destination_size", C.c_int32),
                ("active_length", C.c_double), ("shift", C.c_double),
                ("kernel", C.c_int32), ("taps", C.c_int32), ("b", C.c_double),
                ("c", C.c_double), ("blur", C.c_double), ("border", C.c_int32),
                ("f64_mode", C.c_int32)]


class ConversionC(C.Structure):
    _fields_ = [("input_offset", C.c_float), ("input_scale", C.c_float),
                ("output_scale", C.c_float), ("output_offset", C.c_float),
                ("output_maximum", C.c_uint32)]


class PlanArraysC(C.Structure):
    """dsmvc_gb_plan_arrays: a plan built elsewhere, by pointers and counts."""
    _fields_ = [("source_size", C.c_int32), ("destination_size", C.c_int32),
                ("support", C.c_int32), ("half_bandwidth", C.c_int32),
                ("active_length", C.c_double), ("shift", C.c_double),
                ("normal_rcond", C.c_double), ("normal_inf_norm", C.c_double)] + [
        (f, t) for name in ("transpose_offsets", "transpose_indices", "transpose_weights", "lower_ld",
                            "upper_l", "inverse_diagonal", "transpose_weights_f64", "normal_bands_f64",
                            "ldlt_bands_f64", "inverse_diagonal_f64")
        for f, t in ((name, C.c_void_p), (name + "_count", C.c_uint64))]


class PlanInfoC(C.Structure):
    _fields_ = [("source_size", C.c_int32), ("destination_size", C.c_int32),
                ("support", C.c_int32), ("half_bandwidth", C.c_int32),
                ("requires_float64", C.c_int32), ("max_row_entries", C.c_int32),
                ("active_length", C.c_double), ("shift", C.c_double),
                ("normal_rcond", C.c_double), ("normal_inf_norm", C.c_double),
                ("nonzeros", C.c_uint64), ("storage_bytes", C.c_uint64)]


class PlannerStatsC(C.Structure):
    _fields_ = [("plan_hits", C.c_uint64), ("plan_builds", C.c_uint64),
                ("plan_entries", C.c_uint64), ("plan_resident_bytes", C.c_uint64)]


class ExecutorStatsC(C.Structure):
    _fields_ = [("launches", C.c_uint64), ("plane_tasks", C.c_uint64),
                ("plan_uploads", C.c_uint64), ("device_plan_bytes", C.c_uint64),
                ("workspace_bytes", C.c_uint64), ("plan_cache_hits", C.c_uint64),
                ("plan_cache_misses", C.c_uint64), ("plan_cache_evictions", C.c_uint64),
                ("plan_cache_bytes", C.c_uint64), ("compile_reuses", C.c_uint64)]


class PlaneTaskC(C.Structure):
    _fields_ = [("horizontal", C.c_void_p), ("vertical", C.c_void_p),
                ("input", C.c_void_p), ("input_stride", C.c_int64),
                ("output", C.c_void_p), ("output_stride", C.c_int64),
                ("sample", C.c_int32), ("vectors", C.c_int32),
                ("conversion", ConversionC)]


class StreamInfoC(C.Structure):
    _fields_ = [("eligible", C.c_int32), ("window", C.c_int32),
                ("forward_stride", C.c_int32), ("backward_stride", C.c_int32),
                ("ring_ok_u16", C.c_int32), ("ring_ok_u8", C.c_int32),
                ("chunk", C.c_int32), ("ring", C.c_int32),
                ("backward_transfer", C.c_double), ("reason", C.c_char * 96),
                ("ring_ok_transposed", C.c_int32), ("exact", C.c_int32),
                ("segmentable", C.c_int32), ("forward_transfer", C.c_double),
                ("group_union", C.c_int32), ("group_stride", C.c_int32),
                ("f64_eligible", C.c_int32), ("f64_segmentable", C.c_int32),
                ("f64_margin", C.c_int32), ("f64_margin_transfer", C.c_double),
                ("exact_margin", C.c_int32), ("exact_margin_transfer", C.c_double)]


class SweepOptionsC(C.Structure):
    _fields_ = [("memory_budget", C.c_int64), ("autotune", C.c_int32), ("graph", C.c_int32),
                ("fused_scoring", C.c_int32), ("reserved", C.c_int32)]


class SweepInfoC(C.Structure):
    _fields_ = [("candidates", C.c_int32), ("waves", C.c_int32), ("device_bytes", C.c_int64),
                ("kernel_launches", C.c_int64), ("tune_milliseconds", C.c_double),
                ("segment_rows", C.c_int32), ("tuned_groups", C.c_int32),
                ("vectors_per_warp", C.c_int32), ("fused_candidates", C.c_int32)]


class ServerOptionsC(C.Structure):
    _fields_ = [("memory_budget", C.c_int64), ("streams", C.c_int32), ("max_batch", C.c_int32)]


class HostPlaneC(C.Structure):
    _fields_ = [("horizontal", C.c_void_p), ("vertical", C.c_void_p),
                ("input", C.c_void_p), ("input_stride", C.c_int64),
                ("output", C.c_void_p), ("output_stride", C.c_int64),
                ("sample", C.c_int32), ("conversion", ConversionC)]


class ServerStatsC(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("batches", C.c_uint64), ("latency_p50_ms", C.c_double),
                ("latency_p99_ms", C.c_double), ("latency_mean_ms", C.c_double),
                ("latency_max_ms", C.c_double), ("peak_device_bytes", C.c_int64),
                ("source_pixels", C.c_uint64), ("mean_batch_requests", C.c_double)]


class KernelTimeC(C.Structure):
    _fields_ = [("name", C.c_char * 64), ("launches", C.c_uint64),
                ("milliseconds", C.c_double), ("bytes", C.c_uint64)]


CUSTOM_FN = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)

# Every symbol the header declares, with its ctypes signature.
SIGNATURES = {
    "dsmvc_gb_last_error": ([], C.c_char_p),
    "dsmvc_gb_abi_version": ([], C.c_int),
    "dsmvc_gb_cuda_available": ([], C.c_int),
    "dsmvc_gb_plan_build": ([C.POINTER(AxisRequestC), CUSTOM_FN, C.c_void_p,
                             C.POINTER(C.c_void_p)], C.c_int),
    "dsmvc_gb_plan_get_or_build": ([C.POINTER(AxisRequestC), CUSTOM_FN, C.c_void_p,
                                    C.POINTER(C.c_void_p)], C.c_int),
    "dsmvc_gb_plan_release": ([C.c_void_p], None),
    "dsmvc_gb_plan_get_info": ([C.c_void_p, C.POINTER(PlanInfoC)], C.c_int),
    "dsmvc_gb_plan_get_array": ([C.c_void_p, C.c_int32, C.POINTER(C.c_void_p),
                                 C.POINTER(C.c_uint64)], C.c_int),
    "dsmvc_gb_plan_hashes": ([C.c_void_p, C.POINTER(AxisRequestC), C.POINTER(C.c_uint64),
                              C.POINTER(C.c_uint64)], C.c_int),
    "dsmvc_gb_plan_stream_info": ([C.c_void_p, C.POINTER(StreamInfoC), C.c_void_p, C.c_uint64,
                                   C.c_void_p, C.c_uint64], C.c_int),
    "dsmvc_gb_plan_stream_groups": ([C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)], C.c_int),
    "dsmvc_gb_planner_cache_stats": ([C.POINTER(PlannerStatsC)], C.c_int),
    "dsmvc_gb_clear_planner_caches": ([], None),
    "dsmvc_gb_executor_create": ([C.c_int32, C.POINTER(C.c_void_p)], C.c_int),
    "dsmvc_gb_executor_destroy": ([C.c_void_p], None),
    "dsmvc_gb_prepare": ([C.c_void_p, C.c_void_p], C.c_int),
    "dsmvc_gb_prepare_many": ([C.c_void_p, C.POINTER(C.c_void_p), C.c_int32], C.c_int),
    "dsmvc_gb_seal": ([C.c_void_p], C.c_int),
    "dsmvc_gb_executor_get_stats": ([C.c_void_p, C.POINTER(ExecutorStatsC)], C.c_int),
    "dsmvc_gb_inverse_rows": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                               C.c_int64, C.c_int32], C.c_int),
    "dsmvc_gb_inverse_columns": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                  C.c_void_p, C.c_int64, C.c_int32], C.c_int),
    "dsmvc_gb_inverse_2d": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                             C.c_void_p, C.c_int64], C.c_int),
    "dsmvc_gb_inverse_2d_u8": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                C.c_void_p, C.c_int64, C.POINTER(ConversionC)], C.c_int),
    "dsmvc_gb_inverse_2d_u16": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                 C.c_void_p, C.c_int64, C.POINTER(ConversionC)], C.c_int),
    "dsmvc_gb_inverse_2d_planes": ([C.c_void_p, C.POINTER(HostPlaneC), C.c_int32], C.c_int),
    "dsmvc_gb_run_batch": ([C.c_void_p, C.POINTER(PlaneTaskC), C.c_int32, C.c_void_p,
                            C.c_int32], C.c_int),
    "dsmvc_gb_stream_check": ([C.c_void_p, C.c_void_p], C.c_int),
    "dsmvc_gb_stream_release": ([C.c_void_p, C.c_void_p], C.c_int),
    "dsmvc_gb_batch_create": ([C.c_void_p, C.POINTER(PlaneTaskC), C.c_int32,
                               C.POINTER(C.c_void_p)], C.c_int),
    "dsmvc_gb_batch_launch": ([C.c_void_p, C.c_void_p], C.c_int),
    "dsmvc_gb_batch_check": ([C.c_void_p, C.c_void_p], C.c_int),
    "dsmvc_gb_batch_create_parts": ([C.c_void_p, C.POINTER(PlaneTaskC), C.c_int32, C.c_int32,
                                     C.POINTER(C.c_void_p)], C.c_int),
    "dsmvc_gb_batch_parts": ([C.c_void_p, C.POINTER(C.c_int32)], C.c_int),
    "dsmvc_gb_batch_info": ([C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                             C.POINTER(C.c_int64)], C.c_int),
    "dsmvc_gb_batch_destroy": ([C.c_void_p], None),
    "dsmvc_gb_inverse_2d_noalloc": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int64,
                                     C.c_void_p, C.c_int64, C.POINTER(ConversionC), C.c_void_p],
                                    C.c_int),
    "dsmvc_gb_plan_import": ([C.POINTER(PlanArraysC), C.POINTER(C.c_void_p)], C.c_int),
    "dsmvc_gb_plan_build_many_device": ([C.POINTER(AxisRequestC), C.c_int32, C.c_int32, C.c_int32,
                                         C.POINTER(C.c_void_p)], C.c_int),
    "dsmvc_gb_plan_build_many": ([C.POINTER(AxisRequestC), C.c_int32, C.c_int32,
                                  C.POINTER(C.c_void_p)], C.c_int),
    "dsmvc_gb_sweep_create": ([C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int32,
                               C.c_void_p, C.c_int64, C.POINTER(SweepOptionsC),
                               C.POINTER(C.c_void_p)], C.c_int),
    "dsmvc_gb_sweep_run": ([C.c_void_p, C.c_void_p], C.c_int),
    "dsmvc_gb_sweep_run_plain": ([C.c_void_p, C.c_void_p], C.c_int),
    "dsmvc_gb_sweep_scores": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "dsmvc_gb_sweep_get_info": ([C.c_void_p, C.POINTER(SweepInfoC)], C.c_int),
    "dsmvc_gb_sweep_profile": ([C.c_void_p, C.c_void_p, C.POINTER(C.c_double)], C.c_int),
    "dsmvc_gb_sweep_destroy": ([C.c_void_p], None),
    "dsmvc_gb_server_create": ([C.c_void_p, C.POINTER(ServerOptionsC), C.POINTER(C.c_void_p)],
                               C.c_int),
    "dsmvc_gb_server_submit": ([C.c_void_p, C.POINTER(HostPlaneC), C.c_int32,
                               C.POINTER(C.c_uint64)], C.c_int),
    "dsmvc_gb_server_wait": ([C.c_void_p, C.c_uint64], C.c_int),
    "dsmvc_gb_server_poll": ([C.c_void_p, C.c_uint64, C.POINTER(C.c_int32)], C.c_int),
    "dsmvc_gb_server_get_stats": ([C.c_void_p, C.POINTER(ServerStatsC)], C.c_int),
    "dsmvc_gb_server_reset_stats": ([C.c_void_p], C.c_int),
    "dsmvc_gb_server_destroy": ([C.c_void_p], None),
    "dsmvc_gb_measure_fp64_peak": ([C.c_int32, C.POINTER(C.c_double)], C.c_int),
    "dsmvc_gb_host_blocks_set_limit": ([C.c_void_p, C.c_int64], C.c_int),
    "dsmvc_gb_host_blocks_note_use": ([C.c_void_p, C.c_void_p, C.c_int64], C.c_int),
    "dsmvc_gb_host_blocks_covered": ([C.c_void_p, C.c_int64, C.POINTER(C.c_int32)], C.c_int),
    "dsmvc_gb_host_blocks_release": ([C.c_void_p, C.c_int64], C.c_int),
    "dsmvc_gb_host_blocks_drop_owner": ([C.c_void_p], C.c_int),
    "dsmvc_gb_host_blocks_get_stats": ([C.c_void_p], C.c_int),
    "dsmvc_gb_host_blocks_test_registrar": ([C.c_int32], C.c_int),
    "dsmvc_gb_host_register": ([C.c_void_p, C.c_int64, C.POINTER(C.c_int32)], C.c_int),
    "dsmvc_gb_host_unregister": ([C.c_void_p], C.c_int),
    "dsmvc_gb_profile": ([C.c_void_p, C.c_int32], C.c_int),
    "dsmvc_gb_profile_read": ([C.c_void_p, C.POINTER(KernelTimeC), C.c_int32,
                               C.POINTER(C.c_int32)], C.c_int),
}

_lib = None


def build(force: bool = False) -> str:
    """Compile the library in-tree (see ../build.py)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "_dsmvc_gb300_build", os.path.join(os.path.dirname(HERE), "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def lib():
    """Load libdsmvc_gb300.so; raises when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run build.py (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _check(code: int) -> None:
    if code != OK:
        msg = lib().dsmvc_gb_last_error().decode(errors="replace")
        cls = _EXC.get(code)
        if cls is not None:
            raise cls(msg)
        raise DescaleError(code, msg)


def cuda_available() -> bool:
    return bool(lib().dsmvc_gb_cuda_available())


@dataclass(frozen=True)
class AxisRequest:
    """AxisRequest (include/dsmvc/engine.hpp:68-76)."""
    source_size: int
    destination_size: int
    active_length: float
    shift: float = 0.0
    kernel: str = "bicubic"
    taps: int = 3
    b: float = 0.0
    c: float = 0.5
    blur: float = 1.0
    border: str = "symmetric"
    f64_mode: int = 0

    def to_c(self) -> AxisRequestC:
        return AxisRequestC(int(self.source_size), int(self.destination_size),
                            float(self.active_length), float(self.shift),
                            KERNELS[self.kernel] if isinstance(self.kernel, str) else int(self.kernel),
                            int(self.taps), float(self.b), float(self.c), float(self.blur),
                            BORDERS[self.border] if isinstance(self.border, str) else int(self.border),
                            int(self.f64_mode))


class AxisPlan:
    """A host plan handle (shared, immutable)."""

    _ARRAYS = [("transpose_offsets", np.uint32), ("transpose_indices", np.int32),
               ("transpose_weights", np.float32), ("lower_ld", np.float32),
               ("upper_l", np.float32), ("inverse_diagonal", np.float32),
               ("transpose_weights_f64", np.float64), ("normal_bands_f64", np.float64),
               ("ldlt_bands_f64", np.float64), ("inverse_diagonal_f64", np.float64)]

    def __init__(self, request: AxisRequest, custom: Optional[Callable[[float], float]] = None,
                 cached: bool = True, _handle=None):
        self.request = request
        self._req_c = request.to_c()
        self._custom = CUSTOM_FN(lambda x, _u: float(custom(x))) if custom else CUSTOM_FN()
        h = C.c_void_p()
        if _handle is not None:
            h = C.c_void_p(_handle)
        else:
            fn = lib().dsmvc_gb_plan_get_or_build if cached else lib().dsmvc_gb_plan_build
            _check(fn(C.byref(self._req_c), self._custom, None, C.byref(h)))
        self._h = h
        info = PlanInfoC()
        _check(lib().dsmvc_gb_plan_get_info(h, C.byref(info)))
        for name, _ in info._fields_:
            setattr(self, name, getattr(info, name))
        self.requires_float64 = bool(info.requires_float64)

    @property
    def handle(self):
        return self._h

    def array(self, name: str) -> np.ndarray:
        for i, (n, dt) in enumerate(self._ARRAYS):
            if n == name:
                ptr, count = C.c_void_p(), C.c_uint64()
                _check(lib().dsmvc_gb_plan_get_array(self._h, i, C.byref(ptr), C.byref(count)))
                if count.value == 0:
                    return np.zeros(0, dt)
                nbytes = count.value * np.dtype(dt).itemsize
                return np.frombuffer((C.c_char * nbytes).from_address(ptr.value), dt).copy()
        raise KeyError(name)

    def stream_info(self, records: bool = False) -> dict:
        """Streaming-kernel eligibility and (optionally) packed records."""
        info = StreamInfoC()
        _check(lib().dsmvc_gb_plan_stream_info(self._h, C.byref(info), None, 0, None, 0))
        out = {k: getattr(info, k) for k, _ in info._fields_}
        out["reason"] = info.reason.decode()
        if records and (info.eligible or info.exact):
            # Records cover whole chunks: zero records past the last destination.
            n = -(-self.destination_size // info.chunk) * info.chunk
            fwd = np.zeros(n * info.forward_stride, np.float32)
            bwd = np.zeros(n * info.backward_stride, np.float32)
            _check(lib().dsmvc_gb_plan_stream_info(self._h, C.byref(info), fwd.ctypes.data, fwd.size,
                                                   bwd.ctypes.data, bwd.size))
            out["forward"] = fwd.reshape(n, info.forward_stride)
            out["backward"] = bwd.reshape(n, info.backward_stride)
            if info.group_union:
                count = C.c_uint64()
                _check(lib().dsmvc_gb_plan_stream_groups(self._h, None, 0, C.byref(count)))
                groups = np.zeros(count.value, np.float32)
                _check(lib().dsmvc_gb_plan_stream_groups(self._h, groups.ctypes.data, groups.size, C.byref(count)))
                out["groups"] = groups.reshape(-1, info.group_stride)
        return out

    def hashes(self):
        f, c = C.c_uint64(), C.c_uint64()
        _check(lib().dsmvc_gb_plan_hashes(self._h, C.byref(self._req_c), C.byref(f), C.byref(c)))
        return "%016x" % f.value, "%016x" % c.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.dsmvc_gb_plan_release(h)
            self._h = None


def import_plan(source) -> AxisPlan:
    """A plan built elsewhere (any object with the reference AxisPlan's
    scalars and arrays as attributes, e.g. the reference engine's own plan)
    imported through dsmvc_gb_plan_import: copied and validated.  An
    imported plan carries no request: the returned plan's `request` holds
    only its sizes and shift (kernel "custom")."""
    keep = []
    a = PlanArraysC()
    for name in ("source_size", "destination_size", "support", "half_bandwidth"):
        setattr(a, name, int(getattr(source, name)))
    for name in ("active_length", "shift", "normal_rcond", "normal_inf_norm"):
        setattr(a, name, float(getattr(source, name, 0.0)))
    for name, dt in AxisPlan._ARRAYS:
        arr = np.ascontiguousarray(getattr(source, name, np.zeros(0, dt)), dt)
        keep.append(arr)
        setattr(a, name, arr.ctypes.data if arr.size else None)
        setattr(a, name + "_count", int(arr.size))
    h = C.c_void_p()
    _check(lib().dsmvc_gb_plan_import(C.byref(a), C.byref(h)))
    req = AxisRequest(a.source_size, a.destination_size, a.active_length, a.shift, "custom")
    return AxisPlan(req, _handle=h.value)


class HostBlockStatsC(C.Structure):
    _fields_ = [(name, C.c_uint64) for name in ("registrations", "failures", "cap_refusals", "hits", "misses",
                                                 "released", "registered_bytes", "peak_bytes")]


class host_blocks:
    """dsmvc_gb_host_blocks_*: host blocks (a frame pool's allocations)
    page-locked on their second transfer within a per-owner byte limit, so
    that plane copies from and to them run as DMA.  Owners are integers
    (opaque tokens); blocks are (address, size) pairs."""

    @staticmethod
    def set_limit(owner: int, nbytes: int) -> None:
        _check(lib().dsmvc_gb_host_blocks_set_limit(C.c_void_p(owner), int(nbytes)))

    @staticmethod
    def note_use(owner: int, base: int, size: int) -> None:
        _check(lib().dsmvc_gb_host_blocks_note_use(C.c_void_p(owner), C.c_void_p(base), int(size)))

    @staticmethod
    def note_array(owner: int, array: np.ndarray) -> None:
        """note_use of the memory a numpy array spans."""
        host_blocks.note_use(owner, array.ctypes.data, array.nbytes)

    @staticmethod
    def covered(pointer: int, nbytes: int) -> bool:
        out = C.c_int32()
        _check(lib().dsmvc_gb_host_blocks_covered(C.c_void_p(pointer), int(nbytes), C.byref(out)))
        return bool(out.value)

    @staticmethod
    def release(base: int, size: int) -> None:
        _check(lib().dsmvc_gb_host_blocks_release(C.c_void_p(base), int(size)))

    @staticmethod
    def drop_owner(owner: int) -> None:
        _check(lib().dsmvc_gb_host_blocks_drop_owner(C.c_void_p(owner)))

    @staticmethod
    def stats() -> dict:
        out = HostBlockStatsC()
        _check(lib().dsmvc_gb_host_blocks_get_stats(C.byref(out)))
        return {k: getattr(out, k) for k, _ in out._fields_}

    @staticmethod
    def test_registrar(mode: int) -> None:
        """0: CUDA; fakes for tests: 1 registers, 2 finds blocks registered
        elsewhere, 3 fails (each switch releases every block first)."""
        _check(lib().dsmvc_gb_host_blocks_test_registrar(int(mode)))

    @staticmethod
    def register(base: int, size: int) -> int:
        """Page-locks one block outside the registry (dsmvc_gb_host_register):
        0 page-locked here, 1 already page-locked elsewhere, -1 failed."""
        out = C.c_int32()
        _check(lib().dsmvc_gb_host_register(C.c_void_p(base), int(size), C.byref(out)))
        return out.value

    @staticmethod
    def unregister(base: int) -> None:
        _check(lib().dsmvc_gb_host_unregister(C.c_void_p(base)))


def measure_fp64_peak(device: int = 0) -> float:
    """Measured FP64 TFLOP/s of the device (dsmvc_gb_measure_fp64_peak)."""
    t = C.c_double()
    _check(lib().dsmvc_gb_measure_fp64_peak(int(device), C.byref(t)))
    return t.value


def build_plans(requests: Sequence[AxisRequest], threads: int = 0, device: Optional[int] = None) -> list:
    """Uncached plans: dsmvc_gb_plan_build_many on `threads` host threads
    (0 = all hardware threads), or with `device` (a CUDA device index, -1 =
    the current one) dsmvc_gb_plan_build_many_device: the normal band, LDL^T,
    condition estimate and Float32 arrays of every plan on that GPU, bit
    for bit the same plans."""
    reqs = (AxisRequestC * len(requests))(*[r.to_c() for r in requests])
    out = (C.c_void_p * len(requests))()
    if device is None:
        _check(lib().dsmvc_gb_plan_build_many(reqs, len(requests), int(threads), out))
    else:
        _check(lib().dsmvc_gb_plan_build_many_device(reqs, len(requests), int(device), int(threads), out))
    return [AxisPlan(r, _handle=out[i]) for i, r in enumerate(requests)]


def planner_cache_stats() -> dict:
    s = PlannerStatsC()
    _check(lib().dsmvc_gb_planner_cache_stats(C.byref(s)))
    return {k: getattr(s, k) for k, _ in s._fields_}


def clear_planner_caches() -> None:
    lib().dsmvc_gb_clear_planner_caches()


def _conv(conversion) -> ConversionC:
    if conversion is None:
        return ConversionC(0.0, 1.0, 1.0, 0.0, 255)
    if isinstance(conversion, ConversionC):
        return conversion
    return ConversionC(*[float(x) for x in conversion[:4]], int(conversion[4]))


@dataclass
class PlaneTask:
    """One device plane of a batch (pointers are device addresses)."""
    horizontal: Optional[AxisPlan]
    vertical: Optional[AxisPlan]
    input: int
    input_stride: int
    output: int
    output_stride: int
    sample: int = 0
    vectors: int = 0
    conversion: object = None


class Executor:
    """CudaExecutor equivalent (src/cuda/cuda_executor.hpp:11-110)."""

    def __init__(self, device: int = -1):
        h = C.c_void_p()
        _check(lib().dsmvc_gb_executor_create(int(device), C.byref(h)))
        self._h = h
        self._keep = []
        # Batches, sweeps and request loops built on this executor: closed
        # before it, whoever still holds them.
        self._dependents = weakref.WeakSet()

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value and _lib is not None:
            for d in list(getattr(self, "_dependents", ())):
                d.close()
            _lib.dsmvc_gb_executor_destroy(self._h)
            self._h = None

    __del__ = close

    def prepare(self, plan: AxisPlan) -> None:
        _check(lib().dsmvc_gb_prepare(self._h, plan.handle))
        self._keep.append(plan)

    def prepare_many(self, plans: Sequence[AxisPlan]) -> None:
        """dsmvc_gb_prepare_many: many plans packed on host threads and
        uploaded in one allocation."""
        arr = (C.c_void_p * len(plans))(*[p.handle.value for p in plans])
        _check(lib().dsmvc_gb_prepare_many(self._h, arr, len(plans)))
        self._keep.extend(plans)

    def seal(self) -> None:
        _check(lib().dsmvc_gb_seal(self._h))

    def stats(self) -> dict:
        s = ExecutorStatsC()
        _check(lib().dsmvc_gb_executor_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    # -- synchronous host calls --------------------------------------------
    def inverse_rows(self, plan: AxisPlan, x: np.ndarray, out: Optional[np.ndarray] = None):
        x = np.asarray(x, np.float32)
        if out is None:
            out = np.empty((x.shape[0], plan.destination_size), np.float32)
        _check(lib().dsmvc_gb_inverse_rows(self._h, plan.handle, x.ctypes.data,
                                           x.strides[0] // 4, out.ctypes.data,
                                           out.strides[0] // 4, x.shape[0]))
        return out

    def inverse_columns(self, plan: AxisPlan, x: np.ndarray, out: Optional[np.ndarray] = None):
        x = np.asarray(x, np.float32)
        if out is None:
            out = np.empty((plan.destination_size, x.shape[1]), np.float32)
        _check(lib().dsmvc_gb_inverse_columns(self._h, plan.handle, x.ctypes.data,
                                              x.strides[0] // 4, out.ctypes.data,
                                              out.strides[0] // 4, x.shape[1]))
        return out

    def inverse_2d(self, h: AxisPlan, v: AxisPlan, x: np.ndarray, conversion=None,
                   out: Optional[np.ndarray] = None):
        """inverse_2d / inverse_2d_u8 / inverse_2d_u16 on a host plane; row
        strides come from the arrays (padding is never touched)."""
        assert x.strides[1] == x.itemsize, "rows must be contiguous"
        if out is None:
            out = np.empty((v.destination_size, h.destination_size), x.dtype)
        es = x.itemsize
        if x.dtype == np.float32:
            _check(lib().dsmvc_gb_inverse_2d(self._h, h.handle, v.handle, x.ctypes.data,
                                             x.strides[0] // es, out.ctypes.data,
                                             out.strides[0] // es))
        elif x.dtype in (np.uint8, np.uint16):
            fn = lib().dsmvc_gb_inverse_2d_u8 if x.dtype == np.uint8 else lib().dsmvc_gb_inverse_2d_u16
            conv = _conv(conversion)
            _check(fn(self._h, h.handle, v.handle, x.ctypes.data, x.strides[0] // es,
                      out.ctypes.data, out.strides[0] // es, C.byref(conv)))
        else:
            raise ValueError(f"unsupported sample type {x.dtype}")
        return out

    def inverse_2d_planes(self, planes: Sequence[tuple]) -> None:
        """dsmvc_gb_inverse_2d_planes: [(h, v, input, output[, conversion])]
        with 2D numpy arrays (rows contiguous, same dtype in and out); the
        planes are pipelined in groups (uploads, kernels and downloads of
        successive groups overlap)."""
        self.host_planes(planes).run()

    def host_planes(self, planes: Sequence[tuple]) -> "HostPlanes":
        """The plane descriptors of inverse_2d_planes built once, for
        callers that run the same buffers repeatedly (a frame ring)."""
        return HostPlanes(self, planes)

    # -- device-resident batches ------------------------------------------
    def run_batch(self, tasks: Sequence[PlaneTask], stream: int = 0, synchronize: bool = True):
        arr = _task_array(tasks)
        _check(lib().dsmvc_gb_run_batch(self._h, arr, len(tasks), C.c_void_p(stream or None),
                                        1 if synchronize else 0))

    def prepare_batch(self, tasks: Sequence[PlaneTask], parts: int = 0) -> "PreparedBatch":
        """Routes and uploads `tasks` once; PreparedBatch.launch() then
        issues only the kernels (capturable into a CUDA graph).  `parts`: 1
        or 2 (overlapping halves on two streams), 0 = 2 for 8 tasks or more."""
        return PreparedBatch(self, tasks, parts)

    def stream_check(self, stream: int = 0) -> None:
        _check(lib().dsmvc_gb_stream_check(self._h, C.c_void_p(stream or None)))

    def release_stream(self, stream: int) -> None:
        _check(lib().dsmvc_gb_stream_release(self._h, C.c_void_p(stream or None)))

    def profile(self, enable: bool) -> None:
        _check(lib().dsmvc_gb_profile(self._h, 1 if enable else 0))

    def kernel_times(self) -> list:
        """[{name, launches, milliseconds, bytes}] since profile(True)."""
        buf = (KernelTimeC * 64)()
        n = C.c_int32()
        _check(lib().dsmvc_gb_profile_read(self._h, buf, 64, C.byref(n)))
        return [{"name": buf[i].name.decode(), "launches": buf[i].launches,
                 "milliseconds": buf[i].milliseconds, "bytes": buf[i].bytes}
                for i in range(min(n.value, 64))]


class HostPlanes:
    """A descriptor array for dsmvc_gb_inverse_2d_planes; keeps its plans
    and arrays alive."""

    def __init__(self, executor: Executor, planes: Sequence[tuple]):
        arr = (HostPlaneC * len(planes))()
        keep = []
        for i, pl in enumerate(planes):
            h, v, x, out = pl[:4]
            conversion = pl[4] if len(pl) > 4 else None
            assert x.strides[1] == x.itemsize and out.strides[1] == out.itemsize and x.dtype == out.dtype
            es = x.itemsize
            arr[i] = HostPlaneC(h.handle.value, v.handle.value, x.ctypes.data, x.strides[0] // es,
                                out.ctypes.data, out.strides[0] // es, SAMPLES[x.dtype], _conv(conversion))
            keep += [h, v, x, out]
        self._arr, self._keep, self._executor, self.count = arr, keep, executor, len(planes)

    def run(self) -> None:
        _check(lib().dsmvc_gb_inverse_2d_planes(self._executor._h, self._arr, self.count))


def _task_array(tasks: Sequence[PlaneTask]):
    arr = (PlaneTaskC * len(tasks))()
    for i, t in enumerate(tasks):
        arr[i] = PlaneTaskC(t.horizontal.handle if t.horizontal else None,
                            t.vertical.handle if t.vertical else None,
                            int(t.input), int(t.input_stride), int(t.output),
                            int(t.output_stride), int(t.sample), int(t.vectors),
                            _conv(t.conversion))
    return arr


class PreparedBatch:
    """A task list packed once (dsmvc_gb_batch_create); keeps its executor
    and plans alive.  The task buffers must outlive it."""

    def __init__(self, executor: Executor, tasks: Sequence[PlaneTask], parts: int = 0):
        h = C.c_void_p()
        _check(lib().dsmvc_gb_batch_create_parts(executor._h, _task_array(tasks), len(tasks), int(parts),
                                                 C.byref(h)))
        self._h = h
        self._executor = executor
        executor._dependents.add(self)
        self._plans = [p for t in tasks for p in (t.horizontal, t.vertical) if p is not None]

    def launch(self, stream: int = 0) -> None:
        _check(lib().dsmvc_gb_batch_launch(self._h, C.c_void_p(stream or None)))

    def check(self, stream: int = 0) -> None:
        _check(lib().dsmvc_gb_batch_check(self._h, C.c_void_p(stream or None)))

    def info(self) -> dict:
        k, s, t = C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().dsmvc_gb_batch_info(self._h, C.byref(k), C.byref(s), C.byref(t)))
        parts = C.c_int32()
        _check(lib().dsmvc_gb_batch_parts(self._h, C.byref(parts)))
        return {"kernel_launches": k.value, "scratch_bytes": s.value, "table_bytes": t.value,
                "parts": parts.value}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value and _lib is not None:
            _lib.dsmvc_gb_batch_destroy(self._h)
            self._h = None

    __del__ = close


class Sweep:
    """dsmvc_gb_sweep_*: candidates (h, v) descaled from one device frame,
    re-upscaled and scored (mean absolute error), one CUDA graph per run.
    `fused_scoring`: score each candidate inside its columns pass where it
    allows (its descaled plane never reaches HBM) instead of by a kernel of
    its own over the descaled plane."""

    def __init__(self, executor: Executor, candidates: Sequence[tuple], frame_ptr: int,
                 frame_stride: int, memory_budget: int = 0, autotune: bool = True,
                 graph: bool = True, fused_scoring: bool = False):
        n = len(candidates)
        hs = (C.c_void_p * n)(*[h.handle.value for h, _ in candidates])
        vs = (C.c_void_p * n)(*[v.handle.value for _, v in candidates])
        opts = SweepOptionsC(int(memory_budget), 1 if autotune else 0, 1 if graph else 0,
                             1 if fused_scoring else 0, 0)
        h = C.c_void_p()
        _check(lib().dsmvc_gb_sweep_create(executor._h, hs, vs, n, C.c_void_p(frame_ptr),
                                           int(frame_stride), C.byref(opts), C.byref(h)))
        self._h = h
        self._executor = executor
        executor._dependents.add(self)
        self.count = n

    def run(self, stream: int = 0) -> None:
        _check(lib().dsmvc_gb_sweep_run(self._h, C.c_void_p(stream or None)))

    def run_plain(self, stream: int = 0) -> None:
        _check(lib().dsmvc_gb_sweep_run_plain(self._h, C.c_void_p(stream or None)))

    def scores(self, stream: int = 0) -> np.ndarray:
        out = np.empty(self.count, np.float32)
        _check(lib().dsmvc_gb_sweep_scores(self._h, out.ctypes.data, C.c_void_p(stream or None)))
        return out

    def profile(self, stream: int = 0) -> dict:
        """Stage milliseconds of one ungraphed run."""
        ms = (C.c_double * 3)()
        _check(lib().dsmvc_gb_sweep_profile(self._h, C.c_void_p(stream or None), ms))
        return dict(zip(("descale", "score", "finalize"), list(ms)))

    def info(self) -> dict:
        i = SweepInfoC()
        _check(lib().dsmvc_gb_sweep_get_info(self._h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in i._fields_}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value and _lib is not None:
            _lib.dsmvc_gb_sweep_destroy(self._h)
            self._h = None

    __del__ = close


class Server:
    """dsmvc_gb_server_*: continuous batching of host-frame requests.
    A request is a list of planes (h, v, input, output[, conversion]) with
    2D numpy arrays (rows contiguous); the arrays are kept alive until the
    request is waited for."""

    def __init__(self, executor: Executor, memory_budget: int = 0, streams: int = 4,
                 max_batch: int = 32):
        h = C.c_void_p()
        opts = ServerOptionsC(int(memory_budget), int(streams), int(max_batch))
        _check(lib().dsmvc_gb_server_create(executor._h, C.byref(opts), C.byref(h)))
        self._h = h
        self._executor = executor
        executor._dependents.add(self)
        self._held = {}

    def submit(self, planes: Sequence[tuple]) -> int:
        arr = (HostPlaneC * len(planes))()
        keep = []
        for i, pl in enumerate(planes):
            h, v, x, out = pl[:4]
            conversion = pl[4] if len(pl) > 4 else None
            assert x.strides[1] == x.itemsize and out.strides[1] == out.itemsize
            assert x.dtype == out.dtype
            es = x.itemsize
            arr[i] = HostPlaneC(h.handle.value, v.handle.value, x.ctypes.data, x.strides[0] // es,
                                 out.ctypes.data, out.strides[0] // es, SAMPLES[x.dtype],
                                 _conv(conversion))
            keep += [h, v, x, out]
        t = C.c_uint64()
        _check(lib().dsmvc_gb_server_submit(self._h, arr, len(planes), C.byref(t)))
        self._held[t.value] = keep
        return t.value

    def wait(self, ticket: int) -> None:
        rc = lib().dsmvc_gb_server_wait(self._h, C.c_uint64(ticket))
        self._held.pop(ticket, None)
        _check(rc)

    def done(self, ticket: int) -> bool:
        d = C.c_int32()
        _check(lib().dsmvc_gb_server_poll(self._h, C.c_uint64(ticket), C.byref(d)))
        return bool(d.value)

    def stats(self) -> dict:
        s = ServerStatsC()
        _check(lib().dsmvc_gb_server_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def reset_stats(self) -> None:
        _check(lib().dsmvc_gb_server_reset_stats(self._h))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value and _lib is not None:
            _lib.dsmvc_gb_server_destroy(self._h)
            self._h = None
            self._held.clear()

    __del__ = close


NOALLOC_SCRATCH_BYTES = 32 << 20


def inverse_2d_noalloc(h: AxisPlan, v: AxisPlan, sample: int, input_ptr: int, input_stride: int,
                       output_ptr: int, output_stride: int, conversion=None, stream: int = 0) -> None:
    """Allocation-free 2D descale on device pointers (see the C header):
    for callers that cannot allocate device memory.  Float32 route only;
    frames whose scratch (plans, intermediate, and a forward plane for
    integer output) exceeds NOALLOC_SCRATCH_BYTES are rejected; the plan
    uploads come from pageable memory, so the call may block and is refused
    on a capturing stream; calls that overlap on the GPU race on the shared
    scratch array."""
    conv = _conv(conversion)
    _check(lib().dsmvc_gb_inverse_2d_noalloc(h.handle, v.handle, int(sample), C.c_void_p(input_ptr),
                                             int(input_stride), C.c_void_p(output_ptr),
                                             int(output_stride), C.byref(conv),
                                             C.c_void_p(stream or None)))


def integer_conversion(bits: int, chroma: bool, full_range: bool) -> tuple:
    """integer_conversion (src/vs_plugin.cpp:761-782): returns
    (input_offset, input_scale, output_scale, output_offset, output_maximum)."""
    maximum = (1 << bits) - 1
    offset, scale = 0, maximum
    if not full_range:
        depth = 1 << (bits - 8)
        offset = (128 if chroma else 16) * depth
        scale = (224 if chroma else 219) * depth
    elif chroma:
        offset = 1 << (bits - 1)
    return (float(offset), float(np.float32(1.0) / np.float32(scale)), float(scale),
            float(offset), maximum)


from .plugin import (Debicubic, Debilinear, Delanczos, Descale, Despline16,  # noqa: E402
                     Despline36, Despline64, Frame, VideoFormat)
