"""ctypes binding of the CPU oracle (test infrastructure only).

Tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
use it as the checker; nothing in the shipped package imports it.  The
oracle restates the reference's planner (src/axis_plan.cpp) and its
CpuExecutor scalar routes (src/cpu_executor.cpp) in plain C.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

KINDS = {"bilinear": 0, "bicubic": 1, "lanczos": 2, "spline16": 3,
         "spline36": 4, "spline64": 5, "custom": 6}
BORDERS = {"zero": 0, "repeat": 1, "reflect101": 2, "symmetric": 3,
           "mirror": 4}

ERRORS = {1: ValueError, 2: RuntimeError, 3: OverflowError, 4: MemoryError}


class Request(C.Structure):
    _fields_ = [("source_size", C.c_int32), ("destination_size", C.c_int32),
                ("active_length", C.c_double), ("shift", C.c_double),
                ("kind", C.c_int32), ("taps", C.c_int32),
                ("b", C.c_double), ("c", C.c_double), ("blur", C.c_double),
                ("border", C.c_int32), ("f64_mode", C.c_int32)]


class Conversion(C.Structure):
    _fields_ = [("input_offset", C.c_float), ("input_scale", C.c_float),
                ("output_scale", C.c_float), ("output_offset", C.c_float),
                ("output_maximum", C.c_uint32)]


class _Plan(C.Structure):
    _fields_ = [("source_size", C.c_int32), ("destination_size", C.c_int32),
                ("support", C.c_int32), ("half_bandwidth", C.c_int32),
                ("active_length", C.c_double), ("shift", C.c_double),
                ("normal_rcond", C.c_double), ("normal_inf_norm", C.c_double),
                ("nnz", C.c_size_t),
                ("transpose_offsets", C.POINTER(C.c_uint32)),
                ("transpose_indices", C.POINTER(C.c_int32)),
                ("transpose_weights", C.POINTER(C.c_float)),
                ("lower_ld", C.POINTER(C.c_float)),
                ("upper_l", C.POINTER(C.c_float)),
                ("inverse_diagonal", C.POINTER(C.c_float)),
                ("has_f64", C.c_int32),
                ("transpose_weights_f64", C.POINTER(C.c_double)),
                ("normal_bands_f64", C.POINTER(C.c_double)),
                ("ldlt_bands_f64", C.POINTER(C.c_double)),
                ("inverse_diagonal_f64", C.POINTER(C.c_double))]


CUSTOM_FN = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)

_lib = None


def build() -> str:
    """Compile the oracle with its Makefile (plain gcc, any architecture)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER(_Plan)
        L.orc_plan_build.argtypes = [C.POINTER(Request), CUSTOM_FN, C.c_void_p,
                                     C.POINTER(P)]
        L.orc_plan_free.argtypes = [P]
        L.orc_f32_plan_hash.argtypes = [C.POINTER(Request), P]
        L.orc_f32_plan_hash.restype = C.c_uint64
        L.orc_complete_plan_hash.argtypes = [C.POINTER(Request), P]
        L.orc_complete_plan_hash.restype = C.c_uint64
        L.orc_output_hash_f32.argtypes = [C.c_void_p, C.c_size_t]
        L.orc_output_hash_f32.restype = C.c_uint64
        L.orc_output_hash_f64.argtypes = [C.c_void_p, C.c_size_t]
        L.orc_output_hash_f64.restype = C.c_uint64
        L.orc_make_normal_input.argtypes = [C.c_void_p, C.c_size_t, C.c_uint32]
        L.orc_padding_index.argtypes = [C.c_int64, C.c_int32, C.c_int32]
        L.orc_padding_index.restype = C.c_int32
        for name in ("orc_inverse_axis_f32", "orc_inverse_axis_f32_ordered",
                     "orc_inverse_axis_f64", "orc_inverse_axis_f64_ordered"):
            getattr(L, name).argtypes = [P, C.c_void_p, C.c_ssize_t,
                                         C.c_void_p, C.c_ssize_t]
        for name in ("orc_inverse_rows", "orc_inverse_columns"):
            getattr(L, name).argtypes = [P, C.c_void_p, C.c_ssize_t,
                                         C.c_void_p, C.c_ssize_t, C.c_int32]
        L.orc_inverse_2d.argtypes = [P, P, C.c_void_p, C.c_ssize_t,
                                     C.c_void_p, C.c_ssize_t]
        L.orc_inverse_axis_f32_gpu.argtypes = [P, C.c_void_p, C.c_ssize_t,
                                               C.c_void_p, C.c_ssize_t]
        L.orc_inverse_2d_gpu_order.argtypes = [P, P, C.c_int, C.c_void_p, C.c_ssize_t,
                                               C.c_void_p, C.c_ssize_t,
                                               C.POINTER(Conversion)]
        for name in ("orc_inverse_2d_u8", "orc_inverse_2d_u16"):
            getattr(L, name).argtypes = [P, P, C.c_void_p, C.c_ssize_t,
                                         C.c_void_p, C.c_ssize_t,
                                         C.POINTER(Conversion)]
        _lib = L
    return _lib


def _check(status: int, what: str) -> None:
    if status:
        raise ERRORS.get(status, RuntimeError)(f"oracle {what} failed ({status})")


def make_request(source, destination, active_length=None, shift=0.0,
                 kernel="bicubic", taps=3, b=0.0, c=0.5, blur=1.0,
                 border="symmetric", f64_mode=0) -> Request:
    return Request(int(source), int(destination),
                   float(destination if active_length is None else active_length),
                   float(shift), KINDS[kernel] if isinstance(kernel, str) else int(kernel),
                   int(taps), float(b), float(c), float(blur),
                   BORDERS[border] if isinstance(border, str) else int(border),
                   int(f64_mode))


class Plan:
    """An oracle axis plan; arrays are copied out as numpy views."""

    def __init__(self, request: Request, custom=None):
        self.request = request
        self._custom = CUSTOM_FN(lambda x, _u: float(custom(x))) if custom else CUSTOM_FN()
        ptr = C.POINTER(_Plan)()
        _check(lib().orc_plan_build(C.byref(request), self._custom, None,
                                    C.byref(ptr)), "plan build")
        self._ptr = ptr
        p = ptr.contents
        self.source_size = p.source_size
        self.destination_size = p.destination_size
        self.support = p.support
        self.half_bandwidth = p.half_bandwidth
        self.normal_rcond = p.normal_rcond
        self.normal_inf_norm = p.normal_inf_norm
        self.requires_float64 = bool(p.has_f64)
        n, hb, nnz = p.destination_size, p.half_bandwidth, p.nnz

        def arr(ptr_, count, dtype):
            if count == 0:
                return np.zeros(0, dtype)
            return np.ctypeslib.as_array(ptr_, shape=(count,)).astype(dtype, copy=True)

        self.transpose_offsets = arr(p.transpose_offsets, n + 1, np.uint32)
        self.transpose_indices = arr(p.transpose_indices, nnz, np.int32)
        self.transpose_weights = arr(p.transpose_weights, nnz, np.float32)
        self.lower_ld = arr(p.lower_ld, hb * n, np.float32)
        self.upper_l = arr(p.upper_l, hb * n, np.float32)
        self.inverse_diagonal = arr(p.inverse_diagonal, n, np.float32)
        if p.has_f64:
            self.transpose_weights_f64 = arr(p.transpose_weights_f64, nnz, np.float64)
            self.normal_bands_f64 = arr(p.normal_bands_f64, (hb + 1) * n, np.float64)
            self.ldlt_bands_f64 = arr(p.ldlt_bands_f64, (hb + 1) * n, np.float64)
            self.inverse_diagonal_f64 = arr(p.inverse_diagonal_f64, n, np.float64)

    def __del__(self):
        if getattr(self, "_ptr", None) and _lib is not None:
            _lib.orc_plan_free(self._ptr)
            self._ptr = None

    def f32_hash(self) -> str:
        return "%016x" % lib().orc_f32_plan_hash(C.byref(self.request), self._ptr)

    def complete_hash(self) -> str:
        return "%016x" % lib().orc_complete_plan_hash(C.byref(self.request), self._ptr)

    # -- single-axis solves ---------------------------------------------
    def inverse_axis_f32(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        out = np.empty(self.destination_size, np.float32)
        _check(lib().orc_inverse_axis_f32(self._ptr, x.ctypes.data, 1,
                                          out.ctypes.data, 1), "inverse_axis_f32")
        return out

    def inverse_axis_f32_ordered(self, x):
        x = np.ascontiguousarray(x, np.float32)
        out = np.empty(self.destination_size, np.float32)
        lib().orc_inverse_axis_f32_ordered(self._ptr, x.ctypes.data, 1, out.ctypes.data, 1)
        return out

    def inverse_axis_f32_gpu(self, x):
        """Reference CUDA operation order (fmaf chains)."""
        x = np.ascontiguousarray(x, np.float32)
        out = np.empty(self.destination_size, np.float32)
        lib().orc_inverse_axis_f32_gpu(self._ptr, x.ctypes.data, 1, out.ctypes.data, 1)
        return out

    def inverse_axis_f64(self, x):
        x = np.ascontiguousarray(x, np.float64)
        out = np.empty(self.destination_size, np.float64)
        lib().orc_inverse_axis_f64(self._ptr, x.ctypes.data, 1, out.ctypes.data, 1)
        return out

    def inverse_axis_f64_ordered(self, x):
        x = np.ascontiguousarray(x, np.float64)
        out = np.empty(self.destination_size, np.float64)
        lib().orc_inverse_axis_f64_ordered(self._ptr, x.ctypes.data, 1, out.ctypes.data, 1)
        return out


def output_hash(values: np.ndarray) -> str:
    v = np.ascontiguousarray(values)
    if v.dtype == np.float64:
        return "%016x" % lib().orc_output_hash_f64(v.ctypes.data, v.size)
    v = np.ascontiguousarray(v, np.float32)
    return "%016x" % lib().orc_output_hash_f32(v.ctypes.data, v.size)


def make_normal_input(count: int, seed: int) -> np.ndarray:
    out = np.empty(count, np.float32)
    lib().orc_make_normal_input(out.ctypes.data, count, seed & 0xFFFFFFFF)
    return out


def inverse_rows(plan: Plan, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty((x.shape[0], plan.destination_size), np.float32)
    _check(lib().orc_inverse_rows(plan._ptr, x.ctypes.data, x.shape[1],
                                  out.ctypes.data, out.shape[1], x.shape[0]),
           "inverse_rows")
    return out


def inverse_columns(plan: Plan, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty((plan.destination_size, x.shape[1]), np.float32)
    _check(lib().orc_inverse_columns(plan._ptr, x.ctypes.data, x.shape[1],
                                     out.ctypes.data, out.shape[1], x.shape[1]),
           "inverse_columns")
    return out


def inverse_2d(h: Plan, v: Plan, x: np.ndarray, conversion=None) -> np.ndarray:
    """CpuExecutor(scalar).inverse_2d / inverse_2d_u8 / inverse_2d_u16."""
    x = np.ascontiguousarray(x)
    out = np.empty((v.destination_size, h.destination_size), x.dtype)
    if x.dtype == np.float32:
        _check(lib().orc_inverse_2d(h._ptr, v._ptr, x.ctypes.data, x.shape[1],
                                    out.ctypes.data, out.shape[1]), "inverse_2d")
        return out
    conv = Conversion(*conversion)
    fn = {np.dtype(np.uint8): lib().orc_inverse_2d_u8,
          np.dtype(np.uint16): lib().orc_inverse_2d_u16}[x.dtype]
    _check(fn(h._ptr, v._ptr, x.ctypes.data, x.shape[1], out.ctypes.data,
              out.shape[1], C.byref(conv)), "inverse_2d_integer")
    return out


def inverse_2d_into(h: Plan, v: Plan, x: np.ndarray, out: np.ndarray,
                    conversion=None) -> None:
    """Same as inverse_2d, writing into a preallocated array (no Python
    allocation in the timed loop of the CPU baseline)."""
    if x.dtype == np.float32:
        _check(lib().orc_inverse_2d(h._ptr, v._ptr, x.ctypes.data, x.shape[1],
                                    out.ctypes.data, out.shape[1]), "inverse_2d")
        return
    conv = Conversion(*conversion)
    fn = lib().orc_inverse_2d_u8 if x.dtype == np.uint8 else lib().orc_inverse_2d_u16
    _check(fn(h._ptr, v._ptr, x.ctypes.data, x.shape[1], out.ctypes.data,
              out.shape[1], C.byref(conv)), "inverse_2d_integer")


def inverse_2d_gpu_order(h: Plan, v: Plan, x: np.ndarray, conversion=None) -> np.ndarray:
    """Float32 2D in the reference CUDA kernels' operation order: the exact
    expectation of the sequential GB300 kernels."""
    x = np.ascontiguousarray(x)
    out = np.empty((v.destination_size, h.destination_size), x.dtype)
    kind = {np.dtype(np.float32): 0, np.dtype(np.uint8): 1, np.dtype(np.uint16): 2}[x.dtype]
    conv = Conversion(*(conversion or (0.0, 1.0, 1.0, 0.0, 255)))
    _check(lib().orc_inverse_2d_gpu_order(h._ptr, v._ptr, kind, x.ctypes.data, x.shape[1],
                                          out.ctypes.data, out.shape[1], C.byref(conv)),
           "inverse_2d_gpu_order")
    return out


def inverse_rows_gpu_order(plan: Plan, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    return np.stack([plan.inverse_axis_f32_gpu(r) for r in x])


def inverse_columns_gpu_order(plan: Plan, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    return np.stack([plan.inverse_axis_f32_gpu(c) for c in x.T]).T.copy()
