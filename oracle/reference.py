"""ctypes binding of the reference's own CPU engine built by oracle/ref
(test infrastructure only; the library exists where the reference sources
were present at build time, i.e. not on machines without them).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libdsmvc_ref.so")
REFERENCE_ROOT = "/root/reference"

from oracle import Request, Conversion, ERRORS  # noqa: E402

_lib = None


def available() -> bool:
    if os.path.exists(LIB_PATH):
        try:
            lib()
            return True
        except OSError:
            return False
    return False


def build() -> bool:
    """Compile the reference engine when its sources are present."""
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "src")):
        return False
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref"),
                    f"REF={REFERENCE_ROOT}"], check=True)
    return True


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB_PATH)
        L.ref_plan_build.argtypes = [C.POINTER(Request), C.POINTER(C.c_void_p)]
        L.ref_plan_free.argtypes = [C.c_void_p]
        L.ref_plan_array.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
        L.ref_plan_array.restype = C.c_size_t
        L.ref_plan_ints.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        L.ref_plan_rcond.argtypes = [C.c_void_p]
        L.ref_plan_rcond.restype = C.c_double
        for name in ("ref_inverse_rows", "ref_inverse_columns"):
            getattr(L, name).argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_ssize_t,
                                         C.c_void_p, C.c_ssize_t, C.c_int32]
        L.ref_inverse_2d.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_ssize_t, C.c_void_p, C.c_ssize_t]
        for name in ("ref_inverse_2d_u8", "ref_inverse_2d_u16"):
            getattr(L, name).argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_ssize_t, C.c_void_p, C.c_ssize_t,
                                         C.POINTER(Conversion)]
        _lib = L
    return _lib


def _check(status, what):
    if status:
        raise ERRORS.get(status, RuntimeError)(f"reference {what} failed ({status})")


_ARRAYS = [("transpose_offsets", np.uint32), ("transpose_indices", np.int32),
           ("transpose_weights", np.float32), ("lower_ld", np.float32),
           ("upper_l", np.float32), ("inverse_diagonal", np.float32),
           ("transpose_weights_f64", np.float64), ("normal_bands_f64", np.float64),
           ("ldlt_bands_f64", np.float64), ("inverse_diagonal_f64", np.float64)]


class Plan:
    def __init__(self, request: Request):
        self.request = request
        h = C.c_void_p()
        _check(lib().ref_plan_build(C.byref(request), C.byref(h)), "plan build")
        self._h = h
        ints = (C.c_int32 * 5)()
        lib().ref_plan_ints(h, ints)
        (self.source_size, self.destination_size, self.support,
         self.half_bandwidth, f64) = list(ints)
        self.requires_float64 = bool(f64)
        self.normal_rcond = lib().ref_plan_rcond(h)
        for i, (name, dt) in enumerate(_ARRAYS):
            ptr = C.c_void_p()
            n = lib().ref_plan_array(h, i, C.byref(ptr))
            if n:
                buf = (C.c_char * (n * np.dtype(dt).itemsize)).from_address(ptr.value)
                setattr(self, name, np.frombuffer(buf, dt).copy())
            else:
                setattr(self, name, np.zeros(0, dt))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ref_plan_free(self._h)
            self._h = None


def inverse_rows(plan, x, path=0):
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty((x.shape[0], plan.destination_size), np.float32)
    _check(lib().ref_inverse_rows(path, plan._h, x.ctypes.data, x.shape[1],
                                  out.ctypes.data, out.shape[1], x.shape[0]), "rows")
    return out


def inverse_columns(plan, x, path=0):
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty((plan.destination_size, x.shape[1]), np.float32)
    _check(lib().ref_inverse_columns(path, plan._h, x.ctypes.data, x.shape[1],
                                     out.ctypes.data, out.shape[1], x.shape[1]), "columns")
    return out


def inverse_2d(h, v, x, conversion=None, path=0, out=None):
    x = np.ascontiguousarray(x)
    if out is None:
        out = np.empty((v.destination_size, h.destination_size), x.dtype)
    if x.dtype == np.float32:
        _check(lib().ref_inverse_2d(path, h._h, v._h, x.ctypes.data, x.shape[1],
                                    out.ctypes.data, out.shape[1]), "inverse_2d")
        return out
    conv = Conversion(*conversion)
    fn = lib().ref_inverse_2d_u8 if x.dtype == np.uint8 else lib().ref_inverse_2d_u16
    _check(fn(path, h._h, v._h, x.ctypes.data, x.shape[1], out.ctypes.data,
              out.shape[1], C.byref(conv)), "inverse_2d_integer")
    return out
