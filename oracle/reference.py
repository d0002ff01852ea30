"""ctypes binding of the reference's own CPU engine built by oracle/ref
(test infrastructure only: the checker and the timed CPU baseline).

Where the reference tree is: $DSMVC_REFERENCE if set, else a staged copy of
its engine sources under baseline/_ref/dsmvc (made by `stage()` on a machine
that has the tree, kept out of version control, and carried along with the
working copy so that a machine without the tree can build the engine for its
own CPU), else /root/reference.  The library exists only where one of them
was present at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "_ref", "libdsmvc_ref.so")
STAGED_ROOT = os.path.join(REPO, "baseline", "_ref", "dsmvc")
# The reference engine's CPU sources and headers (src/, include/dsmvc/); no
# CUDA, Vulkan, Metal or VapourSynth file is needed for the CPU routes.
ENGINE_FILES = (
    ["include/dsmvc/engine.hpp", "include/dsmvc/host_blocks.hpp"]
    + ["src/" + f for f in (
        "axis_plan.cpp", "axis_plan_internal.hpp", "backend.cpp", "checked_size.hpp",
        "cpu_executor.cpp", "cpu_executor_avx2.cpp", "cpu_executor_avx2_fixed.cpp",
        "cpu_executor_avx512.cpp", "cpu_executor_neon.cpp", "cpu_float_workspace.hpp",
        "cpu_horizontal_window.hpp", "cpu_packed.hpp", "cpu_rhs_span.hpp", "executor.cpp",
        "host_blocks.cpp", "host_copy.cpp", "host_copy.hpp", "solve_partition.cpp",
        "solve_partition.hpp")])


def _tree_ok(root: str) -> bool:
    return all(os.path.exists(os.path.join(root, f)) for f in ENGINE_FILES)


def reference_root():
    """The reference tree to build from, or None."""
    env = os.environ.get("DSMVC_REFERENCE")
    for root in ([env] if env else []) + [STAGED_ROOT, "/root/reference"]:
        if root and _tree_ok(root):
            return root
    return None


REFERENCE_ROOT = reference_root() or ""

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


def stage() -> bool:
    """Copies the engine's CPU sources from the reference tree into the
    ignored baseline/_ref/dsmvc, so that a machine without the tree (another
    CPU architecture: the NEON route) can build the engine.  No-op when the
    tree is absent or the staged copy is current."""
    env = os.environ.get("DSMVC_REFERENCE")
    src = next((r for r in ([env] if env else []) + ["/root/reference"] if r and _tree_ok(r)), None)
    if src is None or os.path.realpath(src) == os.path.realpath(STAGED_ROOT):
        return False
    for f in ENGINE_FILES:
        dst = os.path.join(STAGED_ROOT, f)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        a = os.path.join(src, f)
        if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(a):
            shutil.copy2(a, dst)
    return True


def build() -> bool:
    """Compile the reference engine (scalar route plus this CPU's SIMD
    route) when a reference tree is present."""
    root = reference_root()
    if root is None:
        return False
    subprocess.run(["make", "-s", f"-j{os.cpu_count() or 8}", "-C", os.path.join(HERE, "ref"),
                    f"REF={root}"], check=True)
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
