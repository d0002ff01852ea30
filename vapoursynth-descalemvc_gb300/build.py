"""Builds libdsmvc_gb300.so in-tree: host C++ with g++, CUDA for sm_103a
with nvcc, translation units compiled in parallel, static CUDA runtime.

    python vapoursynth-descalemvc_gb300/build.py [--force]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "dsmvc_gb300")
LIB = os.path.join(OUT_DIR, "libdsmvc_gb300.so")
BUILD_DIR = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: the planner's FP64 arithmetic must round every multiply
# and add separately (GCC contracts by default on aarch64).
CXXFLAGS = ["-std=c++20", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
            "-Wall", "-Wextra"]
NVCCFLAGS = ARCH + ["-std=c++20", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                    "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]

HOST_SOURCES = ["planner.cpp", "stream_plan.cpp", "executor.cpp", "sweep.cpp", "server.cpp",
                "host_blocks.cpp", "capi.cpp"]
TSTREAM2_SOURCES = [f"tstream2_hb{hb}_k{k}.cu" for hb in (1, 3, 5, 7) for k in (0, 8)]
TSOLVE_SOURCES = ([f"tsolve_hb{hb}.cu" for hb in (1, 3, 5, 7, 9, 11)]
                  + [f"tsolve64_hb{hb}.cu" for hb in (1, 3, 5, 7, 9, 11)])
CUDA_SOURCES = TSTREAM2_SOURCES + TSOLVE_SOURCES + ["kernels.cu", "stream.cu", "stream_hb1.cu", "stream_hb3.cu", "stream_hb5.cu",
                "stream_hb7.cu", "tstream_hb1.cu", "tstream_hb3.cu",
                "tstream_hb5.cu", "tstream_hb7.cu", "tstream_hb1_g.cu", "tstream_hb3_g.cu",
                "tstream_hb5_g.cu", "tstream_hb7_g.cu", "tscore_hb1.cu", "tscore_hb3.cu",
                "tscore_hb5.cu", "tscore_hb7.cu", "noalloc.cu", "score.cu",
                "peak.cu", "gpu_planner.cu", "refine64.cu"]


def cuda_home() -> str:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "dsmvc_gb300.h"))
    jobs, objects = [], []
    for src in HOST_SOURCES + CUDA_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD_DIR, src + ".o")
        objects.append(obj)
        if not force and not _stale(obj, [path] + headers):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc] + NVCCFLAGS + ["-I", INCLUDE, "-c", path, "-o", obj]
        else:
            cmd = ["g++"] + CXXFLAGS + ["-I", INCLUDE, "-I", os.path.join(cuda, "include"),
                                         "-c", path, "-o", obj]
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as pool:
        for out in pool.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or _stale(LIB, objects):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objects
             + ["-cudart", "static", "-Xlinker", "--no-undefined", "-lpthread"])
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))
    sys.exit(0)
