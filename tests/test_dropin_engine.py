"""The maintainer's switch-over carried out on the reference engine itself:
its own src/executor.cpp and src/backend.cpp, with the CUDA backend replaced
by the drop-in class (adapter/gb300_cuda_executor.*) in the three places a
maintainer changes (the include, the executor type, the two device probes), are
compiled with DSMVC_HAS_CUDA and linked with the rest of the reference engine
(the objects oracle/ref built from its sources) and libdsmvc_gb300.so.
tests/adapter/dropin_check.cpp then drives it through the reference's public
API only:

  * CPU: the capability table lists the CUDA backend as compiled and available
    exactly when a GPU is; without one, Executor(BackendKind::cuda) is refused;
  * GPU: Executor(BackendKind::cuda) descales prepared Delanczos 1080p -> 810p
    luma within 1 code of Executor(BackendKind::cpu, CpuPath::scalar) and bit
    for bit like the GB300 C ABI's own call.

The patched sources are written to a temporary folder at test time (nothing
of the reference is copied into the repository).  Skipped where the
reference headers or the reference engine's objects are absent."""
import os
import platform
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(REPO, "vapoursynth-descalemvc_gb300", "adapter")
PKG_LIB = os.path.join(REPO, "vapoursynth-descalemvc_gb300", "dsmvc_gb300")

# The switch-over, as (file, old, new, expected count).
SWITCH = [
    ("src/executor.cpp", '#include "cuda/cuda_executor.hpp"', '#include "gb300_cuda_executor.hpp"', 1),
    ("src/executor.cpp", "cuda_detail::CudaExecutor", "gb300_detail::Gb300Executor", 3),
    ("src/backend.cpp", '#include "cuda/cuda_executor.hpp"', '#include "gb300_cuda_executor.hpp"', 1),
    ("src/backend.cpp", "cuda_detail::backend_available()", "gb300_detail::backend_available()", 2),
]
ENGINE_OBJECTS = ["axis_plan", "cpu_executor", "host_blocks", "host_copy", "solve_partition"]
SIMD = {"x86_64": (["cpu_executor_avx2", "cpu_executor_avx2_fixed", "cpu_executor_avx512"],
                   ["-DDSMVC_HAS_AVX2_OBJECT=1", "-DDSMVC_HAS_AVX512_OBJECT=1"]),
        "aarch64": (["cpu_executor_neon"], ["-DDSMVC_HAS_NEON_OBJECT=1"])}


@pytest.fixture(scope="module")
def dropin_check(gb, tmp_path_factory):
    import reference
    root = reference.reference_root()
    if root is None or not reference.available():
        pytest.skip("reference headers or engine not present on this machine")
    arch = platform.machine()
    objdir = os.path.join(REPO, "oracle", "_ref", f"obj-{arch}")
    simd_objs, simd_defs = SIMD.get(arch, ([], []))
    objs = [os.path.join(objdir, n + ".o") for n in ENGINE_OBJECTS + simd_objs]
    if not all(os.path.exists(o) for o in objs):
        pytest.skip("the reference engine's objects are not built for this CPU")
    tmp = tmp_path_factory.mktemp("dropin")
    patched = {}
    for rel, old, new, count in SWITCH:
        text = patched.get(rel) or open(os.path.join(root, rel)).read()
        assert text.count(old) == count, (rel, old, text.count(old))
        patched[rel] = text.replace(old, new)
    sources = []
    for rel, text in patched.items():
        path = tmp / os.path.basename(rel)
        path.write_text(text)
        sources.append(str(path))
    exe = str(tmp / "dropin_check")
    cmd = (["g++", "-std=c++23", "-O1", "-pthread", "-ffp-contract=off", "-DDSMVC_HAS_CUDA=1"] + simd_defs
           + ["-I", os.path.join(root, "include"), "-I", os.path.join(root, "src"), "-I", ADAPTER,
              "-I", os.path.join(REPO, "include")]
           + sources + [os.path.join(ADAPTER, "gb300_cuda_executor.cpp"),
                        os.path.join(REPO, "tests", "adapter", "dropin_check.cpp")] + objs
           + ["-L", PKG_LIB, "-ldsmvc_gb300", f"-Wl,-rpath,{PKG_LIB}", "-o", exe])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def _run(exe, mode):
    r = subprocess.run([exe, mode], capture_output=True, text=True, timeout=600)
    sys.stdout.write(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_reference_engine_lists_the_gb300_backend(dropin_check):
    assert "caps ok" in _run(dropin_check, "caps")


@pytest.mark.gpu
def test_reference_executor_runs_on_the_gb300_backend(dropin_check):
    assert "dropin gpu ok" in _run(dropin_check, "gpu")
