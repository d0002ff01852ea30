"""The drop-in backend for the reference engine
(vapoursynth-descalemvc_gb300/adapter/gb300_cuda_executor.*): a class with
the public interface of the reference's dsmvc::cuda_detail::CudaExecutor
(src/cuda/cuda_executor.hpp:11-110) over the GB300 C ABI.  The test compiles
it against the reference's own include/dsmvc/engine.hpp, links it with the
reference engine built from its sources (oracle/_ref) and with
libdsmvc_gb300.so, and runs tests/adapter/adapter_check.cpp:

  * CPU: plans built by the reference planner import bit-identical to the
    GB300 planner's plans for the same requests (arrays, scalars, plan
    hashes), for eight fixed requests and 400 seeded random ones (every
    kernel, border and Float64 mode); invalid plans are refused like
    AxisPlan::check_valid refuses them;
  * GPU: reference plans run through the adapter, prepared and unprepared,
    Float32, Float64 and u16, give the executor's own results bit for bit;
    the adapter installs the CUDA domain's registrar in the engine's host
    block registry (page-locking frame-pool blocks reported twice) unless
    DSMVC_CUDA_DIRECT_IO=0.

Skipped where the reference headers or the reference engine are absent."""
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(REPO, "vapoursynth-descalemvc_gb300", "adapter")
PKG_LIB = os.path.join(REPO, "vapoursynth-descalemvc_gb300", "dsmvc_gb300")
REF_LIB = os.path.join(REPO, "oracle", "_ref")


@pytest.fixture(scope="module")
def adapter_check(gb, tmp_path_factory):
    import reference
    root = reference.reference_root()
    if root is None or not reference.available():
        pytest.skip("reference headers or engine not present on this machine")
    exe = str(tmp_path_factory.mktemp("adapter") / "adapter_check")
    cmd = ["g++", "-std=c++23", "-O1", "-Wall", "-Wextra", "-pthread",
           "-I", os.path.join(root, "include"), "-I", os.path.join(REPO, "include"), "-I", ADAPTER,
           os.path.join(ADAPTER, "gb300_cuda_executor.cpp"),
           os.path.join(REPO, "tests", "adapter", "adapter_check.cpp"),
           "-L", REF_LIB, "-ldsmvc_ref", "-L", PKG_LIB, "-ldsmvc_gb300",
           f"-Wl,-rpath,{REF_LIB}", f"-Wl,-rpath,{PKG_LIB}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def _run(exe, mode, env=None, *args):
    r = subprocess.run([exe, mode, *args], capture_output=True, text=True, timeout=600,
                       env=None if env is None else {**os.environ, **env})
    sys.stdout.write(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_reference_plans_import_bit_identical(adapter_check):
    out = _run(adapter_check, "plans")
    assert "plans ok: 8 imported bit-identical" in out


def test_random_requests_plan_bit_identical_to_the_reference(adapter_check):
    out = _run(adapter_check, "random", None, "400")
    assert "random plans ok:" in out and "FAIL" not in out


@pytest.mark.gpu
def test_adapter_runs_reference_plans_like_the_executor(adapter_check):
    out = _run(adapter_check, "gpu")
    assert "gpu ok" in out


@pytest.mark.gpu
@pytest.mark.parametrize("direct_io", ["1", "0"])
def test_adapter_registers_frame_pool_blocks(adapter_check, direct_io):
    out = _run(adapter_check, "blocks", {"DSMVC_CUDA_DIRECT_IO": direct_io})
    assert ("blocks ok (registrar installed)" if direct_io == "1" else "blocks ok (no registrar)") in out
