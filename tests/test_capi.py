"""The C-ABI library loads and exports every symbol include/dsmvc_gb300.h
declares; no compute call is made here (CPU)."""
import os
import re
import subprocess

from conftest import REPO

HEADER = os.path.join(REPO, "include", "dsmvc_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(dsmvc_gb_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree(gb):
    assert declared_symbols() == sorted(gb.SIGNATURES)


def test_library_exports_every_declared_symbol(gb):
    out = subprocess.run(["nm", "-D", "--defined-only", gb.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (dsmvc_gb_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    lib = gb.lib()
    for s in declared_symbols():
        assert hasattr(lib, s)


def test_abi_version(gb):
    assert gb.lib().dsmvc_gb_abi_version() == 1


def test_executor_without_device_is_unavailable(gb):
    if gb.cuda_available():
        return
    import pytest
    with pytest.raises(gb.DescaleError) as e:
        gb.Executor(0)
    assert e.value.code == gb.UNAVAILABLE


def test_library_does_not_link_the_oracle(gb):
    out = subprocess.run(["nm", "-D", gb.LIB_PATH], capture_output=True, text=True).stdout
    assert "orc_" not in out and "ref_" not in out.replace("_ref", "")


def test_bench_host_calls_driver_builds(gb, tmp_path):
    """bench.py's native per-plane driver (bench_host_calls.cpp) compiles
    against the header and library; it refuses a wrong argument count, and
    on a machine without a GPU reports the executor error as its JSON line."""
    import json
    exe = str(tmp_path / "bench_host_calls")
    lib_dir = os.path.dirname(gb.LIB_PATH)
    subprocess.run(["g++", "-std=c++20", "-O1", "-Wall", "-Wextra", "-pthread",
                    "-I", os.path.join(REPO, "include"), os.path.join(REPO, "bench_host_calls.cpp"),
                    "-L", lib_dir, "-ldsmvc_gb300", f"-Wl,-rpath,{lib_dir}", "-o", exe], check=True)
    r = subprocess.run([exe, "1"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in json.loads(r.stdout)["error"]
    if gb.cuda_available():
        return
    req = "1920,1440,1440.0,0.0,2,3,0.0,0.5,1.0,1,0"
    conv = "4096.0,1.7e-05,56064.0,4096.0,65535"
    r = subprocess.run([exe, "2", "1", "1", req, req, req, req, conv, conv], capture_output=True, text=True)
    assert r.returncode == 1 and "executor" in json.loads(r.stdout)["error"]
