import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("", "oracle", "vapoursynth-descalemvc_gb300", "tests"):
    path = os.path.join(REPO, sub)
    if path not in sys.path:
        sys.path.insert(0, path)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def _ensure_library():
    import dsmvc_gb300
    if not os.path.exists(dsmvc_gb300.LIB_PATH):
        dsmvc_gb300.build()
    return dsmvc_gb300


@pytest.fixture(scope="session")
def gb():
    """The product package with its library loaded."""
    mod = _ensure_library()
    mod.lib()
    return mod


@pytest.fixture(scope="session")
def executor(gb):
    if not gb.cuda_available():
        pytest.skip("no CUDA device")
    ex = gb.Executor(0)
    yield ex
    ex.close()


def _executor_with(gb, name, value="0", **more):
    """An executor created under environment settings (name=value and
    `more`), restored afterwards."""
    if not gb.cuda_available():
        pytest.skip("no CUDA device")
    settings = {name: value, **more}
    old = {k: os.environ.get(k) for k in settings}
    os.environ.update(settings)
    try:
        return gb.Executor(0)
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


@pytest.fixture(scope="session")
def seq_executor(gb):
    """An executor pinned to the sequential kernels (DSMVC_GB_STREAM=0)."""
    ex = _executor_with(gb, "DSMVC_GB_STREAM")
    yield ex
    ex.close()


@pytest.fixture(scope="session")
def exact_executor(gb):
    """An executor whose admitted 2D planes use the two-pass transposing
    kernels (DSMVC_GB_EXACT=1) on whole vectors (DSMVC_GB_SEGMENTS=1): bit
    for bit the reference CUDA operation order."""
    ex = _executor_with(gb, "DSMVC_GB_EXACT", "1", DSMVC_GB_SEGMENTS="1")
    yield ex
    ex.close()


@pytest.fixture(scope="session")
def f64_exact_executor(gb):
    """An executor whose Float64 two-pass kernels run the CPU scalar route's
    operation order (DSMVC_GB_F64_EXACT=1): bit for bit its results; the
    default fused kernels stay within 1 float32 ULP / 1 code of them."""
    ex = _executor_with(gb, "DSMVC_GB_F64_EXACT", "1")
    yield ex
    ex.close()


@pytest.fixture(scope="session")
def paired_executor(gb):
    """An executor whose admitted 2D planes use the paired transposing
    kernels (DSMVC_GB_PAIRED=1)."""
    ex = _executor_with(gb, "DSMVC_GB_PAIRED", "1")
    yield ex
    ex.close()


@pytest.fixture(scope="session")
def whole_executor(gb):
    """An executor that never splits vectors into segments
    (DSMVC_GB_SEGMENTS=1): its results do not depend on what else shares a
    launch, so batched and single calls agree bit for bit."""
    ex = _executor_with(gb, "DSMVC_GB_SEGMENTS", "1")
    yield ex
    ex.close()
