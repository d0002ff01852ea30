"""Host block registry with CUDA's registration: pageable frames that a frame
host reports twice are page-locked (cudaHostRegister) and unregistered on
release, a block page-locked elsewhere is used but left alone, and the
executor's results from registered frames are the same bytes as from
unregistered ones."""
import numpy as np
import pytest

from common import make_input, product_request

pytestmark = pytest.mark.gpu

LUMA_H = (1920, 1440, 1440.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "symmetric", 1)
LUMA_V = (1080, 810, 810.0, 0.0, "lanczos", 3, 0, 0.5, 1.0, "symmetric", 1)


def test_registered_frames_descale_alike(gb, executor):
    hb = gb.host_blocks
    hb.test_registrar(0)
    h = gb.AxisPlan(product_request(gb, LUMA_H), cached=False)
    v = gb.AxisPlan(product_request(gb, LUMA_V), cached=False)
    conv = gb.integer_conversion(16, False, False)
    x = make_input(1080, 1920, "u16", 11)
    want = executor.inverse_2d(h, v, x, conv)
    # A frame pool: one pageable input block and one output block, reused.
    src = np.empty_like(x)
    dst = np.zeros((810, 1440), np.uint16)
    owner = 0x5EED
    hb.set_limit(owner, 64 << 20)
    s0 = hb.stats()
    for _ in range(3):
        src[...] = x
        hb.note_array(owner, src)
        hb.note_array(owner, dst)
        executor.inverse_2d(h, v, src, conv, out=dst)
        assert np.array_equal(dst, want)
    s1 = hb.stats()
    assert s1["registrations"] - s0["registrations"] == 2 and s1["failures"] == s0["failures"]
    assert s1["registered_bytes"] - s0["registered_bytes"] == src.nbytes + dst.nbytes
    assert hb.covered(src.ctypes.data, src.nbytes) and hb.covered(dst.ctypes.data, dst.nbytes)
    hb.release(src.ctypes.data, src.nbytes)
    hb.drop_owner(owner)
    s2 = hb.stats()
    assert s2["released"] - s1["released"] == 2 and s2["registered_bytes"] == s0["registered_bytes"]
    # Unregistered again, still the same bytes.
    executor.inverse_2d(h, v, src, conv, out=dst)
    assert np.array_equal(dst, want)


def test_block_registered_elsewhere_is_left_registered(gb):
    torch = pytest.importorskip("torch")
    cudart = torch.cuda.cudart()
    if not hasattr(cudart, "cudaHostRegister"):
        pytest.skip("this torch exposes no cudaHostRegister")
    hb = gb.host_blocks
    hb.test_registrar(0)
    a = np.zeros(4 << 20, np.uint8)
    assert int(cudart.cudaHostRegister(a.ctypes.data, a.nbytes, 0)) == 0
    try:
        owner = 0xF0E
        hb.set_limit(owner, 64 << 20)
        s0 = hb.stats()
        hb.note_array(owner, a)
        hb.note_array(owner, a)
        s1 = hb.stats()
        assert s1["registrations"] - s0["registrations"] == 1
        assert s1["registered_bytes"] == s0["registered_bytes"]
        assert hb.covered(a.ctypes.data, a.nbytes)
        hb.drop_owner(owner)
        assert hb.stats()["released"] == s1["released"]
    finally:
        # Still registered by its owner: unregistering it succeeds.
        assert int(cudart.cudaHostUnregister(a.ctypes.data)) == 0
