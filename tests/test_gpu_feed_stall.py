"""Bounded feed waits: with DSMVC_GB_FEED_STALL_TEST=1 the chunk-delayed
kernels' staged feeds wait for a barrier phase that nothing completes, so
every wait runs out (about 65 ms, bounded); the kernels finish, set the
status word, and the host call and the prepared batch's check raise.  No
fault, no hang: the same context keeps serving calls, bit for bit as before."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = (192, 144, 144.0, 0.0, "lanczos", 3, 0.0, 0.5, 1.0, "repeat", 0)
V = (108, 81, 81.0, 0.0, "lanczos", 3, 0.0, 0.5, 1.0, "repeat", 0)


def _stalling_executor(gb):
    os.environ["DSMVC_GB_FEED_STALL_TEST"] = "1"
    try:
        return gb.Executor(0)
    finally:
        del os.environ["DSMVC_GB_FEED_STALL_TEST"]


def test_stalled_feed_is_reported_and_the_context_survives(gb, executor):
    torch = pytest.importorskip("torch")
    h, v = gb.AxisPlan(gb.AxisRequest(*H)), gb.AxisPlan(gb.AxisRequest(*V))
    rng = np.random.default_rng(3)
    x = (rng.random((108, 192)) * 56064 + 4096).astype(np.uint16)
    conv = gb.integer_conversion(16, chroma=False, full_range=False)
    want = executor.inverse_2d(h, v, x, conv)
    assert h.stream_info()["ring_ok_transposed"] and v.stream_info()["ring_ok_transposed"]
    ex = _stalling_executor(gb)
    try:
        for _ in range(2):
            with pytest.raises(gb.DescaleError, match="feed wait ran out"):
                ex.inverse_2d(h, v, x, conv)
        # A prepared batch reports through its own status word.
        dx = torch.from_numpy(x.view(np.int16)).cuda()
        dy = torch.zeros((81, 144), dtype=torch.int16, device="cuda")
        batch = ex.prepare_batch([gb.PlaneTask(h, v, dx.data_ptr(), 192, dy.data_ptr(), 144, 2, 0, conv)])
        sid = torch.cuda.current_stream().cuda_stream
        batch.launch(sid)
        with pytest.raises(gb.DescaleError, match="feed wait ran out"):
            batch.check(sid)
        batch.close()
    finally:
        ex.close()
    torch.cuda.synchronize()
    # The context is intact: the same call gives the same bytes.
    assert np.array_equal(executor.inverse_2d(h, v, x, conv), want)
