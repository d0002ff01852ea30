"""Host block registry (dsmvc_gb_host_blocks_*): the reference's direct block
registration (include/dsmvc/host_blocks.hpp), checked on the CPU with fake
registrations (the registry's state machine, caps, ownership, releases and
concurrent use).  The page-locking itself is checked under -m gpu in
tests/test_gpu_host_blocks.py."""
import threading

import numpy as np
import pytest

MIB = 1 << 20


@pytest.fixture
def hb(gb):
    gb.host_blocks.test_registrar(1)
    yield gb.host_blocks
    gb.host_blocks.test_registrar(0)


def _delta(hb, before):
    now = hb.stats()
    return {k: now[k] - before[k] for k in now if k not in ("registered_bytes", "peak_bytes")}


def test_second_use_registers_within_the_limit(hb):
    a = np.zeros(2 * MIB, np.uint8)
    base = a.ctypes.data
    hb.set_limit(101, 4 * MIB)
    s0 = hb.stats()
    hb.note_array(101, a)
    assert not hb.covered(base, 16)
    hb.note_array(101, a)
    assert hb.covered(base, a.nbytes) and hb.covered(base + MIB, MIB)
    assert not hb.covered(base + MIB, MIB + 1) and not hb.covered(base - 1, 2)
    d = _delta(hb, s0)
    assert d["registrations"] == 1 and d["failures"] == 0 and d["hits"] == 2 and d["misses"] == 3
    assert hb.stats()["registered_bytes"] == a.nbytes
    hb.note_array(101, a)                       # further uses change nothing
    assert _delta(hb, s0)["registrations"] == 1
    hb.release(base, a.nbytes)
    assert _delta(hb, s0)["released"] == 1 and hb.stats()["registered_bytes"] == 0
    assert not hb.covered(base, 16)


def test_limit_refuses_then_admits(hb):
    a, b = np.zeros(3 * MIB, np.uint8), np.zeros(2 * MIB, np.uint8)
    hb.set_limit(102, 4 * MIB)
    s0 = hb.stats()
    for _ in range(2):
        hb.note_array(102, a)
        hb.note_array(102, b)
    # a fits; b would pass the limit: refused, and tried again on its next use.
    assert hb.covered(a.ctypes.data, a.nbytes) and not hb.covered(b.ctypes.data, b.nbytes)
    assert _delta(hb, s0)["cap_refusals"] == 1
    hb.set_limit(102, 5 * MIB)
    hb.note_array(102, b)
    assert hb.covered(b.ctypes.data, b.nbytes)
    hb.drop_owner(102)
    assert not hb.covered(a.ctypes.data, 1) and not hb.covered(b.ctypes.data, 1)
    assert _delta(hb, s0)["released"] == 2 and hb.stats()["registered_bytes"] == 0


def test_default_limit_registers_nothing(hb):
    a = np.zeros(MIB, np.uint8)
    s0 = hb.stats()
    for _ in range(3):
        hb.note_array(103, a)
    assert not hb.covered(a.ctypes.data, 1)
    d = _delta(hb, s0)
    assert d["registrations"] == 0 and d["cap_refusals"] == 2
    hb.drop_owner(103)


def test_foreign_blocks_are_used_but_never_unregistered(gb):
    hb = gb.host_blocks
    hb.test_registrar(2)
    try:
        a = np.zeros(MIB, np.uint8)
        hb.set_limit(104, MIB)
        s0 = hb.stats()
        hb.note_array(104, a)
        hb.note_array(104, a)
        assert hb.covered(a.ctypes.data, a.nbytes)
        assert _delta(hb, s0)["registrations"] == 1 and hb.stats()["registered_bytes"] == 0
        # The owner's limit is not spent on a foreign block.
        b = np.zeros(MIB, np.uint8)
        hb.note_array(104, b)
        hb.note_array(104, b)
        assert hb.covered(b.ctypes.data, 1)
        hb.release(a.ctypes.data, a.nbytes)
        assert _delta(hb, s0)["released"] == 0 and not hb.covered(a.ctypes.data, 1)
        hb.drop_owner(104)
    finally:
        hb.test_registrar(0)


def test_failed_registration_is_counted_and_not_retried(gb):
    hb = gb.host_blocks
    hb.test_registrar(3)
    try:
        a = np.zeros(MIB, np.uint8)
        hb.set_limit(105, 8 * MIB)
        s0 = hb.stats()
        for _ in range(4):
            hb.note_array(105, a)
        assert not hb.covered(a.ctypes.data, 1)
        d = _delta(hb, s0)
        assert d["failures"] == 1 and d["registrations"] == 0
        hb.drop_owner(105)
    finally:
        hb.test_registrar(0)


def test_address_reused_by_another_block(hb):
    a = np.zeros(2 * MIB, np.uint8)
    base = a.ctypes.data
    hb.set_limit(106, 8 * MIB)
    hb.set_limit(107, 8 * MIB)
    s0 = hb.stats()
    hb.note_use(106, base, MIB)
    hb.note_use(106, base, MIB)
    assert hb.covered(base, MIB) and not hb.covered(base, MIB + 1)
    # Same address, another size (the pool reused it): the old block goes,
    # the new one starts counting uses again.
    hb.note_use(106, base, 2 * MIB)
    assert not hb.covered(base, 1) and _delta(hb, s0)["released"] == 1
    hb.note_use(106, base, 2 * MIB)
    assert hb.covered(base, 2 * MIB)
    # Another owner at the same address.
    hb.note_use(107, base, 2 * MIB)
    assert not hb.covered(base, 1)
    hb.drop_owner(106)
    hb.drop_owner(107)
    assert hb.stats()["registered_bytes"] == 0


def test_switching_registrars_releases_everything(gb):
    hb = gb.host_blocks
    hb.test_registrar(1)
    a = np.zeros(MIB, np.uint8)
    hb.set_limit(108, MIB)
    hb.note_array(108, a)
    hb.note_array(108, a)
    assert hb.covered(a.ctypes.data, 1)
    hb.test_registrar(0)
    assert not hb.covered(a.ctypes.data, 1) and hb.stats()["registered_bytes"] == 0
    hb.drop_owner(108)


def test_concurrent_frame_hosts(hb):
    """16 threads, each an owner cycling through its own pool of blocks:
    every block registers once, every release balances."""
    pools = [[np.zeros((k % 3 + 1) * 64 * 1024, np.uint8) for k in range(6)] for _ in range(16)]
    s0 = hb.stats()
    errors = []

    def host(t):
        try:
            owner = 200 + t
            hb.set_limit(owner, 64 * MIB)
            for _ in range(5):
                for blk in pools[t]:
                    hb.note_array(owner, blk)
                    hb.covered(blk.ctypes.data, blk.nbytes)
            for blk in pools[t][:3]:
                hb.release(blk.ctypes.data, blk.nbytes)
            hb.drop_owner(owner)
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(e)

    threads = [threading.Thread(target=host, args=(t,)) for t in range(16)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors
    d = _delta(hb, s0)
    assert d["registrations"] == 16 * 6 and d["released"] == 16 * 6
    assert hb.stats()["registered_bytes"] == 0


def test_invalid_arguments(gb):
    with pytest.raises(ValueError):
        gb.host_blocks.set_limit(1, -1)
    with pytest.raises(ValueError):
        gb.host_blocks.test_registrar(9)
