"""Host side of the batch API, without a GPU: memory planning, argument
checks and the refusal to run without a device."""
import ctypes as C

import pytest

from pbrt_rust_gb300 import abi
from pbrt_rust_gb300.batch import batch_bytes, limits


def test_batch_bytes_grow_with_the_limits(lib):
    d0, h0 = batch_bytes(max_jobs=8, max_samples=1 << 16)
    d1, h1 = batch_bytes(max_jobs=8, max_samples=1 << 18)
    d2, h2 = batch_bytes(max_jobs=64, max_samples=1 << 18)
    assert d1 > d0 and h1 == h0 and h2 > h1
    # per sample at least rays, hits, film positions, Le and L (88 B); per
    # light sample light samples, contributions, occlusion and the queue
    assert d1 - d0 >= 88 * ((1 << 18) - (1 << 16))


def test_batch_limits_are_checked(lib):
    d = C.c_uint64()
    bad = limits(max_jobs=0)
    assert lib.pbrtgpu_batch_bytes(C.byref(bad), C.byref(d), None) == 1
    assert lib.pbrtgpu_batch_bytes(C.byref(limits(max_samples=1 << 31)), C.byref(d), None) == 1
    assert b"2^31" in lib.pbrtgpu_last_error()


def test_batch_needs_a_device(lib):
    from conftest import HAS_GPU
    if HAS_GPU:
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert lib.pbrtgpu_batch_create(C.byref(limits()), C.byref(h)) == 10  # PBRT_ERR_NO_DEVICE
    assert not h.value


def test_server_pool_must_hold_its_slots(lib):
    """A server's device-memory pool is charged its slots' arenas at creation
    (before any device work): a pool smaller than them is refused."""
    per_slot, _ = batch_bytes(max_jobs=8, max_samples=1 << 16)
    cfg = abi.PbrtServerConfig()
    cfg.slots = 2
    cfg.limits = limits(max_jobs=8, max_samples=1 << 16)
    cfg.pool_bytes = 2 * per_slot - 1
    h = C.c_void_p()
    assert lib.pbrtgpu_server_create(C.byref(cfg), C.byref(h)) == 7  # PBRT_ERR_BUDGET
    assert b"exceed the pool" in lib.pbrtgpu_last_error()
    assert not h.value
