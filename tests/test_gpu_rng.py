"""The device's ChaCha code (chacha.cuh) through the C ABI: its block
routines at 20 rounds against OpenSSL's ChaCha20 keystream
(tests/golden/chacha20_openssl.npz), at 12 and 8 rounds against the oracle
(including counters whose low word carries), and the seekable word reader
the render kernels use against the oracle's sequential RNG::new(seed)
stream (src/rng.rs:11-21)."""
import numpy as np
import pytest

from test_rng_pin import golden_cases, oracle_blocks, ptr

pytestmark = pytest.mark.gpu


def device_blocks(lib, key, ctr, sid, rounds, n, paired):
    out = np.full((n, 16), 0xDEADBEEF, np.uint32)
    st = lib.pbrtgpu_chacha_blocks(ptr(key), ctr, sid, rounds, 1 if paired else 0, n, ptr(out))
    assert st == 0, lib.pbrtgpu_last_error()
    return out


def test_device_block_routines_at_20_rounds_match_openssl(lib):
    for key, ctr, sid, n, want in golden_cases():
        assert np.array_equal(device_blocks(lib, key, ctr, sid, 20, n, False), want), (ctr, sid)
        if n % 2 == 0:
            assert np.array_equal(device_blocks(lib, key, ctr, sid, 20, n, True), want), (ctr, sid)


def test_device_blocks_match_the_oracle_at_12_and_8_rounds(lib, oracle):
    olib = oracle.load()
    from pbrt_rust_gb300.generators import PCG32
    rng = PCG32(31)
    for ctr in (0, 5, 0xFFFFFFFE, (1 << 32) - 1, (7 << 32) + 3, (1 << 64) - 4):
        key = rng.uint32(8)
        sid = int(rng.uint32(1)[0]) if ctr & 1 else 0
        for rounds in (12, 8):
            want = oracle_blocks(olib, key, ctr, sid, rounds, 4)
            assert np.array_equal(device_blocks(lib, key, ctr, sid, rounds, 4, False), want), (ctr, rounds)
            assert np.array_equal(device_blocks(lib, key, ctr, sid, rounds, 4, True), want), (ctr, rounds)


@pytest.mark.parametrize("segment", [1, 5, 16, 17, 37, 64, 1000])
def test_seekable_reader_matches_the_sequential_stream(lib, oracle, segment):
    olib = oracle.load()
    for seed, first in ((0, 0), (3, 15), (77, 1 << 20), (12345, (1 << 36) + 9)):
        n = 3000
        want = np.zeros(n, np.uint32)
        olib.oracle_rng_words(seed, first, n, ptr(want))
        got = np.zeros(n, np.uint32)
        assert lib.pbrtgpu_rng_words(seed, first, n, segment, ptr(got)) == 0, lib.pbrtgpu_last_error()
        assert np.array_equal(got, want), (seed, first, segment)
