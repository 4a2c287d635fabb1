"""The sampler's random stream pinned against an independent implementation.

The reference's RNG (src/rng.rs:4-21) is rand 0.8.5's StdRng: the ChaCha
block function with 12 rounds (rand_chacha 0.3.1) over constants | key |
64-bit block counter | 64-bit stream id, the key expanded from the task
index by rand_core 0.6.4's seed_from_u64.  tests/golden/chacha20_openssl.npz
holds ChaCha20 keystream blocks computed by OpenSSL (through the
`cryptography` package; tests/golden/make_chacha_vectors.py): the same block
function and state layout at 20 rounds.  The oracle's block function with
its round count set to 20 must reproduce them word for word, which pins the
constants, the key, counter and stream-id words, the quarter round, the
column/diagonal order and the final addition; StdRng's blocks differ from
those only in the number of double rounds.  What stays unpinned against the
Rust crates: the seed_from_u64 expansion of the task index into the key, the
12-round count itself, the carry of the low counter word into the high one,
and next_u64's word order (low word first).
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden" / "chacha20_openssl.npz"


def ptr(a):
    return C.c_void_p(a.ctypes.data)


def golden_cases():
    d = np.load(GOLD)
    keys, meta, blocks = d["keys"], d["meta"], d["blocks"]
    out, off = [], 0
    for key, (ctr, sid, n) in zip(keys, meta):
        n = int(n)
        out.append((np.ascontiguousarray(key, np.uint32), int(ctr), int(sid), n,
                    blocks[off:off + 16 * n].reshape(n, 16)))
        off += 16 * n
    assert off == blocks.size
    return out


def oracle_blocks(lib, key, ctr, sid, rounds, n):
    out = np.zeros((n, 16), np.uint32)
    lib.oracle_chacha_blocks(ptr(key), ctr, sid, rounds, n, ptr(out))
    return out


def test_fixture_is_what_openssl_computes():
    pytest.importorskip("cryptography")
    import importlib.util
    spec = importlib.util.spec_from_file_location("mcv", GOLD.parent / "make_chacha_vectors.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    for key, ctr, sid, n, want in golden_cases():
        assert np.array_equal(m.openssl_blocks(key, ctr, sid, n), want)


def test_oracle_block_function_at_20_rounds_matches_openssl(oracle):
    lib = oracle.load()
    cases = golden_cases()
    assert len(cases) >= 8
    for key, ctr, sid, n, want in cases:
        assert np.array_equal(oracle_blocks(lib, key, ctr, sid, 20, n), want), (ctr, sid)


def test_stdrng_stream_is_the_12_round_keystream_of_the_seed_key(oracle):
    """RNG::new(seed)'s u32 words are the ChaCha12 keystream words of the
    seed's key, stream 0, blocks 0, 1, 2, ... in order."""
    lib = oracle.load()
    for seed in (0, 1, 7, 123456789, (1 << 64) - 1):
        key = np.zeros(8, np.uint32)
        lib.oracle_rng_key(seed, ptr(key))
        words = np.zeros(16 * 5, np.uint32)
        lib.oracle_rng_words(seed, 0, words.size, ptr(words))
        assert np.array_equal(words, oracle_blocks(lib, key, 0, 0, 12, 5).reshape(-1))
        # 12 rounds is not 20: the round count matters
        assert not np.array_equal(words[:16], oracle_blocks(lib, key, 0, 0, 20, 1).reshape(-1))


def test_rng_entry_points_reject_bad_arguments(lib):
    """Argument checks come before any device work (the values themselves
    are checked on the device in tests/test_gpu_rng.py)."""
    assert lib.pbrtgpu_rng_words(1, 0, 16, 0, None) == 1  # segment 0
    assert lib.pbrtgpu_chacha_blocks(None, 0, 0, 12, 0, 1, None) == 1
    k = np.zeros(8, np.uint32)
    assert lib.pbrtgpu_chacha_blocks(ptr(k), 0, 0, 13, 0, 1, ptr(np.zeros(16, np.uint32))) == 1
    assert lib.pbrtgpu_chacha_blocks(ptr(k), 0, 0, 12, 1, 3, ptr(np.zeros(48, np.uint32))) == 1
