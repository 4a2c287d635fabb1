"""Writes tests/golden/chacha20_openssl.npz: ChaCha20 keystream blocks from
an implementation independent of this repository - OpenSSL's, reached
through the ``cryptography`` package - for pinning the block function that
the sampler's random stream is built on.

    python tests/golden/make_chacha_vectors.py

The reference's RNG (src/rng.rs:4-21) is rand 0.8.5's StdRng, which is the
ChaCha block function with 12 rounds (rand_chacha 0.3.1) over the state
constants | 256-bit key | 64-bit block counter (words 12-13) | 64-bit stream
id (words 14-15).  No ChaCha12 implementation outside this repository is
available here, but OpenSSL's ChaCha20 is the same block function with 20
rounds over the same state: its 16-byte IV is state words 12-15
little-endian, word 12 being the block counter it increments.  So every
case below fixes words 12-15 through the IV and records the keystream of a
few consecutive blocks (the low counter word never wraps inside a case, which
OpenSSL refuses).  The oracle and the device compute the same blocks with
their round count set to 20 (tests/test_rng_pin.py, tests/test_gpu_rng.py);
their 12-round blocks then differ from these only in the loop bound.

Cases: key, counter (words 12-13 as one u64), stream id (words 14-15),
number of blocks; the keys are drawn from a fixed PCG32 stream.
"""
from __future__ import annotations

import struct
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))


def cases():
    from pbrt_rust_gb300.generators import PCG32
    rng = PCG32(0xC4AC4A)
    out = []
    specs = [(0, 0, 4), (1, 0, 2), (7, 0, 3), (0xFFFFFFF0, 0, 8), ((5 << 32) | 11, 0, 2), (3, 0x0123456789ABCDEF, 2),
             (0, (1 << 63) | 1, 2), ((0xDEADBEEF << 32) | 0x1234, 0xFFFFFFFFFFFFFFFF, 4)]
    for k, (ctr, sid, n) in enumerate(specs):
        key = np.zeros(8, np.uint32) if k == 0 else rng.uint32(8)
        out.append((key, ctr, sid, n))
    return out


def openssl_blocks(key: np.ndarray, ctr: int, sid: int, n: int) -> np.ndarray:
    from cryptography.hazmat.primitives.ciphers import Cipher, algorithms
    assert (ctr & 0xFFFFFFFF) + n <= 1 << 32, "OpenSSL does not carry the low counter word"
    iv = struct.pack("<IIII", ctr & 0xFFFFFFFF, ctr >> 32, sid & 0xFFFFFFFF, sid >> 32)
    ks = Cipher(algorithms.ChaCha20(key.astype("<u4").tobytes(), iv), mode=None).encryptor().update(bytes(64 * n))
    return np.frombuffer(ks, dtype="<u4").astype(np.uint32).reshape(n, 16)


def main() -> None:
    cs = cases()
    keys = np.stack([c[0] for c in cs])
    meta = np.array([[c[1], c[2], c[3]] for c in cs], dtype=np.uint64)
    blocks = np.concatenate([openssl_blocks(*c).reshape(-1) for c in cs])
    np.savez_compressed(HERE / "chacha20_openssl.npz", keys=keys, meta=meta, blocks=blocks)
    print(f"wrote {len(cs)} cases, {blocks.size // 16} blocks")


if __name__ == "__main__":
    main()
