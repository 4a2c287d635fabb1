// chacha.cuh - the reference RNG stream on the device.
//
// src/rng.rs wraps rand 0.8.5's StdRng, which is ChaCha with 12 rounds
// (rand_chacha 0.3.1): 16-word state of the four constants, the 8-word key,
// a 64-bit block counter (words 12-13) and a zero 64-bit stream id (words
// 14-15); output words are the keystream words in order.  Because the
// keystream is a function of the block counter, a thread seeks directly to
// the first word of its pixel instead of replaying the task's stream.
// The key is expanded on the host from the task index (rand_core 0.6.4
// seed_from_u64, see host_scene.cpp).
#pragma once
#include <stdint.h>

namespace pbrt {

__device__ __forceinline__ uint32_t rotl32(uint32_t v, int c) { return __funnelshift_l(v, v, c); }

#define PBRT_QR(a, b, c, d) \
    a += b;                 \
    d ^= a;                 \
    d = rotl32(d, 16);      \
    c += d;                 \
    b ^= c;                 \
    b = rotl32(b, 12);      \
    a += b;                 \
    d ^= a;                 \
    d = rotl32(d, 8);       \
    c += d;                 \
    b ^= c;                 \
    b = rotl32(b, 7);

// out[k * stride] = keystream word k of block `ctr`.  DR double rounds (6:
// ChaCha12, StdRng's cipher) and stream id `sid` (0 for StdRng) are
// parameters only so that the same code can be checked against other
// ChaCha implementations (pbrtgpu_chacha_blocks); the sampler uses the
// defaults.
template <int DR = 6>
__device__ __forceinline__ void chacha12_block(const uint32_t* key, uint64_t ctr, uint32_t* out, uint32_t stride,
                                               uint64_t sid = 0) {
    const uint32_t s14 = (uint32_t)sid, s15 = (uint32_t)(sid >> 32);
    uint32_t x0 = 0x61707865u, x1 = 0x3320646eu, x2 = 0x79622d32u, x3 = 0x6b206574u;
    uint32_t x4 = key[0], x5 = key[1], x6 = key[2], x7 = key[3];
    uint32_t x8 = key[4], x9 = key[5], x10 = key[6], x11 = key[7];
    uint32_t x12 = (uint32_t)ctr, x13 = (uint32_t)(ctr >> 32), x14 = s14, x15 = s15;
#pragma unroll
    for (int r = 0; r < DR; ++r) {
        PBRT_QR(x0, x4, x8, x12);
        PBRT_QR(x1, x5, x9, x13);
        PBRT_QR(x2, x6, x10, x14);
        PBRT_QR(x3, x7, x11, x15);
        PBRT_QR(x0, x5, x10, x15);
        PBRT_QR(x1, x6, x11, x12);
        PBRT_QR(x2, x7, x8, x13);
        PBRT_QR(x3, x4, x9, x14);
    }
    out[0u * stride] = x0 + 0x61707865u;
    out[1u * stride] = x1 + 0x3320646eu;
    out[2u * stride] = x2 + 0x79622d32u;
    out[3u * stride] = x3 + 0x6b206574u;
    out[4u * stride] = x4 + key[0];
    out[5u * stride] = x5 + key[1];
    out[6u * stride] = x6 + key[2];
    out[7u * stride] = x7 + key[3];
    out[8u * stride] = x8 + key[4];
    out[9u * stride] = x9 + key[5];
    out[10u * stride] = x10 + key[6];
    out[11u * stride] = x11 + key[7];
    out[12u * stride] = x12 + (uint32_t)ctr;
    out[13u * stride] = x13 + (uint32_t)(ctr >> 32);
    out[14u * stride] = x14 + s14;
    out[15u * stride] = x15 + s15;
}
// Blocks ctr and ctr + 1 at once (two independent chains for the
// scheduler): word k of block ctr + j at out[(16 j + k) * stride].
template <int DR = 6>
__device__ __forceinline__ void chacha12_block2(const uint32_t* key, uint64_t ctr, uint32_t* out, uint32_t stride,
                                                uint64_t sid = 0) {
    const uint64_t c1 = ctr + 1;
    const uint32_t s14 = (uint32_t)sid, s15 = (uint32_t)(sid >> 32);
    uint32_t x0 = 0x61707865u, x1 = 0x3320646eu, x2 = 0x79622d32u, x3 = 0x6b206574u;
    uint32_t x4 = key[0], x5 = key[1], x6 = key[2], x7 = key[3];
    uint32_t x8 = key[4], x9 = key[5], x10 = key[6], x11 = key[7];
    uint32_t x12 = (uint32_t)ctr, x13 = (uint32_t)(ctr >> 32), x14 = s14, x15 = s15;
    uint32_t y0 = 0x61707865u, y1 = 0x3320646eu, y2 = 0x79622d32u, y3 = 0x6b206574u;
    uint32_t y4 = key[0], y5 = key[1], y6 = key[2], y7 = key[3];
    uint32_t y8 = key[4], y9 = key[5], y10 = key[6], y11 = key[7];
    uint32_t y12 = (uint32_t)c1, y13 = (uint32_t)(c1 >> 32), y14 = s14, y15 = s15;
#pragma unroll
    for (int r = 0; r < DR; ++r) {
        PBRT_QR(x0, x4, x8, x12);
        PBRT_QR(y0, y4, y8, y12);
        PBRT_QR(x1, x5, x9, x13);
        PBRT_QR(y1, y5, y9, y13);
        PBRT_QR(x2, x6, x10, x14);
        PBRT_QR(y2, y6, y10, y14);
        PBRT_QR(x3, x7, x11, x15);
        PBRT_QR(y3, y7, y11, y15);
        PBRT_QR(x0, x5, x10, x15);
        PBRT_QR(y0, y5, y10, y15);
        PBRT_QR(x1, x6, x11, x12);
        PBRT_QR(y1, y6, y11, y12);
        PBRT_QR(x2, x7, x8, x13);
        PBRT_QR(y2, y7, y8, y13);
        PBRT_QR(x3, x4, x9, x14);
        PBRT_QR(y3, y4, y9, y14);
    }
    const uint32_t xs[16] = {x0 + 0x61707865u, x1 + 0x3320646eu, x2 + 0x79622d32u, x3 + 0x6b206574u,
                             x4 + key[0],      x5 + key[1],      x6 + key[2],      x7 + key[3],
                             x8 + key[4],      x9 + key[5],      x10 + key[6],     x11 + key[7],
                             x12 + (uint32_t)ctr, x13 + (uint32_t)(ctr >> 32), x14 + s14, x15 + s15};
    const uint32_t ys[16] = {y0 + 0x61707865u, y1 + 0x3320646eu, y2 + 0x79622d32u, y3 + 0x6b206574u,
                             y4 + key[0],      y5 + key[1],      y6 + key[2],      y7 + key[3],
                             y8 + key[4],      y9 + key[5],      y10 + key[6],     y11 + key[7],
                             y12 + (uint32_t)c1, y13 + (uint32_t)(c1 >> 32), y14 + s14, y15 + s15};
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        out[(uint32_t)k * stride] = xs[k];
        out[(uint32_t)(16 + k) * stride] = ys[k];
    }
}
#undef PBRT_QR

// The one copy of the pair computation in a kernel (each inlined read site
// would otherwise carry its own ~1200 instructions); the key goes by value
// so that it stays in registers.
static __device__ __noinline__ void chacha12_fill2(uint32_t k0, uint32_t k1, uint32_t k2, uint32_t k3, uint32_t k4,
                                                   uint32_t k5, uint32_t k6, uint32_t k7, uint64_t ctr,
                                                   uint32_t* out, uint32_t stride) {
    const uint32_t key[8] = {k0, k1, k2, k3, k4, k5, k6, k7};
    chacha12_block2(key, ctr, out, stride);
}
// The last block of a reader's range alone (the pair's second block would
// belong to the next reader): 0.473 -> 0.455 ms for 1024^2 x 16 samples.
static __device__ __noinline__ void chacha12_fill1(uint32_t k0, uint32_t k1, uint32_t k2, uint32_t k3, uint32_t k4,
                                                   uint32_t k5, uint32_t k6, uint32_t k7, uint64_t ctr,
                                                   uint32_t* out, uint32_t stride) {
    const uint32_t key[8] = {k0, k1, k2, k3, k4, k5, k6, k7};
    chacha12_block(key, ctr, out, stride);
}

// A seekable reader of one task's word stream.  Blocks are computed in
// pairs (two independent chains keep the scheduler busy) when a word of
// them is read, so words skipped over (whole pairs of blocks) cost nothing;
// the last block of the reader's range [word, end_word) is computed alone.
// The current pair lives in the caller's shared-memory column of 32 words
// (word k at buf[k * stride]): a per-thread array would go to local memory,
// whose loads and stores throttle the generate kernels.
struct WordStream {
    uint32_t key[8];
    uint64_t block;   // block of the next word
    uint64_t loaded;  // first block held in buf (~1: none, so block - loaded >= span)
    uint64_t end;     // first block past the reader's words
    uint32_t span;    // blocks held in buf: 2, or 1 for the range's last block
    uint32_t* buf;
    uint32_t stride;
    int idx;          // next word inside `block` (16: the block is used up)

    __device__ void seek(const uint32_t* k, uint64_t word, uint64_t end_word, uint32_t* column,
                         uint32_t column_stride) {
        end = (end_word + 15) >> 4;
        span = 2;
#pragma unroll
        for (int i = 0; i < 8; ++i) key[i] = k[i];
        block = word >> 4;
        idx = (int)(word & 15);
        loaded = ~1ull;
        buf = column;
        stride = column_stride;
    }
    // Moves n words ahead without reading them.
    __device__ __forceinline__ void skip(uint32_t n) {
        const uint64_t pos = block * 16u + (uint64_t)idx + n;
        block = pos >> 4;
        idx = (int)(pos & 15u);
    }
    __device__ __forceinline__ uint32_t next_u32() {
        if (idx == 16) {
            ++block;
            idx = 0;
        }
        if (block - loaded >= span) {  // not among the blocks held (also when none is)
            span = block + 1 < end ? 2u : 1u;
            if (span == 2u)
                chacha12_fill2(key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7], block, buf, stride);
            else
                chacha12_fill1(key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7], block, buf, stride);
            loaded = block;
        }
        return buf[((uint32_t)(block - loaded) * 16u + (uint32_t)idx++) * stride];
    }
    __device__ __forceinline__ uint64_t next_u64() {  // low word first
        uint64_t lo = next_u32();
        uint64_t hi = next_u32();
        return lo | (hi << 32);
    }
    // rng.rs:15-17 - gen::<f32>(): (u32 >> 8) * 2^-24
    __device__ __forceinline__ float random_float() { return (float)(next_u32() >> 8) * (1.0f / 16777216.0f); }
    // rng.rs:19-21
    __device__ __forceinline__ uint64_t random_uint() {
        uint64_t v = next_u64();
        return v == 0xFFFFFFFFFFFFFFFFull ? 0ull : v;  // v % usize::MAX
    }
};

}  // namespace pbrt
