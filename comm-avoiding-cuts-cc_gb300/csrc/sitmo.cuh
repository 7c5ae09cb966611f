// Device (and host) restatement of the sitmo counter-based engine of the reference
// (lib/prng_engine.hpp:307-343): a 20-mix Threefish-256-style ARX cipher of a 256-bit counter
// under a 256-bit key. Being counter-based, any draw of any stream is computed directly from
// (key, counter) with no sequential state, which is what lets every trial, node and sample of
// the GPU path address its own random numbers and replay identically on the host.
//
// Stream view used throughout libcac: u64 draw d of round `rnd` of the stream with key K is
// word d % 4 of the block at counter (d / 4, rnd, 0, 0). The reference's 32-bit outputs of
// sitmo::prng_engine(seed) are the low / high halves of the same words (output k is word
// (k % 8) / 2 of block k / 8, low half first), so stream (seed, 0, 0, 0) at round 0 is exactly
// the reference engine's stream.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define CAC_HD __host__ __device__ __forceinline__
#else
#define CAC_HD inline
#endif

namespace cac {

struct u64x4 {
    uint64_t x[4];
};

CAC_HD uint64_t rotl64(uint64_t v, unsigned r) { return (v << r) | (v >> (64u - r)); }

// One mix of the pairs (b0, b[x1]) and (b2, b[z1]) with rotations rx, rz.
#define CAC_SITMO_MIX(X1, Z1, RX, RZ) \
    b0 += X1;                          \
    b2 += Z1;                          \
    X1 = rotl64(X1, RX);               \
    Z1 = rotl64(Z1, RZ);               \
    X1 ^= b0;                          \
    Z1 ^= b2;

// Mix with key injection: k-words (ka, kb, kc, kd) added as in the reference's MIXK.
#define CAC_SITMO_MIXK(RX, RZ, KA, KB, KC, KD) \
    b1 += KB;                                 \
    b3 += KD;                                 \
    b0 += b1 + KA;                            \
    b2 += b3 + KC;                            \
    b1 = rotl64(b1, RX);                      \
    b3 = rotl64(b3, RZ);                      \
    b1 ^= b0;                                 \
    b3 ^= b2;

CAC_HD u64x4 sitmo_block(uint64_t k0, uint64_t k1, uint64_t k2, uint64_t k3, uint64_t c0, uint64_t c1,
                         uint64_t c2, uint64_t c3) {
    const uint64_t k4 = 0x1BD11BDAA9FC1A22ull ^ k0 ^ k1 ^ k2 ^ k3;
    uint64_t b0 = c0, b1 = c1, b2 = c2, b3 = c3;
    // group 0
    CAC_SITMO_MIXK(14, 16, k0, k1, k2, k3)
    CAC_SITMO_MIX(b3, b1, 52, 57)
    CAC_SITMO_MIX(b1, b3, 23, 40)
    CAC_SITMO_MIX(b3, b1, 5, 37)
    // group 1
    CAC_SITMO_MIXK(25, 33, k1, k2, k3, k4 + 1)
    CAC_SITMO_MIX(b3, b1, 46, 12)
    CAC_SITMO_MIX(b1, b3, 58, 22)
    CAC_SITMO_MIX(b3, b1, 32, 32)
    // group 2
    CAC_SITMO_MIXK(14, 16, k2, k3, k4, k0 + 2)
    CAC_SITMO_MIX(b3, b1, 52, 57)
    CAC_SITMO_MIX(b1, b3, 23, 40)
    CAC_SITMO_MIX(b3, b1, 5, 37)
    // group 3
    CAC_SITMO_MIXK(25, 33, k3, k4, k0, k1 + 3)
    CAC_SITMO_MIX(b3, b1, 46, 12)
    CAC_SITMO_MIX(b1, b3, 58, 22)
    CAC_SITMO_MIX(b3, b1, 32, 32)
    // group 4
    CAC_SITMO_MIXK(14, 16, k4, k0, k1, k2 + 4)
    CAC_SITMO_MIX(b3, b1, 52, 57)
    CAC_SITMO_MIX(b1, b3, 23, 40)
    CAC_SITMO_MIX(b3, b1, 5, 37)
    u64x4 o;
    o.x[0] = b0 + k0;
    o.x[1] = b1 + k1;
    o.x[2] = b2 + k2;
    o.x[3] = b3 + k3 + 5;
    return o;
}

#undef CAC_SITMO_MIX
#undef CAC_SITMO_MIXK

// 64x64 -> high 64 bits of the 128-bit product.
CAC_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// u64 draw d of round rnd of stream (k0..k3).
CAC_HD uint64_t draw64(uint64_t k0, uint64_t k1, uint64_t k2, uint64_t k3, uint64_t rnd, uint64_t d) {
    u64x4 o = sitmo_block(k0, k1, k2, k3, d >> 2, rnd, 0, 0);
    unsigned j = (unsigned)(d & 3);
    return j == 0 ? o.x[0] : j == 1 ? o.x[1] : j == 2 ? o.x[2] : o.x[3];
}

}  // namespace cac
