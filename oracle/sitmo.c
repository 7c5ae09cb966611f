/*
 * ORACLE (test infrastructure) — restatement of the sitmo counter-based engine of the
 * reference's lib/prng_engine.hpp (MIT, vendored there from sitmo.com).
 *
 * Block function (prng_engine.hpp:307-343): a 20-mix Threefish-256-style ARX cipher of the
 * 256-bit counter under the 256-bit key, with a key injection before every fourth mix and
 * a final key addition. The stream view (prng_engine.hpp:195-212): call k of operator()
 * returns 32-bit word k%8 of the block at counter k/8 (low half of out[j] before the high
 * half), so a u64 draw d of a stream is simply out[d%4] of block d/4.
 */
#include "oracle.h"

static uint64_t rotl64(uint64_t x, unsigned r) { return (x << r) | (x >> (64 - r)); }

/* rotation pairs for the four mixes of an even / odd injection group */
static const unsigned ROT[2][4][2] = {
    {{14, 16}, {52, 57}, {23, 40}, {5, 37}},
    {{25, 33}, {46, 12}, {58, 22}, {32, 32}},
};

void orc_sitmo_block(const uint64_t key[4], const uint64_t ctr[4], uint64_t out[4]) {
    uint64_t k[5];
    uint64_t b[4];
    for (int i = 0; i < 4; i++) { k[i] = key[i]; b[i] = ctr[i]; }
    k[4] = 0x1BD11BDAA9FC1A22ull ^ k[0] ^ k[1] ^ k[2] ^ k[3];

    for (int s = 0; s < 5; s++) {
        const unsigned (*rot)[2] = ROT[s & 1];
        for (int j = 0; j < 4; j++) {
            /* mixes alternate between pairing (b0,b1)(b2,b3) and (b0,b3)(b2,b1) */
            int x1 = (j & 1) ? 3 : 1, z1 = (j & 1) ? 1 : 3;
            if (j == 0) {
                /* key injection s: words k[s..s+3 mod 5], the last one plus s */
                b[1] += k[(s + 1) % 5];
                b[3] += k[(s + 3) % 5] + (uint64_t)s;
                b[0] += b[1] + k[s % 5];
                b[2] += b[3] + k[(s + 2) % 5];
            } else {
                b[0] += b[x1];
                b[2] += b[z1];
            }
            b[x1] = rotl64(b[x1], rot[j][0]);
            b[z1] = rotl64(b[z1], rot[j][1]);
            b[x1] ^= b[0];
            b[z1] ^= b[2];
        }
    }
    for (int i = 0; i < 4; i++) out[i] = b[i] + k[i];
    out[3] += 5;
}

/* 256-bit counter + z, with carry (prng_engine.hpp:345-371 generalised). */
static void ctr_add(const uint64_t c[4], uint64_t z, uint64_t r[4]) {
    r[0] = c[0] + z;
    uint64_t carry = r[0] < c[0];
    for (int i = 1; i < 4; i++) {
        r[i] = c[i] + carry;
        carry = carry && r[i] == 0;
    }
}

static uint32_t word32(const uint64_t out[4], unsigned idx) {
    uint64_t w = out[idx >> 1];
    return (idx & 1) ? (uint32_t)(w >> 32) : (uint32_t)w;
}

uint32_t orc_sitmo_seed_output(uint32_t seed, uint64_t k) {
    uint64_t key[4] = {seed, 0, 0, 0}, ctr[4] = {k >> 3, 0, 0, 0}, out[4];
    orc_sitmo_block(key, ctr, out);
    return word32(out, (unsigned)(k & 7));
}

void orc_sitmo_outputs(const uint64_t key[4], const uint64_t ctr[4], uint64_t count, uint32_t *dst) {
    uint64_t out[4], c[4];
    for (uint64_t k = 0; k < count; k++) {
        if ((k & 7) == 0) {
            ctr_add(ctr, k >> 3, c);
            orc_sitmo_block(key, c, out);
        }
        dst[k] = word32(out, (unsigned)(k & 7));
    }
}

uint64_t orc_draw64(const uint64_t key[4], uint64_t round, uint64_t d) {
    uint64_t ctr[4] = {d >> 2, round, 0, 0}, out[4];
    orc_sitmo_block(key, ctr, out);
    return out[d & 3];
}
