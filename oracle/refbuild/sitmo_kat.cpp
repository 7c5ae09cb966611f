// Known-answer dump of the reference's sitmo engine (lib/prng_engine.hpp), used to pin
// the oracle's and the device's sitmo restatements. Test infrastructure only.
// Output: one line per case, "case <name> <k0> <k1> <k2> <k3> <c0> <c1> <c2> <c3> : v0 v1 ...",
// where v_i are consecutive 32-bit outputs of operator().
#include <cstdio>
#include <cstdint>
#include "prng_engine.hpp"

static void dump(const char *name, sitmo::prng_engine &e, const uint64_t k[4], const uint64_t c[4], int count) {
    std::printf("case %s %llu %llu %llu %llu %llu %llu %llu %llu :", name,
                (unsigned long long)k[0], (unsigned long long)k[1], (unsigned long long)k[2], (unsigned long long)k[3],
                (unsigned long long)c[0], (unsigned long long)c[1], (unsigned long long)c[2], (unsigned long long)c[3]);
    for (int i = 0; i < count; i++) std::printf(" %u", (unsigned)e());
    std::printf("\n");
}

int main() {
    const uint32_t seeds[] = {0u, 1u, 2u, 3u, 42u, 5226u, 123456789u, 4294967295u};
    for (uint32_t s : seeds) {
        sitmo::prng_engine e(s);
        uint64_t k[4] = {s, 0, 0, 0}, c[4] = {0, 0, 0, 0};
        dump("seed", e, k, c, 40);
    }
    const uint64_t keys[][4] = {
        {0, 0, 0, 0}, {7, 3, 0x100000002ull, 0}, {0xdeadbeefull, 12, 5, 9}, {1, 0xffffffffffffffffull, 0, 1}};
    const uint64_t ctrs[][4] = {
        {0, 0, 0, 0}, {5, 0, 0, 0}, {0xfffffffffffffffeull, 0, 0, 0}, {123, 7, 0, 0},
        {0xffffffffffffffffull, 0xffffffffffffffffull, 3, 0}};
    for (auto &k : keys) {
        for (auto &c : ctrs) {
            sitmo::prng_engine e;
            e.set_key(k[0], k[1], k[2], k[3]);
            e.set_counter(c[0], c[1], c[2], c[3], 0);
            dump("keyctr", e, k, c, 24);
        }
    }
    return 0;
}
