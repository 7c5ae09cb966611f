// Known-answer dump of the draws approx_cut makes: std::binomial_distribution<int>(w, 2^-level)
// on the reference's sitmo engine, constructed per draw as in ApproximateCut::run
// (src/ApproximateCut.cpp:33-48). Test infrastructure only.
//
//   binom_stream SEED LEVEL COUNT W1 [W2 ...]      (draw k uses weight W[k mod #W])
//
// Output: the COUNT draws, ':', then the engine's next raw 32-bit output, which shows how many
// outputs the draws consumed.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "prng_engine.hpp"

int main(int argc, char **argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: binom_stream SEED LEVEL COUNT W1 [W2 ...]\n");
        return 1;
    }
    const uint32_t seed = (uint32_t)std::strtoul(argv[1], nullptr, 10);
    const int level = std::atoi(argv[2]);
    const long count = std::atol(argv[3]);
    std::vector<unsigned long> w;
    for (int i = 4; i < argc; i++) w.push_back(std::strtoul(argv[i], nullptr, 10));
    sitmo::prng_engine engine(seed);
    const double p = std::pow(2, -level);
    for (long k = 0; k < count; k++) {
        std::binomial_distribution<int> d(w[k % w.size()], p);
        std::printf("%d ", d(engine));
    }
    std::printf(": %u\n", (unsigned)engine());
    return 0;
}
