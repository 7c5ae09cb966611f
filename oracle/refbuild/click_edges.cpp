// Harness (test infrastructure): prints the CLICK graph that the reference's approx_cut builds
// on P ranks -- rank r calls CLICK::generateSlice (src/input/CLICK.hpp:10-49) with seed + r
// (ApproximateCut.hpp:35, :70-82) -- as "n m" then one "u v w" line per edge, slices in rank order.
//   click_edges N P SEED
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "CLICK.hpp"

int main(int argc, char **argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: click_edges N P SEED\n");
        return 1;
    }
    const unsigned n = (unsigned)std::strtoul(argv[1], nullptr, 10);
    const unsigned p = (unsigned)std::strtoul(argv[2], nullptr, 10);
    const uint32_t seed = (uint32_t)std::strtoul(argv[3], nullptr, 10);
    const unsigned edges = n * (n - 1) / 2;
    std::vector<AdjacencyListGraph::Edge> all;
    for (unsigned r = 0; r < p; r++) {
        std::vector<AdjacencyListGraph::Edge> slice;
        CLICK::generateSlice(slice, edges, p, (int)r, (int32_t)(seed + r), n);
        all.insert(all.end(), slice.begin(), slice.end());
    }
    std::printf("%u %zu\n", n, all.size());
    for (const auto &e : all) std::printf("%u %u %llu\n", e.from, e.to, (unsigned long long)e.weight);
    return 0;
}
