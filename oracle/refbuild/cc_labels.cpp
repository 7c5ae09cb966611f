// Runs the reference's UnweightedIteratedSparseSampling::connectedComponents
// (src/UnweightedIteratedSparseSampling.cpp:40-72) on one rank and prints the component
// count followed by every vertex's label. Test infrastructure only.
//   cc_labels INPUT_FILE SEED
#include <cstdio>
#include <vector>
#include <string>
#include "UnweightedIteratedSparseSampling.hpp"

int main(int argc, char **argv) {
    if (argc != 3) { std::fprintf(stderr, "usage: cc_labels INPUT_FILE SEED\n"); return 1; }
    MPI_Init(&argc, &argv);
    GraphInputIterator input(argv[1]);
    uint32_t seed = (uint32_t)std::stoul(argv[2]);
    UnweightedIteratedSparseSampling sampler(MPI_COMM_WORLD, 0, 1, seed, 1, input.vertexCount(), input.edgeCount());
    sampler.loadSlice(input);
    std::vector<unsigned> labels;
    unsigned count = sampler.connectedComponents(labels);
    std::printf("%u %zu\n", count, labels.size());
    for (size_t i = 0; i < labels.size(); i++) std::printf("%u\n", labels[i]);
    MPI_Finalize();
    return 0;
}
