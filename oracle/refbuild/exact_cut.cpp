// Exact minimum cut with the reference's deterministic Stoer-Wagner path
// (comincut::deterministic_minimum_cut, src/karger-stein/co_mincut.h:529-541), input in the
// reference's edge-list format. Test infrastructure only.
//   exact_cut INPUT_FILE
#include <cstdio>
#include "input/GraphInputIterator.hpp"
#include "sparse_graph.hpp"
#include "stack_allocator.h"
#include "co_mincut.h"

int main(int argc, char **argv) {
    if (argc != 2) { std::fprintf(stderr, "usage: exact_cut INPUT_FILE\n"); return 1; }
    GraphInputIterator input(argv[1]);
    stack_allocator allocator(sizeof(edge<unsigned long>) * input.edgeCount());
    array<edge<unsigned long>> ks_edges = allocator.allocate<edge<unsigned long>>(input.edgeCount());
    GraphInputIterator::Iterator it = input.begin();
    for (unsigned i = 0; i < input.edgeCount(); i++) {
        edge<unsigned long> e;
        e.set_vertices(it->from, it->to);
        e.weight = it->weight;
        ks_edges[i] = e;
        ++it;
    }
    sparse_graph<unsigned long, edge<unsigned long>> g(input.vertexCount(), ks_edges);
    unsigned long cut = comincut::deterministic_minimum_cut(&g);
    std::printf("%lu\n", cut);
    return 0;
}
