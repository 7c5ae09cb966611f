// Drop-in for the reference's parallel_cc executable (src/executables/parallel_cc.cpp:6-64):
// same arguments, one CSV line per iteration
//   input,seed,p,n,m,time,mpi,cc,components
// As in the reference, every iteration replays the same random stream (the sampler is copied
// from one seeded with seed + rank) while the printed seed increments.
#include <iostream>
#include <string>

#include "cli_common.h"

int main(int argc, char *argv[]) {
    if ((argc != 3) && (argc != 4)) {
        std::cout << "Usage: connected_components INPUT_FILE SEED [ITERATONS]" << std::endl;
        return 1;
    }
    uint32_t seed = {(uint32_t)std::stoi(argv[2])};
    int iterations = argc == 4 ? std::stoi(argv[3]) : 1;
    const unsigned ranks = cli_virtual_ranks();
    cac_config cfg{cli_device(), nullptr, 0};
    cac_ctx *ctx = nullptr;
    int st = cac_ctx_create(&cfg, &ctx);
    if (st) return cli_fail("cac_ctx_create", st);
    cac_graph *g = nullptr;
    st = cac_graph_load_file(ctx, argv[1], &g);
    if (st) return cli_fail("cac_graph_load_file", st);
    uint32_t n = 0;
    uint64_t m = 0;
    cac_graph_info(g, &n, &m, nullptr);
    const uint32_t stream_seed = seed;
    for (int i = 0; i < iterations; i++) {
        cac_cc_result res{};
        st = cac_cc(ctx, g, stream_seed, ranks, nullptr, CAC_HOST, &res);
        if (st) return cli_fail("cac_cc", st);
        std::cout << std::fixed;
        std::cout << argv[1] << "," << seed << "," << ranks << "," << n << "," << m << "," << res.device_ms / 1000.0
                  << "," << 0.0 << "," << "cc" << "," << res.num_components << std::endl;
        seed++;
    }
    cac_graph_free(g);
    cac_ctx_destroy(ctx);
    return 0;
}
