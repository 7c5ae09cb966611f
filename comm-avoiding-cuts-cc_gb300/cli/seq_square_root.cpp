// Drop-in for the reference's seq_square_root executable (src/executables/seq_square_root.cpp,
// SquareRootCut::seqMaster, SquareRootCut.cpp:308-): square_root on one process; same arguments
// (including the usage text) and CSV line
//   input,seed,1,n,m,cuttingTime,mpiTime,trials,low,weight
#include <iostream>
#include <string>

#include "cli_common.h"

int main(int argc, char *argv[]) {
    if (argc != 4) {
        std::cout << "Usage: square_root PROBABILITY INPUT_FILE SEED" << std::endl;
        return 1;
    }
    float success_probability{std::stof(argv[1], nullptr)};
    const uint32_t seed = {(uint32_t)std::stoi(argv[3])};
    cac_config cfg{cli_device(), nullptr, 0};
    cac_ctx *ctx = nullptr;
    int st = cac_ctx_create(&cfg, &ctx);
    if (st) return cli_fail("cac_ctx_create", st);
    cac_graph *g = nullptr;
    st = cac_graph_load_file(ctx, argv[2], &g);
    if (st) return cli_fail("cac_graph_load_file", st);
    uint32_t n = 0;
    uint64_t m = 0;
    cac_graph_info(g, &n, &m, nullptr);
    cac_mincut_result res{};
    st = cac_mincut(ctx, g, success_probability, seed, 1, &res);
    if (st) return cli_fail("cac_mincut", st);
    std::cout << std::fixed;
    std::cout << argv[2] << "," << seed << "," << 1 << "," << n << "," << m << "," << res.device_ms / 1000.0 << ","
              << 0.0 << "," << res.trials_per_rank << ",low," << res.cut << std::endl;
    cac_graph_free(g);
    cac_ctx_destroy(ctx);
    return 0;
}
