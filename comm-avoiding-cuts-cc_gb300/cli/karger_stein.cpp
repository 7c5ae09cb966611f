// Drop-in for the reference's karger_stein executable (src/executables/karger_stein.cpp): plain
// Karger-Stein (comincut::minimum_cut with success probability 0.90) on the whole input graph;
// same arguments and CSV line
//   input,seed,1,n,m,time,?,co-karger-stein,cut
#include <iostream>
#include <string>

#include "cli_common.h"

int main(int argc, char *argv[]) {
    if (argc != 3) {
        std::cout << "Usage: karger_stein INPUT_FILE SEED" << std::endl;
        return 1;
    }
    const uint32_t seed = {(uint32_t)std::stoi(argv[2])};
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
    cac_mincut_result res{};
    st = cac_karger_stein(ctx, g, 0.90, seed, &res);
    if (st) return cli_fail("cac_karger_stein", st);
    std::cout << argv[1] << "," << seed << "," << 1 << "," << n << "," << m << "," << res.device_ms / 1000.0 << ","
              << "?" << ","
              << "co-karger-stein," << res.cut << std::endl;
    cac_graph_free(g);
    cac_ctx_destroy(ctx);
    return 0;
}
