// Drop-in for the reference's approx_cut executable (src/executables/approx_cut.cpp:5-43):
// same arguments, same CSV line
//   input,seed,p,n,m,cuttingTime,mpiTime,trials,weight
// On unit-weight graphs the draws are the reference's own (seed replay), so the line carries the
// reference's weight and trials for the same file, seed and CAC_VIRTUAL_RANKS.
#include <iostream>
#include <string>

#include "cli_common.h"

int main(int argc, char *argv[]) {
    if ((argc != 4) && (argc != 5)) {
        std::cout << "Usage: slimGraph-Light PROBABILITY INPUT_FILE|CLICK [SIZE] SEED" << std::endl;
        return 1;
    }
    float success_probability{std::stof(argv[1], nullptr)};
    uint32_t seed = {(uint32_t)std::stoi(argv[argc == 4 ? 3 : 4])};
    const unsigned ranks = cli_virtual_ranks();
    cac_config cfg{cli_device(), nullptr, 0};
    cac_ctx *ctx = nullptr;
    int st = cac_ctx_create(&cfg, &ctx);
    if (st) return cli_fail("cac_ctx_create", st);
    cac_graph *g = nullptr;
    uint32_t n = 0;
    uint64_t m = 0;
    if (std::string(argv[2]) == "CLICK") {
        // the in-memory complete graph of the reference (CLICK::generateSlice on every rank); like
        // the reference, the CSV line reports its n (n - 1) / 2 enumerated edges
        n = (uint32_t)std::stoul(argv[3]);
        st = cac_graph_click(ctx, n, ranks, seed, &g);
        if (st) return cli_fail("cac_graph_click", st);
        m = (uint64_t)n * (n - 1) / 2;
    } else {
        st = cac_graph_load_file(ctx, argv[2], &g);
        if (st) return cli_fail("cac_graph_load_file", st);
        cac_graph_info(g, &n, &m, nullptr);
    }
    // The reference's own draws where the graph allows them (unit weights), so the line equals the
    // reference's; weighted graphs take the counter-addressed keep test unless CAC_SEED_REPLAY=1
    // demands the replay (then they fail).
    const int replay = cli_seed_replay();
    cac_approx_result res{};
    st = CAC_ERR_UNSUPPORTED;
    if (replay != 0) {
        st = cac_approx_cut_seed_replay(ctx, g, success_probability, seed, ranks, &res);
        if (st && (replay == 1 || st != CAC_ERR_UNSUPPORTED)) return cli_fail("cac_approx_cut_seed_replay", st);
    }
    if (st) {
        st = cac_approx_cut(ctx, g, success_probability, seed, ranks, &res);
        if (st) return cli_fail("cac_approx_cut", st);
    }
    std::cout << std::fixed;
    std::cout << argv[2] << "," << seed << "," << ranks << "," << n << "," << m << "," << res.device_ms / 1000.0
              << "," << 0.0 << "," << res.trials << "," << res.cut << std::endl;
    cac_graph_free(g);
    cac_ctx_destroy(ctx);
    return 0;
}
