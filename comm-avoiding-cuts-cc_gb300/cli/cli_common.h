// Shared helpers of the drop-in command lines.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <string>

#include "cac.h"

// The MPI rank count the reference would have been launched with (`mpiexec -n P`): it fixes the
// seed layout (rank r uses seed + r) and the trial split, and is printed in the CSV `p` column.
inline unsigned cli_virtual_ranks() {
    const char *s = std::getenv("CAC_VIRTUAL_RANKS");
    if (!s || !*s) return 1;
    long v = std::strtol(s, nullptr, 10);
    return v > 0 ? (unsigned)v : 1;
}

// The reference's own random draws where a command line offers them (approx_cut:
// cac_approx_cut_seed_replay): CAC_SEED_REPLAY=1 requires them, 0 turns them off; unset, they are
// used wherever the graph allows (approx_cut: unit edge weights). Returns 1, 0 or -1 (unset).
inline int cli_seed_replay() {
    const char *s = std::getenv("CAC_SEED_REPLAY");
    if (!s || !*s) return -1;
    return std::string(s) != "0" ? 1 : 0;
}

inline int cli_device() {
    const char *s = std::getenv("CAC_DEVICE");
    return s && *s ? std::atoi(s) : 0;
}

inline int cli_fail(const char *what, int status) {
    std::fprintf(stderr, "%s failed: %s (%d): %s\n", what, cac_error_string(status), status, cac_last_error());
    return 1;
}
