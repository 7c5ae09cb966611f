// Minimum cut (placeholder until the trial kernels land).
#include "cac_internal.h"

namespace cac {
int mincut_trials(cac_ctx *, const cac_graph *, uint32_t, uint32_t, uint32_t, uint64_t *, float *) {
    set_error("square_root trials are not built yet");
    return CAC_ERR_UNSUPPORTED;
}
int ks_dense_one(cac_ctx *, uint32_t, const uint64_t *, uint32_t, uint32_t, uint32_t, uint64_t *) {
    set_error("Karger-Stein kernels are not built yet");
    return CAC_ERR_UNSUPPORTED;
}
int exact_small(cac_ctx *, uint32_t, const uint64_t *, uint64_t *) {
    set_error("Stoer-Wagner kernel is not built yet");
    return CAC_ERR_UNSUPPORTED;
}
int approx_run(cac_ctx *, const cac_graph *, double, uint32_t, uint32_t, cac_approx_result *) {
    set_error("approx_cut is not built yet");
    return CAC_ERR_UNSUPPORTED;
}
}  // namespace cac
