// k_learn.cu -- learned contractive projection and tile-pair pruning.
#include "ejoin_internal.cuh"

using namespace ejoin;

extern "C" int ejoin_train_projection(const double* points, uint64_t n, uint32_t d, double eps,
                                      const ejoin_options* opt, float* P_out,
                                      double* sigma_cert_out, ejoin_stats* stats_out) {
    (void)points; (void)n; (void)d; (void)eps; (void)opt; (void)P_out; (void)sigma_cert_out;
    (void)stats_out;
    return set_error(EJOIN_EUNSUPPORTED, "projection training not available in this build");
}
