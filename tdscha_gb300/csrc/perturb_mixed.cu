// Mixed-precision perturbation averages (tensor cores).  Placeholder until
// the tcgen05 GEMM pipeline lands: reports that the mode is unavailable.
#include "common.cuh"

namespace tdscha {

int mixed_prepare(tdscha_ctx *c) { (void)c; return TDSCHA_OK; }
int mixed_release(tdscha_ctx *c) { (void)c; return TDSCHA_OK; }
int perturb_mixed(tdscha_ctx *c, int apply_d4, cudaStream_t st) {
    (void)c; (void)apply_d4; (void)st;
    set_error("mixed precision is not available in this build");
    return TDSCHA_ERR_STATE;
}

}  // namespace tdscha
