// Instantiations of sde_fwd_kernel with antithetic paths (ANTI) and
// time-dependent coefficients or correlations (TDEP: per-step reloads, OU
// rows with the theta term), device noise, groups of up to 8 states: float
#include "sde_kernels.cuh"

namespace sdegpu {

FwdLauncher<float> find_fwd_f32_anti_tdep(int model, int maxm, bool jumps, int *bps) {
#define SDE_AT(MODEL, M, J)                                                                    \
    if (model == MODEL && maxm == M && jumps == J) {                                          \
        if (bps) *bps = fwd_max_blocks_per_sm<float, MODEL, M, false, J, true, true>();        \
        return &launch_fwd<float, MODEL, M, false, J, true, true>;                             \
    }
    SDE_AT(SDE_MODEL_LINEAR, 1, false)
    SDE_AT(SDE_MODEL_LINEAR, 1, true)
    SDE_AT(SDE_MODEL_LINEAR, 2, false)
    SDE_AT(SDE_MODEL_LINEAR, 2, true)
    SDE_AT(SDE_MODEL_LINEAR, 4, false)
    SDE_AT(SDE_MODEL_LINEAR, 4, true)
    SDE_AT(SDE_MODEL_LINEAR, 8, false)
    SDE_AT(SDE_MODEL_LINEAR, 8, true)
    SDE_AT(SDE_MODEL_OU, 1, false)
    SDE_AT(SDE_MODEL_OU, 2, false)
    SDE_AT(SDE_MODEL_OU, 4, false)
    SDE_AT(SDE_MODEL_OU, 8, false)
    SDE_AT(SDE_MODEL_HESTON, 2, false)
    SDE_AT(SDE_MODEL_HESTON, 4, false)
    SDE_AT(SDE_MODEL_HESTON, 8, false)
#undef SDE_AT
    return nullptr;
}

}  // namespace sdegpu
