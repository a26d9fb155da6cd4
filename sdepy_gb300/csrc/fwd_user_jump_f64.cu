// Instantiations of sde_fwd_kernel for user SDEs with Poisson (dn) and / or
// compound Poisson (dj) terms (double): single equations (groups of 1..16
// states; systems in fwd_user_jump_sys_f64.cu), device noise and injected
// increments.
#include "sde_kernels.cuh"

namespace sdegpu {

FwdLauncher<double> find_fwd_f64_user_jump(int maxm, bool inject, bool sys, int *bps) {
    if (sys) return find_fwd_f64_user_jump_sys(maxm, inject, bps);
#define SDE_USER_J(MODEL, M, INJ) \
    if (maxm == M && inject == INJ) { \
        if (bps) *bps = fwd_max_blocks_per_sm<double, MODEL, M, INJ, true>(); \
        return &launch_fwd<double, MODEL, M, INJ, true>; \
    }
    SDE_USER_J(SDE_MODEL_USER, 1, false)
    SDE_USER_J(SDE_MODEL_USER, 1, true)
    SDE_USER_J(SDE_MODEL_USER, 2, false)
    SDE_USER_J(SDE_MODEL_USER, 2, true)
    SDE_USER_J(SDE_MODEL_USER, 4, false)
    SDE_USER_J(SDE_MODEL_USER, 4, true)
    SDE_USER_J(SDE_MODEL_USER, 8, false)
    SDE_USER_J(SDE_MODEL_USER, 8, true)
    SDE_USER_J(SDE_MODEL_USER, 16, false)
    SDE_USER_J(SDE_MODEL_USER, 16, true)
#undef SDE_USER_J
    return nullptr;
}

}  // namespace sdegpu
