// Instantiations of sde_fwd_kernel for user SDEs with Poisson (dn) and / or
// compound Poisson (dj) terms (double): systems of equations (groups of 2..16
// states), device noise and injected increments.
#include "sde_kernels.cuh"

namespace sdegpu {

FwdLauncher<double> find_fwd_f64_user_jump_sys(int maxm, bool inject, int *bps) {
#define SDE_USER_J(MODEL, M, INJ) \
    if (maxm == M && inject == INJ) { \
        if (bps) *bps = fwd_max_blocks_per_sm<double, MODEL, M, INJ, true>(); \
        return &launch_fwd<double, MODEL, M, INJ, true>; \
    }
    SDE_USER_J(SDE_MODEL_USER_SYS, 2, false)
    SDE_USER_J(SDE_MODEL_USER_SYS, 2, true)
    SDE_USER_J(SDE_MODEL_USER_SYS, 4, false)
    SDE_USER_J(SDE_MODEL_USER_SYS, 4, true)
    SDE_USER_J(SDE_MODEL_USER_SYS, 8, false)
    SDE_USER_J(SDE_MODEL_USER_SYS, 8, true)
    SDE_USER_J(SDE_MODEL_USER_SYS, 16, false)
    SDE_USER_J(SDE_MODEL_USER_SYS, 16, true)
#undef SDE_USER_J
    return nullptr;
}

}  // namespace sdegpu
