// Instantiations of sde_fwd_kernel for user SDEs (float): single equations
// (SDE_MODEL_USER, groups of 1..16 states) and systems of equations
// (SDE_MODEL_USER_SYS, groups of 2..16), device noise and injected increments.
#include "sde_kernels.cuh"

namespace sdegpu {

FwdLauncher<float> find_fwd_f32_user(int maxm, bool inject, bool sys, bool jumps, int *bps) {
    if (jumps) return find_fwd_f32_user_jump(maxm, inject, sys, bps);
#define SDE_USER(MODEL, M, INJ)                                                            \
    if (maxm == M && inject == INJ && sys == (MODEL == SDE_MODEL_USER_SYS)) {              \
        if (bps) *bps = fwd_max_blocks_per_sm<float, MODEL, M, INJ, false>();               \
        return &launch_fwd<float, MODEL, M, INJ, false>;                                    \
    }
    SDE_USER(SDE_MODEL_USER, 1, false)
    SDE_USER(SDE_MODEL_USER, 1, true)
    SDE_USER(SDE_MODEL_USER, 2, false)
    SDE_USER(SDE_MODEL_USER, 2, true)
    SDE_USER(SDE_MODEL_USER, 4, false)
    SDE_USER(SDE_MODEL_USER, 4, true)
    SDE_USER(SDE_MODEL_USER, 8, false)
    SDE_USER(SDE_MODEL_USER, 8, true)
    SDE_USER(SDE_MODEL_USER, 16, false)
    SDE_USER(SDE_MODEL_USER, 16, true)
    SDE_USER(SDE_MODEL_USER_SYS, 2, false)
    SDE_USER(SDE_MODEL_USER_SYS, 2, true)
    SDE_USER(SDE_MODEL_USER_SYS, 4, false)
    SDE_USER(SDE_MODEL_USER_SYS, 4, true)
    SDE_USER(SDE_MODEL_USER_SYS, 8, false)
    SDE_USER(SDE_MODEL_USER_SYS, 8, true)
    SDE_USER(SDE_MODEL_USER_SYS, 16, false)
    SDE_USER(SDE_MODEL_USER_SYS, 16, true)
#undef SDE_USER
    return nullptr;
}

}  // namespace sdegpu
