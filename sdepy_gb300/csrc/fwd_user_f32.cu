// Instantiations of sde_fwd_kernel for user SDEs (SDE_MODEL_USER, float): device
// noise and injected increments, groups of 1..16 states.
#include "sde_kernels.cuh"

namespace sdegpu {

FwdLauncher<float> find_fwd_f32_user(int maxm, bool inject, int *bps) {
#define SDE_USER(M, INJ)                                                                   \
    if (maxm == M && inject == INJ) {                                                      \
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_USER, M, INJ, false>();      \
        return &launch_fwd<float, SDE_MODEL_USER, M, INJ, false>;                           \
    }
    SDE_USER(1, false)
    SDE_USER(1, true)
    SDE_USER(2, false)
    SDE_USER(2, true)
    SDE_USER(4, false)
    SDE_USER(4, true)
    SDE_USER(8, false)
    SDE_USER(8, true)
    SDE_USER(16, false)
    SDE_USER(16, true)
#undef SDE_USER
    return nullptr;
}

}  // namespace sdegpu
