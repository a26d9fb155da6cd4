// Instantiations of sde_fwd_kernel with antithetic paths (ANTI), device noise,
// groups of up to 8 states: float
#include "sde_kernels.cuh"

namespace sdegpu {

FwdLauncher<float> find_fwd_f32_anti(int model, int maxm, bool jumps, int *bps) {
    if (model == SDE_MODEL_LINEAR && maxm == 1 && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 1, false, false, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 1, false, false, false, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 1 && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 1, false, true, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 1, false, true, false, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 2 && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 2, false, false, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 2, false, false, false, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 2 && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 2, false, true, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 2, false, true, false, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 4 && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 4, false, false, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 4, false, false, false, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 4 && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 4, false, true, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 4, false, true, false, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 8 && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 8, false, false, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 8, false, false, false, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 8 && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 8, false, true, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 8, false, true, false, true>;
    }
    if (model == SDE_MODEL_OU && maxm == 1 && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_OU, 1, false, false, false, true>();
        return &launch_fwd<float, SDE_MODEL_OU, 1, false, false, false, true>;
    }
    if (model == SDE_MODEL_OU && maxm == 2 && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_OU, 2, false, false, false, true>();
        return &launch_fwd<float, SDE_MODEL_OU, 2, false, false, false, true>;
    }
    if (model == SDE_MODEL_OU && maxm == 4 && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_OU, 4, false, false, false, true>();
        return &launch_fwd<float, SDE_MODEL_OU, 4, false, false, false, true>;
    }
    if (model == SDE_MODEL_OU && maxm == 8 && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_OU, 8, false, false, false, true>();
        return &launch_fwd<float, SDE_MODEL_OU, 8, false, false, false, true>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 2 && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_HESTON, 2, false, false, false, true>();
        return &launch_fwd<float, SDE_MODEL_HESTON, 2, false, false, false, true>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 4 && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_HESTON, 4, false, false, false, true>();
        return &launch_fwd<float, SDE_MODEL_HESTON, 4, false, false, false, true>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 8 && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_HESTON, 8, false, false, false, true>();
        return &launch_fwd<float, SDE_MODEL_HESTON, 8, false, false, false, true>;
    }
    return nullptr;
}

}  // namespace sdegpu
