// Instantiations of sde_fwd_kernel: fwd_f32_linear (generated list, see sde_kernels.cuh)
#include "sde_kernels.cuh"
#include "sde_tab.cuh"

namespace sdegpu {

FwdLauncher<float> find_fwd_f32_linear(int model, int maxm, bool inject, bool jumps, int *bps) {
    if (model == SDE_MODEL_LINEAR && maxm == 1 && inject == false && jumps == false) {
        if (bps) *bps = fwd_tab_max_blocks_per_sm<SDE_MODEL_LINEAR, 1>();
        return &launch_fwd_tab<SDE_MODEL_LINEAR, 1>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 1 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 1, true, false>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 1, true, false>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 1 && inject == false && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 1, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 1, false, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 1 && inject == true && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 1, true, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 1, true, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 2 && inject == false && jumps == false) {
        if (bps) *bps = fwd_tab_max_blocks_per_sm<SDE_MODEL_LINEAR, 2>();
        return &launch_fwd_tab<SDE_MODEL_LINEAR, 2>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 2 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 2, true, false>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 2, true, false>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 2 && inject == false && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 2, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 2, false, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 2 && inject == true && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 2, true, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 2, true, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 4 && inject == false && jumps == false) {
        if (bps) *bps = fwd_tab_max_blocks_per_sm<SDE_MODEL_LINEAR, 4>();
        return &launch_fwd_tab<SDE_MODEL_LINEAR, 4>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 4 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 4, true, false>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 4, true, false>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 4 && inject == false && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 4, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 4, false, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 4 && inject == true && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 4, true, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 4, true, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 8 && inject == false && jumps == false) {
        if (bps) *bps = fwd_tab_max_blocks_per_sm<SDE_MODEL_LINEAR, 8>();
        return &launch_fwd_tab<SDE_MODEL_LINEAR, 8>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 8 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 8, true, false>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 8, true, false>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 8 && inject == false && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 8, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 8, false, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 8 && inject == true && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 8, true, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 8, true, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 16 && inject == false && jumps == false) {
        if (bps) *bps = fwd_tab_max_blocks_per_sm<SDE_MODEL_LINEAR, 16>();
        return &launch_fwd_tab<SDE_MODEL_LINEAR, 16>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 16 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 16, true, false>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 16, true, false>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 16 && inject == false && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 16, false, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 16, false, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 16 && inject == true && jumps == true) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 16, true, true>();
        return &launch_fwd<float, SDE_MODEL_LINEAR, 16, true, true>;
    }
    return nullptr;
}

}  // namespace sdegpu
