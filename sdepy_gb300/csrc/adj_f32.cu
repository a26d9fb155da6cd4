// Instantiations of sde_adj_kernel (float)
#include "sde_adjoint.cuh"
#include "sde_adj_heston.cuh"
#include "sde_adj_ou.cuh"

namespace sdegpu {

AdjLauncher<float> find_adj_f32(int model, int maxm, bool jumps, int *bps) {
    if (model == SDE_MODEL_LINEAR && maxm == 1 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 1, false>();
        return &launch_adj<float, SDE_MODEL_LINEAR, 1, false>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 1 && jumps == true) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 1, true>();
        return &launch_adj<float, SDE_MODEL_LINEAR, 1, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 2 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 2, false>();
        return &launch_adj<float, SDE_MODEL_LINEAR, 2, false>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 2 && jumps == true) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 2, true>();
        return &launch_adj<float, SDE_MODEL_LINEAR, 2, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 4 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 4, false>();
        return &launch_adj<float, SDE_MODEL_LINEAR, 4, false>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 4 && jumps == true) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 4, true>();
        return &launch_adj<float, SDE_MODEL_LINEAR, 4, true>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 8 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 8, false>();
        return &launch_adj<float, SDE_MODEL_LINEAR, 8, false>;
    }
    if (model == SDE_MODEL_LINEAR && maxm == 8 && jumps == true) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_LINEAR, 8, true>();
        return &launch_adj<float, SDE_MODEL_LINEAR, 8, true>;
    }
    if (model == SDE_MODEL_OU && maxm == 1 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_OU, 1, false>();
        return &launch_adj<float, SDE_MODEL_OU, 1, false>;
    }
    if (model == SDE_MODEL_OU && maxm == 2 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_OU, 2, false>();
        return &launch_adj<float, SDE_MODEL_OU, 2, false>;
    }
    if (model == SDE_MODEL_OU && maxm == 4 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_OU, 4, false>();
        return &launch_adj<float, SDE_MODEL_OU, 4, false>;
    }
    if (model == SDE_MODEL_OU && maxm == 8 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_OU, 8, false>();
        return &launch_adj<float, SDE_MODEL_OU, 8, false>;
    }
    if (model == SDE_MODEL_CIR && maxm == 1 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_CIR, 1, false>();
        return &launch_adj<float, SDE_MODEL_CIR, 1, false>;
    }
    if (model == SDE_MODEL_CIR && maxm == 2 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_CIR, 2, false>();
        return &launch_adj<float, SDE_MODEL_CIR, 2, false>;
    }
    if (model == SDE_MODEL_CIR && maxm == 4 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_CIR, 4, false>();
        return &launch_adj<float, SDE_MODEL_CIR, 4, false>;
    }
    if (model == SDE_MODEL_CIR && maxm == 8 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_CIR, 8, false>();
        return &launch_adj<float, SDE_MODEL_CIR, 8, false>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 2 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_HESTON, 2, false>();
        return &launch_adj<float, SDE_MODEL_HESTON, 2, false>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 4 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_HESTON, 4, false>();
        return &launch_adj<float, SDE_MODEL_HESTON, 4, false>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 8 && jumps == false) {
        if (bps) *bps = adj_max_blocks_per_sm<float, SDE_MODEL_HESTON, 8, false>();
        return &launch_adj<float, SDE_MODEL_HESTON, 8, false>;
    }
    return nullptr;
}

AdjLauncher<float> find_adj_ou_f32(int seg, int *bps) {
    if (seg < 1 || seg > ADJ_OU_SEG) return nullptr;
    if (bps) *bps = adj_ou_max_blocks_per_sm(seg);
    return &launch_adj_ou;
}

AdjLauncher<float> find_adj_heston_f32(int seg, int *bps) {
    if (seg < 1 || seg > ADJ_HESTON_SEG) return nullptr;
    if (bps) *bps = adj_heston_max_blocks_per_sm(seg);
    return &launch_adj_heston;
}

}  // namespace sdegpu
