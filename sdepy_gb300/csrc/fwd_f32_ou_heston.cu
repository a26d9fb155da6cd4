// Instantiations of sde_fwd_kernel: fwd_f32_ou_heston (generated list, see sde_kernels.cuh)
#include "sde_kernels.cuh"
#include "sde_tab.cuh"

namespace sdegpu {

FwdLauncher<float> find_fwd_f32_ou_heston(int model, int maxm, bool inject, bool jumps, int *bps) {
    if (model == SDE_MODEL_OU && maxm == 1 && inject == false && jumps == false) {
        if (bps) *bps = fwd_tab_max_blocks_per_sm<SDE_MODEL_OU, 1>();
        return &launch_fwd_tab<SDE_MODEL_OU, 1>;
    }
    if (model == SDE_MODEL_OU && maxm == 1 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_OU, 1, true, false>();
        return &launch_fwd<float, SDE_MODEL_OU, 1, true, false>;
    }
    if (model == SDE_MODEL_OU && maxm == 2 && inject == false && jumps == false) {
        if (bps) *bps = fwd_tab_max_blocks_per_sm<SDE_MODEL_OU, 2>();
        return &launch_fwd_tab<SDE_MODEL_OU, 2>;
    }
    if (model == SDE_MODEL_OU && maxm == 2 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_OU, 2, true, false>();
        return &launch_fwd<float, SDE_MODEL_OU, 2, true, false>;
    }
    if (model == SDE_MODEL_OU && maxm == 4 && inject == false && jumps == false) {
        if (bps) *bps = fwd_tab_max_blocks_per_sm<SDE_MODEL_OU, 4>();
        return &launch_fwd_tab<SDE_MODEL_OU, 4>;
    }
    if (model == SDE_MODEL_OU && maxm == 4 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_OU, 4, true, false>();
        return &launch_fwd<float, SDE_MODEL_OU, 4, true, false>;
    }
    if (model == SDE_MODEL_OU && maxm == 8 && inject == false && jumps == false) {
        if (bps) *bps = fwd_tab_max_blocks_per_sm<SDE_MODEL_OU, 8>();
        return &launch_fwd_tab<SDE_MODEL_OU, 8>;
    }
    if (model == SDE_MODEL_OU && maxm == 8 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_OU, 8, true, false>();
        return &launch_fwd<float, SDE_MODEL_OU, 8, true, false>;
    }
    if (model == SDE_MODEL_OU && maxm == 16 && inject == false && jumps == false) {
        if (bps) *bps = fwd_tab_max_blocks_per_sm<SDE_MODEL_OU, 16>();
        return &launch_fwd_tab<SDE_MODEL_OU, 16>;
    }
    if (model == SDE_MODEL_OU && maxm == 16 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_OU, 16, true, false>();
        return &launch_fwd<float, SDE_MODEL_OU, 16, true, false>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 2 && inject == false && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_HESTON, 2, false, false>();
        return &launch_fwd<float, SDE_MODEL_HESTON, 2, false, false>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 2 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_HESTON, 2, true, false>();
        return &launch_fwd<float, SDE_MODEL_HESTON, 2, true, false>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 4 && inject == false && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_HESTON, 4, false, false>();
        return &launch_fwd<float, SDE_MODEL_HESTON, 4, false, false>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 4 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_HESTON, 4, true, false>();
        return &launch_fwd<float, SDE_MODEL_HESTON, 4, true, false>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 8 && inject == false && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_HESTON, 8, false, false>();
        return &launch_fwd<float, SDE_MODEL_HESTON, 8, false, false>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 8 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_HESTON, 8, true, false>();
        return &launch_fwd<float, SDE_MODEL_HESTON, 8, true, false>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 16 && inject == false && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_HESTON, 16, false, false>();
        return &launch_fwd<float, SDE_MODEL_HESTON, 16, false, false>;
    }
    if (model == SDE_MODEL_HESTON && maxm == 16 && inject == true && jumps == false) {
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_HESTON, 16, true, false>();
        return &launch_fwd<float, SDE_MODEL_HESTON, 16, true, false>;
    }
    return nullptr;
}


// time-dependent coefficients and correlations (device noise, no jumps):
// LINEAR run tables, OU run tables with the theta term, Heston with per-step
// coefficient reloads; all with per-step correlation factors
FwdLauncher<float> find_fwd_f32_tdep(int model, int maxm, int *bps) {
#define SDE_TDEP(MODEL, M)                                                               \
    if (model == MODEL && maxm == M) {                                                   \
        if (bps) *bps = fwd_max_blocks_per_sm<float, MODEL, M, false, false, true>();    \
        return &launch_fwd<float, MODEL, M, false, false, true>;                         \
    }
    SDE_TDEP(SDE_MODEL_LINEAR, 1)
    SDE_TDEP(SDE_MODEL_LINEAR, 2)
    SDE_TDEP(SDE_MODEL_LINEAR, 4)
    SDE_TDEP(SDE_MODEL_LINEAR, 8)
    SDE_TDEP(SDE_MODEL_LINEAR, 16)
    SDE_TDEP(SDE_MODEL_OU, 1)
    SDE_TDEP(SDE_MODEL_OU, 2)
    SDE_TDEP(SDE_MODEL_OU, 4)
    SDE_TDEP(SDE_MODEL_OU, 8)
    SDE_TDEP(SDE_MODEL_OU, 16)
    SDE_TDEP(SDE_MODEL_HESTON, 2)
    SDE_TDEP(SDE_MODEL_HESTON, 4)
    SDE_TDEP(SDE_MODEL_HESTON, 8)
    SDE_TDEP(SDE_MODEL_HESTON, 16)
#undef SDE_TDEP
    return nullptr;
}

}  // namespace sdegpu
