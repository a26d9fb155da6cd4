// Instantiations of sde_adj_kernel with time-dependent parameter slots (TD):
// per-step gradients of the preset models' coefficients, without jumps
#include "sde_adjoint.cuh"

namespace sdegpu {

#define SDE_ADJ_TD(R, MODEL, M)                                                        \
    if (model == MODEL && maxm == M) {                                                 \
        if (bps) *bps = adj_max_blocks_per_sm<R, MODEL, M, false, true>();             \
        return &launch_adj<R, MODEL, M, false, true>;                                  \
    }

AdjLauncher<float> find_adj_td_f32(int model, int maxm, int *bps) {
    SDE_ADJ_TD(float, SDE_MODEL_LINEAR, 1)
    SDE_ADJ_TD(float, SDE_MODEL_LINEAR, 2)
    SDE_ADJ_TD(float, SDE_MODEL_LINEAR, 4)
    SDE_ADJ_TD(float, SDE_MODEL_OU, 1)
    SDE_ADJ_TD(float, SDE_MODEL_OU, 2)
    SDE_ADJ_TD(float, SDE_MODEL_OU, 4)
    SDE_ADJ_TD(float, SDE_MODEL_CIR, 1)
    SDE_ADJ_TD(float, SDE_MODEL_CIR, 2)
    SDE_ADJ_TD(float, SDE_MODEL_HESTON, 2)
    return nullptr;
}

AdjLauncher<double> find_adj_td_f64(int model, int maxm, int *bps) {
    SDE_ADJ_TD(double, SDE_MODEL_LINEAR, 1)
    SDE_ADJ_TD(double, SDE_MODEL_LINEAR, 2)
    SDE_ADJ_TD(double, SDE_MODEL_LINEAR, 4)
    SDE_ADJ_TD(double, SDE_MODEL_OU, 1)
    SDE_ADJ_TD(double, SDE_MODEL_OU, 2)
    SDE_ADJ_TD(double, SDE_MODEL_OU, 4)
    SDE_ADJ_TD(double, SDE_MODEL_CIR, 1)
    SDE_ADJ_TD(double, SDE_MODEL_CIR, 2)
    SDE_ADJ_TD(double, SDE_MODEL_HESTON, 2)
    return nullptr;
}

#undef SDE_ADJ_TD

}  // namespace sdegpu
