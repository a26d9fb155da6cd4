// Instantiations of sde_adj_kernel for user SDEs (single equations driven
// by dt / dw; groups of 1..8 states), float and double.
#include "sde_adjoint.cuh"

namespace sdegpu {

template <typename R>
static AdjLauncher<R> find_adj_user(int maxm, int *bps) {
#define SDE_ADJ_USER(M)                                                        \
    if (maxm == M) {                                                           \
        if (bps) *bps = adj_max_blocks_per_sm<R, SDE_MODEL_USER, M, false>();  \
        return &launch_adj<R, SDE_MODEL_USER, M, false>;                       \
    }
    SDE_ADJ_USER(1)
    SDE_ADJ_USER(2)
    SDE_ADJ_USER(4)
    SDE_ADJ_USER(8)
#undef SDE_ADJ_USER
    return nullptr;
}

AdjLauncher<float> find_adj_user_f32(int maxm, int *bps) { return find_adj_user<float>(maxm, bps); }
AdjLauncher<double> find_adj_user_f64(int maxm, int *bps) { return find_adj_user<double>(maxm, bps); }

}  // namespace sdegpu
