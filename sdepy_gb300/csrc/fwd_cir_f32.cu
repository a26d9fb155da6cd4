// Instantiations of sde_fwd_kernel for the CIR model (float): device noise and
// injected increments for groups of 1..16 states, device noise with
// time-dependent coefficients (TDEP), antithetic pairs for groups of up to 8
// (with and without TDEP).
#include "sde_kernels.cuh"

namespace sdegpu {

FwdLauncher<float> find_fwd_f32_cir(int maxm, bool inject, bool tdep, bool anti, int *bps) {
#define SDE_CIR(M, INJ, TD, AN)                                                               \
    if (maxm == M && inject == INJ && tdep == TD && anti == AN) {                               \
        if (bps) *bps = fwd_max_blocks_per_sm<float, SDE_MODEL_CIR, M, INJ, false, TD, AN>();  \
        return &launch_fwd<float, SDE_MODEL_CIR, M, INJ, false, TD, AN>;                      \
    }
    SDE_CIR(1, false, false, false)
    SDE_CIR(1, true, false, false)
    SDE_CIR(2, false, false, false)
    SDE_CIR(2, true, false, false)
    SDE_CIR(4, false, false, false)
    SDE_CIR(4, true, false, false)
    SDE_CIR(8, false, false, false)
    SDE_CIR(8, true, false, false)
    SDE_CIR(16, false, false, false)
    SDE_CIR(16, true, false, false)
    SDE_CIR(1, false, true, false)
    SDE_CIR(2, false, true, false)
    SDE_CIR(4, false, true, false)
    SDE_CIR(8, false, true, false)
    SDE_CIR(16, false, true, false)
    SDE_CIR(1, false, true, true)
    SDE_CIR(2, false, true, true)
    SDE_CIR(4, false, true, true)
    SDE_CIR(8, false, true, true)
    SDE_CIR(1, false, false, true)
    SDE_CIR(2, false, false, true)
    SDE_CIR(4, false, false, true)
    SDE_CIR(8, false, false, true)
#undef SDE_CIR
    return nullptr;
}

}  // namespace sdegpu
