// Instantiations of sde_fwd_kernel for the CIR model (double): device noise and
// injected increments for groups of 1..16 states (time-dependent coefficients
// are reloaded by every FP64 kernel), antithetic pairs for groups of up to 8.
#include "sde_kernels.cuh"

namespace sdegpu {

FwdLauncher<double> find_fwd_f64_cir(int maxm, bool inject, bool anti, int *bps) {
#define SDE_CIR(M, INJ, TD, AN)                                                               \
    if (maxm == M && inject == INJ && !TD && anti == AN) {                               \
        if (bps) *bps = fwd_max_blocks_per_sm<double, SDE_MODEL_CIR, M, INJ, false, TD, AN>();  \
        return &launch_fwd<double, SDE_MODEL_CIR, M, INJ, false, TD, AN>;                      \
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
    SDE_CIR(1, false, false, true)
    SDE_CIR(2, false, false, true)
    SDE_CIR(4, false, false, true)
    SDE_CIR(8, false, false, true)
#undef SDE_CIR
    return nullptr;
}

}  // namespace sdegpu
