// Runtime compilation of user SDE programs (sde_jit.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/sdepy_gb300.h"

namespace sdegpu {

// true when NVRTC could be loaded
bool jit_available();

// compile (no load) the forward kernel of a program: the code generator and
// NVRTC without a device
int jit_compile_check(const SdeUserProgram &u, bool fp64, int maxm, bool inject, bool jumps, std::string *err);
int jit_compile_check_adjoint(const SdeUserProgram &u, bool fp64, int mg, std::string *err);

// the forward kernel with the program's coefficients compiled in
// (SDE_MODEL_USER_JIT, or SDE_MODEL_USER_SYS_JIT for systems), compiled on
// first use and cached; *bps its resident blocks per SM.  Returns SDE_OK or
// an SDE_ERR_* status with a message in *err.
int jit_fwd_kernel(const SdeUserProgram &u, bool fp64, int maxm, bool inject, bool jumps, cudaKernel_t *kernel,
                   int *bps, std::string *err);

// the adjoint kernel of a program for groups of mg states
// (sde_adj_user_kernel, with the program's coefficients and reverse-mode
// step compiled in), compiled on first use and cached; launched with its
// segment buffer as dynamic shared memory
int jit_adj_kernel(const SdeUserProgram &u, bool fp64, int mg, cudaKernel_t *kernel, std::string *err);

}  // namespace sdegpu
