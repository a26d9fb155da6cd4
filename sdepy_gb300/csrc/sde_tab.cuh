// The FP32 LINEAR / OU forward kernel with device noise and no jumps: the
// hot path of the correlated Ornstein-Uhlenbeck and lognormal workloads.
//
// It computes what sde_fwd_kernel computes for these models (the same
// Philox counters, normals, coefficient run tables and Euler arithmetic),
// written so that every operand of the step loop is a register, a
// constant-bank operand of the parameter block (Philox round keys, the
// packed Cholesky factor) or a float4 load of a coefficient row that hits
// L1.  Two rules keep it so, each measured with ncu instruction counters
// against copies of the kernel:
//   * nothing takes the address of the parameter block (no reference to it
//     is handed to a helper, no pointer into it escapes): once its address
//     is taken, parameter reads in the step loop become loads (19 more
//     instructions per path-step);
//   * no block reduction lives in the kernel: the montecarlo summary of the
//     stored row runs as a second launch (tab_row_partials_kernel), since
//     the reductions' register demand also costs the step loop its
//     constant operands (8 loads and 11 instructions per path-step, 11 % of
//     the kernel's time).
//
// One thread owns one path of one group and walks the grid's runs of steps
// (FwdArgs::runs) with the state in registers:
//   OU      y' = (y - d y) + c (L z'),  y = x - theta0 (rows (d, c));
//   LINEAR  x' = (x + b) + c (L z')                    (rows (b, c));
// with normals z' = z / sqrt(2 ln 2) (the factor sits in c).  Groups of
// four or more states draw one Philox call per four normals per step;
// groups of one or two share one call between two steps (PairedSteps).
// Outputs are stored at the end of each run whose output row is set; the
// summarised row goes to FwdArgs::stats_vals (or is read back from xx), and
// launch_fwd_tab reduces it into the per-block partials of a fused summary.
#pragma once

#include "sde_kernels.cuh"

namespace sdegpu {

// resident blocks per SM for up to 8 states (none asked for 16), and steps
// per iteration of the step loop; compile-time defaults that a build may
// override to compare launch shapes
#ifndef SDE_TAB_MIN_BLOCKS
#define SDE_TAB_MIN_BLOCKS 3
#endif
#ifndef SDE_TAB_UNROLL
#define SDE_TAB_UNROLL 2
#endif
template <int MAXM>
struct TabOccupancy {
    static constexpr int MIN_BLOCKS = MAXM <= 8 ? SDE_TAB_MIN_BLOCKS : 1;
};

// store the group's outputs of one path at output row `row`, and the
// summarised row's values into stats_vals; sh: the state is the deviation
// from theta0.  The parameters come as values read at the call site (a
// reference to the parameter block would take its address).
template <int MAXM>
__device__ __forceinline__ void tab_store(float *xx, float *stats_vals, const float *tshift, int64_t paths,
                                          int64_t n_out_vars, int M, int out_mode, int opg, int stats_row,
                                          int g, int64_t p, int row, bool sh, const float (&s)[MAXM]) {
    float sx[MAXM], ov[MAXM];
#pragma unroll
    for (int m = 0; m < MAXM; ++m) sx[m] = sh ? s[m] + __ldg(tshift + g * 2 * MAXM + m) : s[m];
    const int no = group_outputs<float, MAXM>(sx, M, out_mode, ov);
    if (xx) {
#pragma unroll
        for (int m = 0; m < MAXM; ++m)
            if (m < no) __stcs(&xx[((int64_t)row * n_out_vars + (int64_t)g * opg + m) * paths + p], ov[m]);
    }
    if (row == stats_row && stats_vals) {
#pragma unroll
        for (int m = 0; m < MAXM; ++m)
            if (m < no) __stcs(&stats_vals[((int64_t)g * opg + m) * paths + p], ov[m]);
    }
}

#define SDE_TAB_STORE(row, sh)                                                                                 \
    tab_store<MAXM>(a.xx, a.stats_vals, a.tshift, a.paths, a.n_out_vars, a.M, a.out_mode, a.opg, a.stats_row, g, \
                    p, (row), (sh), st)

template <int MODEL, int MAXM, bool CORR>
__global__ void __launch_bounds__(BLOCK, TabOccupancy<MAXM>::MIN_BLOCKS)
sde_fwd_tab_kernel(const __grid_constant__ FwdArgs<float> a) {
    constexpr bool SHIFT = MODEL == SDE_MODEL_OU;
    constexpr int NCN = (MAXM + 3) / 4;                 // Philox calls of normals per step (MAXM >= 4)
    constexpr int NZ = MAXM == 1 ? 1 : (MAXM == 2 ? 2 : 0);
    constexpr int UNROLL = SDE_TAB_UNROLL;

    const int g = blockIdx.y;
    const int P2 = (a.M + 1) >> 1;
    const int NC = (2 * P2 + 3) >> 2;                   // calls this group needs (<= NCN)
    const int n_steps = a.n_pts - 1;
    const PhiloxKey key = a.key;
    const uint32_t step_offset = a.step_offset;
    if ((a.coef == nullptr || a.runs == nullptr || (SHIFT && a.tshift == nullptr)) && n_steps > 0) {
        if (threadIdx.x == 0 && blockIdx.x == 0 && blockIdx.y == 0) atomicOr(a.err, ERRF_ARGS);
        return;
    }
    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    for (int64_t p = (int64_t)blockIdx.x * BLOCK + threadIdx.x; p < a.paths; p += stride) {
        float st[MAXM];   // x0, read per path: only the step's values stay live across the loop
#pragma unroll
        for (int m = 0; m < MAXM; ++m) st[m] = __ldg(a.x0 + g * a.M + (m < a.M ? m : 0));
        {
            const int r0 = a.out_row[0];
            if (r0 >= 0) SDE_TAB_STORE(r0, false);
        }
        if (SHIFT && n_steps > 0) {
#pragma unroll
            for (int m = 0; m < MAXM; ++m) st[m] = __ldg(a.tshift + (g * 2 + 1) * MAXM + m);
        }
        // first Philox rounds of this path's calls (independent of the step)
        const PathPre<NZ ? 1 : NCN> pre(key, (uint32_t)p + a.path_offset, (uint32_t)g, a.stream);
        PairedSteps<float, NZ ? NZ : 1, true> pair;

#pragma unroll 1
        for (int ri = 0; ri < a.n_runs; ++ri) {
            const int4 run = __ldg(a.runs + ri);
            const float *tb = a.coef + ((int64_t)run.w * a.groups + g) * 2 * MAXM;
#pragma unroll UNROLL
            for (int k = run.x; k < run.y; ++k) {
                float dW[MAXM];
                if constexpr (NZ == 1) {
                    uint32_t w_unused;
                    pair.get(key, pre, k, step_offset, dW[0], w_unused);
                } else if constexpr (NZ == 2) {
                    float z0, z1;
                    pair.get(key, pre, k, step_offset, z0, z1);
                    if (CORR) {
                        dW[0] = a.chol[0] * z0;
                        dW[1] = fmaf(a.chol[2], z1, a.chol[1] * z0);
                    } else {
                        dW[0] = z0;
                        dW[1] = z1;
                    }
                } else {
                    const uint32_t c1w = (uint32_t)k + step_offset;
#pragma unroll
                    for (int c = 0; c < NCN; ++c) {
                        if (c < NC) {
                            const uint4 r = philox_from_round0(pre.r0[c], c1w, key);
                            float zc[4];
                            Rng<float>::normal2_s(r.x, r.y, zc[0], zc[1]);
                            Rng<float>::normal2_s(r.z, r.w, zc[2], zc[3]);
#pragma unroll
                            for (int l = 0; l < 4; ++l) {
                                const int j = 4 * c + l;
                                if (!CORR) {
                                    dW[j] = zc[l];
                                    continue;
                                }
#pragma unroll
                                for (int m = 0; m < MAXM; ++m) {
                                    if (m >= j) {
                                        const float L = a.chol[m * (m + 1) / 2 + j];
                                        dW[m] = (j == 0) ? L * zc[l] : fmaf(L, zc[l], dW[m]);
                                    }
                                }
                            }
                        } else if (!CORR) {
#pragma unroll
                            for (int l = 0; l < 4; ++l) dW[4 * c + l] = 0.0f;
                        }
                    }
                }
                // this step's coefficient row (d or b, c), padded to MAXM
                float ca[MAXM], cc[MAXM];
                if constexpr (MAXM % 4 == 0) {
#pragma unroll
                    for (int q = 0; q < MAXM / 4; ++q) {
                        const float4 va = __ldg(reinterpret_cast<const float4 *>(tb) + q);
                        const float4 vc = __ldg(reinterpret_cast<const float4 *>(tb + MAXM) + q);
                        ca[4 * q] = va.x; ca[4 * q + 1] = va.y; ca[4 * q + 2] = va.z; ca[4 * q + 3] = va.w;
                        cc[4 * q] = vc.x; cc[4 * q + 1] = vc.y; cc[4 * q + 2] = vc.z; cc[4 * q + 3] = vc.w;
                    }
                } else {
#pragma unroll
                    for (int m = 0; m < MAXM; ++m) {
                        ca[m] = __ldg(tb + m);
                        cc[m] = __ldg(tb + MAXM + m);
                    }
                }
#pragma unroll
                for (int m = 0; m < MAXM; ++m) {
                    float x = st[m];
                    if (SHIFT) x = fmaf(-ca[m], x, x);   // y - d y
                    else x = x + ca[m];                  // x + b
                    st[m] = fmaf(cc[m], dW[m], x);
                }
            }
            if (run.z >= 0) SDE_TAB_STORE(run.z, SHIFT);
        }
    }
}

#undef SDE_TAB_STORE

// The summary of the stored row, by a second launch over the values the
// forward kernel stored (4 B per path and output, read once): the same
// block reductions over the same rounds of paths per block as the fused
// kernels, so the per-block partials [groups][blocks][opg][NPART] are the
// ones a fused summary would leave.
struct TabStrikes {
    float k[SDE_MAX_STRIKES];
};

static __global__ void __launch_bounds__(BLOCK)
tab_row_partials_kernel(const float *vals, int64_t paths, int64_t n_out, int opg, int n_strikes,
                        const TabStrikes ks, double *partials) {
    __shared__ float red[BLOCK / 32];
    __shared__ double part[NPART];
    __shared__ float strikes[SDE_MAX_STRIKES];
    if (threadIdx.x < SDE_MAX_STRIKES) strikes[threadIdx.x] = ks.k[threadIdx.x];
    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    const int64_t rounds = (paths + stride - 1) / stride;
    for (int64_t o = blockIdx.y; o < n_out; o += gridDim.y) {   // output = group * opg + m
        __syncthreads();   // the previous output's partial is written out
        if (threadIdx.x == 0) {
            for (int i = 0; i < NPART; ++i) part[i] = 0.0;
            part[5] = INFINITY;
            part[6] = -INFINITY;
        }
        __syncthreads();
        const float *v = vals + o * paths;
        for (int64_t rd = 0; rd < rounds; ++rd) {
            const int64_t p = rd * stride + (int64_t)blockIdx.x * BLOCK + threadIdx.x;
            const bool act = p < paths;
            block_round_stats<float>(act ? __ldcs(v + p) : 0.0f, act, strikes, n_strikes, part, red);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int64_t g = o / opg, m = o % opg;
            double *dst = partials + ((g * gridDim.x + blockIdx.x) * opg + m) * NPART;
            for (int i = 0; i < NPART; ++i) dst[i] = part[i];
        }
    }
}

#ifndef __CUDACC_RTC__
// the forward launch, then the summary of the stored row when partials are
// asked for (FwdArgs::partials): its values are stats_vals, or the row of
// xx (device memory) when stats_vals is not set
template <int MODEL, int MAXM>
void launch_fwd_tab(const FwdArgs<float> &a, dim3 grid, cudaStream_t s) {
    if (a.has_corr && MAXM > 1) sde_fwd_tab_kernel<MODEL, MAXM, true><<<grid, BLOCK, 0, s>>>(a);
    else sde_fwd_tab_kernel<MODEL, MAXM, false><<<grid, BLOCK, 0, s>>>(a);
    if (a.partials && a.stats_row >= 0) {
        const float *vals = a.stats_vals ? a.stats_vals : a.xx ? a.xx + (int64_t)a.stats_row * a.n_out_vars * a.paths
                                                                : nullptr;
        if (!vals) return;   // callers provide one of the two (run_impl, sde_run_stats_static)
        TabStrikes ks;
        for (int i = 0; i < SDE_MAX_STRIKES; ++i) ks.k[i] = a.strikes[i];
        const int64_t n_out = (int64_t)grid.y * a.opg;
        tab_row_partials_kernel<<<dim3(grid.x, (unsigned)(n_out < 65535 ? n_out : 65535)), BLOCK, 0, s>>>(
            vals, a.paths, n_out, a.opg, a.n_strikes, ks, a.partials);
    }
}

template <int MODEL, int MAXM>
int fwd_tab_max_blocks_per_sm() {
    int n = 0, n2 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sde_fwd_tab_kernel<MODEL, MAXM, true>, BLOCK, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n2, sde_fwd_tab_kernel<MODEL, MAXM, false>, BLOCK, 0);
    return n < n2 ? n : n2;
}
#endif

}  // namespace sdegpu
