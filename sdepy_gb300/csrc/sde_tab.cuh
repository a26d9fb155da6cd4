// The FP32 LINEAR / OU forward kernel with device noise and no jumps: the
// hot path of the correlated Ornstein-Uhlenbeck and lognormal workloads.
//
// It computes what sde_fwd_kernel computes for these models (the same
// Philox counters, normals, coefficient run tables and Euler arithmetic),
// written so that every operand of the step loop is a register, a
// constant-bank operand of the parameter block (Philox round keys, the
// packed Cholesky factor) or a float4 load of a coefficient row that hits
// L1.  What keeps it so was found by counting instructions with ncu
// against copies of the kernel (2^18 paths x 1008 steps, OU vshape 8,
// correlated), each change below a cut in thread-instructions per path-step:
//   * no block reduction in the kernel (205 -> 180 when the summary is
//     removed): the montecarlo summary of the stored row runs as a second
//     launch, tab_row_partials_kernel;
//   * every group draws its full calls (no test of the group's call count
//     in the step loop, 204 -> 179): padded states of a group narrower than
//     the kernel take draws that reach no output;
//   * the path loop runs in rounds of the grid's threads (178 -> 170), the
//     initial row (x0 itself) is written by a separate fill launch, and the
//     run-end store is the plain state store unless the output transform
//     is needed (ALT): 7.4 -> 7.0 ms per 2^20-path launch;
//   * nothing takes the address of the parameter block: helpers get values.
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

// the plain store of OUT_STATE: the states (theta0 added back for OU)
template <int MAXM, bool SHIFT>
__device__ __forceinline__ void tab_store_state(float *xx, float *stats_vals, const float *tshift, int64_t paths,
                                                int64_t n_out_vars, int opg, int stats_row, int g, int64_t p,
                                                int row, const float (&s)[MAXM], int M) {
    float ov[MAXM];
#pragma unroll
    for (int m = 0; m < MAXM; ++m) ov[m] = SHIFT ? s[m] + __ldg(tshift + g * 2 * MAXM + m) : s[m];
    if (xx) {
#pragma unroll
        for (int m = 0; m < MAXM; ++m)
            if (m < M) __stcs(&xx[((int64_t)row * n_out_vars + (int64_t)g * opg + m) * paths + p], ov[m]);
    }
    if (row == stats_row && stats_vals) {
#pragma unroll
        for (int m = 0; m < MAXM; ++m)
            if (m < M) __stcs(&stats_vals[((int64_t)g * opg + m) * paths + p], ov[m]);
    }
}

// ALT: an output transform other than OUT_STATE (exp of the states, their
// sum); the initial row is written by tab_row0_kernel.  CK: the OU state
// (theta0 added back) is also stored before every ckpt_seg-th step, the
// adjoint's checkpoints (FwdArgs::ckpt)
template <int MODEL, int MAXM, bool CORR, bool ALT, bool CK = false>
__global__ void __launch_bounds__(BLOCK, TabOccupancy<MAXM>::MIN_BLOCKS)
sde_fwd_tab_kernel(const __grid_constant__ FwdArgs<float> a) {
    constexpr bool SHIFT = MODEL == SDE_MODEL_OU;
    constexpr int NCN = (MAXM + 3) / 4;                 // Philox calls of normals per step (MAXM >= 4)
    constexpr int NZ = MAXM == 1 ? 1 : (MAXM == 2 ? 2 : 0);
    constexpr int UNROLL = SDE_TAB_UNROLL;

    const int g = blockIdx.y;
    const int n_steps = a.n_pts - 1;
    const PhiloxKey key = a.key;
    const uint32_t step_offset = a.step_offset;
    if ((a.coef == nullptr || a.runs == nullptr || (SHIFT && a.tshift == nullptr)) && n_steps > 0) {
        if (threadIdx.x == 0 && blockIdx.x == 0 && blockIdx.y == 0) atomicOr(a.err, ERRF_ARGS);
        return;
    }
    if (n_steps <= 0) return;
    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    const int64_t rounds = (a.paths + stride - 1) / stride;
    for (int64_t rd = 0; rd < rounds; ++rd) {
        const int64_t p = rd * stride + (int64_t)blockIdx.x * BLOCK + threadIdx.x;
        if (p >= a.paths) continue;
        float st[MAXM];   // x0, or x0 - theta0 for OU, read per path
#pragma unroll
        for (int m = 0; m < MAXM; ++m)
            st[m] = SHIFT ? __ldg(a.tshift + (g * 2 + 1) * MAXM + m) : __ldg(a.x0 + g * a.M + (m < a.M ? m : 0));
        // first Philox rounds of this path's calls (independent of the step)
        const PathPre<NZ ? 1 : NCN> pre(key, (uint32_t)p + a.path_offset, (uint32_t)g, a.stream);
        PairedSteps<float, NZ ? NZ : 1, true> pair;
        int next_ck = 0, ci = 0;   // CK: the next checkpoint's step and index

#pragma unroll 1
        for (int ri = 0; ri < a.n_runs; ++ri) {
            const int4 run = __ldg(a.runs + ri);
            const float *tb = a.coef + ((int64_t)run.w * a.groups + g) * 2 * MAXM;
#pragma unroll UNROLL
            for (int k = run.x; k < run.y; ++k) {
                if constexpr (CK) {
                    if (k == next_ck) {
#pragma unroll
                        for (int m = 0; m < MAXM; ++m)
                            if (m < a.M)
                                a.ckpt[((int64_t)ci * a.W + g * a.M + m) * a.paths + p] =
                                    SHIFT ? st[m] + __ldg(a.tshift + g * 2 * MAXM + m) : st[m];
                        ++ci;
                        next_ck += a.ckpt_seg;
                    }
                }
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
                        {
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
            if (run.z >= 0) {
                if (ALT) SDE_TAB_STORE(run.z, SHIFT);
                else tab_store_state<MAXM, SHIFT>(a.xx, a.stats_vals, a.tshift, a.paths, a.n_out_vars, a.opg,
                                                  a.stats_row, g, p, run.z, st, a.M);
            }
        }
    }
}

#undef SDE_TAB_STORE

// The summary of the stored row, by a second launch over the values the
// forward kernel stored (4 B per path and output, read twice, the second
// time from cache): block b of the grid summarises the paths of the same
// rounds a fused summary would give it (b * BLOCK + thread + k * stride),
// in two passes -- the block's mean, then the sums of the deviations from
// it, min, max and payoff sums, each reduced over the block once -- and
// writes its partial [groups][blocks][opg][NPART], recentred in FP64 on the
// refined mean as block_round_stats does.
struct TabStrikes {
    float k[SDE_MAX_STRIKES];
};

static __global__ void __launch_bounds__(BLOCK)
tab_row_partials_kernel(const float *vals, int64_t paths, int64_t n_out, int opg, int n_strikes,
                        const TabStrikes ks, double *partials) {
    __shared__ float red[BLOCK / 32];
    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    const int64_t first = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
    for (int64_t o = blockIdx.y; o < n_out; o += gridDim.y) {   // output = group * opg + m
        const float *v = vals + o * paths;
        float cnt = 0.f, s1 = 0.f;
        for (int64_t p = first; p < paths; p += stride) {
            s1 += __ldg(v + p);
            cnt += 1.f;
        }
        const float n = block_sum<float>(cnt, red);
        const float mean = n > 0.f ? block_sum<float>(s1, red) / n : 0.f;
        float r1 = 0.f, m2 = 0.f, m3 = 0.f, m4 = 0.f, mn = INFINITY, mx = -INFINITY;
        float pay[SDE_MAX_STRIKES];
#pragma unroll
        for (int i = 0; i < SDE_MAX_STRIKES; ++i) pay[i] = 0.f;
        for (int64_t p = first; p < paths; p += stride) {
            const float x = __ldcs(v + p);
            const float d = x - mean, d2 = d * d;
            r1 += d;
            m2 += d2;
            m3 += d2 * d;
            m4 += d2 * d2;
            mn = fminf(mn, x);
            mx = fmaxf(mx, x);
#pragma unroll
            for (int i = 0; i < SDE_MAX_STRIKES; ++i)
                if (i < n_strikes) pay[i] += fmaxf(x - ks.k[i], 0.f);
        }
        const float R1 = block_sum<float>(r1, red), M2 = block_sum<float>(m2, red);
        const float M3 = block_sum<float>(m3, red), M4 = block_sum<float>(m4, red);
        const float MN = block_min<float>(mn, red), MX = block_max<float>(mx, red);
        float P[SDE_MAX_STRIKES];
#pragma unroll
        for (int i = 0; i < SDE_MAX_STRIKES; ++i)
            if (i < n_strikes) P[i] = block_sum<float>(pay[i], red);
        if (threadIdx.x == 0) {
            double B[NPART];
            for (int i = 0; i < NPART; ++i) B[i] = 0.0;
            B[5] = INFINITY;
            B[6] = -INFINITY;
            if (n > 0.f) {
                // recentre on the refined mean (mean + R1/n) in FP64
                const double nn = (double)n, r = (double)R1, e = r / nn;
                const double a2 = (double)M2, a3 = (double)M3, a4 = (double)M4;
                B[0] = nn;
                B[1] = (double)mean + e;
                B[2] = a2 - r * e;
                B[3] = a3 - 3.0 * e * a2 + 2.0 * r * e * e;
                B[4] = a4 - 4.0 * e * a3 + 6.0 * e * e * a2 - 3.0 * r * e * e * e;
                B[5] = (double)MN;
                B[6] = (double)MX;
                for (int i = 0; i < n_strikes; ++i) B[8 + i] = (double)P[i];
            }
            const int64_t g = o / opg, m = o % opg;
            double *dst = partials + ((g * gridDim.x + blockIdx.x) * opg + m) * NPART;
            for (int i = 0; i < NPART; ++i) dst[i] = B[i];
        }
        __syncthreads();   // red is reused by the next output
    }
}

// The initial row: x0 itself, the same for every path (its output
// transform, into xx and, for the summarised row, stats_vals)
template <int MAXM>
__global__ void __launch_bounds__(BLOCK)
tab_row0_kernel(const float *x0, float *xx, float *stats_vals, int64_t paths, int64_t n_out_vars, int M, int out_mode,
                int opg, int row, int stats_row) {
    const int g = blockIdx.y;
    float s[MAXM], ov[MAXM];
#pragma unroll
    for (int m = 0; m < MAXM; ++m) s[m] = __ldg(x0 + g * M + (m < M ? m : 0));
    const int no = group_outputs<float, MAXM>(s, M, out_mode, ov);
    for (int64_t p = (int64_t)blockIdx.x * BLOCK + threadIdx.x; p < paths; p += (int64_t)gridDim.x * BLOCK) {
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
}

#ifndef __CUDACC_RTC__
// the initial row (host-known: FwdArgs::out_row is device memory, so the
// launcher takes the row from FwdArgs::tab_row0), the forward launch, then
// the summary of the stored row when partials are
// asked for (FwdArgs::partials): its values are stats_vals, or the row of
// xx (device memory) when stats_vals is not set
template <int MODEL, int MAXM>
void launch_fwd_tab(const FwdArgs<float> &a, dim3 grid, cudaStream_t s) {
    if (a.tab_row0 >= 0)
        tab_row0_kernel<MAXM><<<grid, BLOCK, 0, s>>>(a.x0, a.xx, a.stats_vals, a.paths, a.n_out_vars, a.M, a.out_mode,
                                                     a.opg, a.tab_row0, a.stats_row);
    const bool corr = a.has_corr && MAXM > 1, alt = a.out_mode != SDE_OUT_STATE;
    bool ck = false;
    if constexpr (MODEL == SDE_MODEL_OU && MAXM <= 8) {   // the OU state with the adjoint's checkpoints
        ck = a.ckpt && !alt;
        if (ck && corr) sde_fwd_tab_kernel<MODEL, MAXM, true, false, true><<<grid, BLOCK, 0, s>>>(a);
        else if (ck) sde_fwd_tab_kernel<MODEL, MAXM, false, false, true><<<grid, BLOCK, 0, s>>>(a);
    }
    if (ck) {
    } else if (corr && alt) {
        sde_fwd_tab_kernel<MODEL, MAXM, true, true><<<grid, BLOCK, 0, s>>>(a);
    } else if (corr) {
        sde_fwd_tab_kernel<MODEL, MAXM, true, false><<<grid, BLOCK, 0, s>>>(a);
    } else if (alt) {
        sde_fwd_tab_kernel<MODEL, MAXM, false, true><<<grid, BLOCK, 0, s>>>(a);
    } else {
        sde_fwd_tab_kernel<MODEL, MAXM, false, false><<<grid, BLOCK, 0, s>>>(a);
    }
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
    int best = 1 << 30;
    const void *ks[] = {(const void *)sde_fwd_tab_kernel<MODEL, MAXM, true, true>,
                        (const void *)sde_fwd_tab_kernel<MODEL, MAXM, true, false>,
                        (const void *)sde_fwd_tab_kernel<MODEL, MAXM, false, true>,
                        (const void *)sde_fwd_tab_kernel<MODEL, MAXM, false, false>};
    for (const void *k : ks) {
        int n = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, BLOCK, 0);
        if (n < best) best = n;
    }
    return best;
}
#endif

}  // namespace sdegpu
