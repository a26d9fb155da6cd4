// The FP32 adjoint of a scalar Ornstein-Uhlenbeck group (one state,
// constant parameters, the state output, one checkpoint level): the
// gradient of E[f(X_T)] w.r.t. x0, k, theta and sigma.
//
// It computes what sde_adj_kernel<float, OU, 1> computes -- the same
// checkpoints every `seg` steps, the same recomputed segments and the same
// backward recursion -- with the segment's states and increments in shared
// memory ([seg][2][BLOCK]), each segment's one dt in registers when its
// steps share it (AdjArgs::segdt), and only the model's four slots
// accumulated, as the FP32 Heston kernel (sde_adj_heston.cuh) does for
// Heston.
#pragma once

#include <type_traits>

#include "sde_adjoint.cuh"

namespace sdegpu {

// CK: checkpoints from the forward run (AdjArgs::ckpt)
template <bool CK>
static __global__ void __launch_bounds__(BLOCK, 3) sde_adj_ou_kernel(const __grid_constant__ AdjArgs<float> a) {
    typedef Ar<float> A;
    constexpr int NPA = NGV + 2;
    extern __shared__ float obuf[];   // [seg][2][BLOCK]: x, dW
    __shared__ float red[BLOCK / 32];
    __shared__ float ks[SDE_MAX_STRIKES], kw[SDE_MAX_STRIKES];
    const int g = blockIdx.y;
    const int W = a.W;
    const PhiloxKey key = a.key;
    const uint32_t step_offset = a.step_offset;
    const int seg = a.seg, nseg = a.nseg, n_steps = a.n_steps;
    const float x0 = a.x0[g], kk = a.prm[g], th = a.prm[W + g], sg = a.prm[2 * W + g];
    const float wmean = a.wmean;
    const int n_strikes = a.n_strikes;
#pragma unroll
    for (int i = 0; i < SDE_MAX_STRIKES; ++i)   // constant indices: no parameter address
        if (threadIdx.x == i) {
            ks[i] = a.strikes[i];
            kw[i] = a.weights[i];
        }
    __syncthreads();

    // Kahan sums of the slots x0, k, theta, sigma and the value
    float acc[5], cmp[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) acc[i] = cmp[i] = 0.f;
    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    for (int64_t p = (int64_t)blockIdx.x * BLOCK + threadIdx.x; p < a.paths; p += stride) {
        const PathPre<1> pre(key, (uint32_t)p + a.path_offset, (uint32_t)g, a.stream);
        PairedSteps<float, 1> pair;
        // steps [k0, k1) from x (fwd_step<float, OU, 1>); BUF: each step's
        // state and increment to the segment buffer
        auto sweep = [&](int k0, int k1, float &x, auto BUF, auto DT, auto SQ) {
            for (int k = k0; k < k1; ++k) {
                float z;
                uint32_t pw;
                pair.get(key, pre, k, step_offset, z, pw);
                const float dW = A::mul(z, SQ(k));
                if constexpr (decltype(BUF)::value) {
                    float *b = obuf + (k - k0) * 2 * BLOCK + threadIdx.x;
                    b[0] = x;
                    b[BLOCK] = dW;
                }
                const float drift = A::mul(kk, A::sub(th, x));
                x = A::add(x, A::add(A::mul(drift, DT(k)), A::mul(sg, dW)));
            }
        };
        // f(DT, SQ) for segment s: its one dt as constants, else the tables
        auto with_dt = [&](int s, auto &&f) {
            const float2 ds = __ldg(reinterpret_cast<const float2 *>(a.segdt) + s);
            if (ds.x == ds.x) f([=](int) { return ds.x; }, [=](int) { return ds.y; });
            else f([&](int k) { return __ldg(a.dt + k); }, [&](int k) { return __ldg(a.sqdt + k); });
        };
        float ck[ADJ_MAXSEG];
        float val = 0.f, xb = 0.f;
        auto terminal = [&](float x) {
            val = wmean * x;
            float d = wmean;
            for (int s = 0; s < n_strikes; ++s) {
                val += kw[s] * fmaxf(x - ks[s], 0.f);
                if (x > ks[s]) d += kw[s];
            }
            xb = d;
        };
        if constexpr (!CK) {
            float x = x0;
            for (int s = 0; s < nseg; ++s) {
                ck[s] = x;
                const int k0 = s * seg, k1 = min(k0 + seg, n_steps);
                with_dt(s, [&](auto DT, auto SQ) { sweep(k0, k1, x, std::false_type(), DT, SQ); });
            }
            terminal(x);
        }
        float gk = 0.f, gdt = 0.f, gsg = 0.f;   // gdt: sum of xb dt (times k: the theta slot)
        for (int s = nseg - 1; s >= 0; --s) {
            const int k0 = s * seg, k1 = min(k0 + seg, n_steps);
            float sx = CK ? a.ckpt[((int64_t)s * W + g) * a.paths + p] : ck[s];
            with_dt(s, [&](auto DT, auto SQ) {
                sweep(k0, k1, sx, std::true_type(), DT, SQ);
                if constexpr (CK)
                    if (s == nseg - 1) terminal(sx);
                for (int k = k1 - 1; k >= k0; --k) {
                    const float *b = obuf + (k - k0) * 2 * BLOCK + threadIdx.x;
                    const float x = b[0], dW = b[BLOCK];
                    const float dt = DT(k);
                    const float xbdt = xb * dt;
                    gk = fmaf(xbdt, th - x, gk);
                    gdt += xbdt;
                    gsg = fmaf(xb, dW, gsg);
                    xb = fmaf(-kk * dt, xb, xb);   // xb (1 - k dt)
                }
            });
        }
        kahan_add(acc[0], cmp[0], xb);
        kahan_add(acc[1], cmp[1], gk);
        kahan_add(acc[2], cmp[2], kk * gdt);
        kahan_add(acc[3], cmp[3], gsg);
        kahan_add(acc[4], cmp[4], val);
    }
    // block reduction into sde_adj_kernel's partial layout (one state):
    // slots 0..3, the value at NGV, then a zero
    const int slot[5] = {0, 1, 2, 3, NGV};
    double *dst = a.partials + ((int64_t)g * gridDim.x + blockIdx.x) * NPA;
    if (threadIdx.x < NPA) dst[threadIdx.x] = 0.0;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const float v = block_sum<float>(acc[i] - cmp[i], red);
        if (threadIdx.x == 0) dst[slot[i]] = (double)v;
    }
}

#ifndef __CUDACC_RTC__
// the segment buffer's bytes: 2 floats per step and thread
static inline size_t adj_ou_smem(int seg) { return sizeof(float) * 2 * (size_t)seg * BLOCK; }

static inline void launch_adj_ou(const AdjArgs<float> &a, dim3 grid, cudaStream_t s) {
    const size_t smem = adj_ou_smem(a.seg);
    if (a.ckpt) {
        cudaFuncSetAttribute(sde_adj_ou_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        sde_adj_ou_kernel<true><<<grid, BLOCK, smem, s>>>(a);
    } else {
        cudaFuncSetAttribute(sde_adj_ou_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        sde_adj_ou_kernel<false><<<grid, BLOCK, smem, s>>>(a);
    }
}

static inline int adj_ou_max_blocks_per_sm(int seg) {
    int n = 0, n1 = 0;
    const size_t smem = adj_ou_smem(seg);
    cudaFuncSetAttribute(sde_adj_ou_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(sde_adj_ou_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sde_adj_ou_kernel<false>, BLOCK, smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, sde_adj_ou_kernel<true>, BLOCK, smem);
    return n < n1 ? n : n1;
}
#endif

}  // namespace sdegpu
