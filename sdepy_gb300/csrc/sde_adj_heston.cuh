// The FP32 adjoint of the 2-variable Heston model (constant parameters, no
// jumps, one checkpoint level): the gradient of configs like E[max(S_T - K,
// 0)] w.r.t. x0, mu, sigma, y0, k, theta, xi and rho.
//
// It computes what sde_adj_kernel<float, HESTON, 2> computes -- the same
// checkpoints every `seg` steps, the same recomputed segments and the same
// backward recursion -- with the segment's values in shared memory instead of
// per-thread local arrays, and the step loop written like the forward table
// kernel (sde_tab.cuh): parameters and Philox keys in registers or
// constant-bank operands, no reference to the parameter block handed to a
// helper.  Per step the recomputation stores the variance before the step
// and the two correlated increments (3 floats, [seg][3][BLOCK] so that a
// warp's stores are contiguous), which the backward pass reads back.  Only
// the eight slots the model has are accumulated (Kahan, per thread), then
// reduced per block into sde_adj_kernel's partial layout.
#pragma once

#include <type_traits>

#include "sde_adjoint.cuh"

namespace sdegpu {

// CK: checkpoints from the forward run (AdjArgs::ckpt), compiled apart so
// that the kernel with its own checkpoint sweep carries no test of it
template <bool CK>
static __global__ void __launch_bounds__(BLOCK, 3) sde_adj_heston_kernel(const __grid_constant__ AdjArgs<float> a) {
    typedef Ar<float> A;
    constexpr int NPA = 2 * NGV + 2;
    extern __shared__ float hbuf[];   // [seg][3][BLOCK]: y, z0, z1
    __shared__ float red[BLOCK / 32];
    __shared__ float ks[SDE_MAX_STRIKES], kw[SDE_MAX_STRIKES];
    const int g = blockIdx.y;
    const int W = a.W;
    const PhiloxKey key = a.key;
    const uint32_t step_offset = a.step_offset;
    const int seg = a.seg, nseg = a.nseg, n_steps = a.n_steps;
    // the group's parameters: x (mu, sigma), y (k, theta, xi)
    const float x0a = a.x0[g * 2], x0b = a.x0[g * 2 + 1];
    const float mu = a.prm[g * 2], sg = a.prm[W + g * 2];
    const float kk = a.prm[g * 2 + 1], th = a.prm[W + g * 2 + 1], xi = a.prm[2 * W + g * 2 + 1];
    const float L00 = a.has_corr ? a.chol[0] : 1.f, L10 = a.has_corr ? a.chol[1] : 0.f,
                L11 = a.has_corr ? a.chol[2] : 1.f;
    const bool corr = a.has_corr != 0, rho_grad = a.rho_grad != 0, out_xy = a.out_mode == SDE_OUT_HESTON_XY;
    const float rho_k = a.rho_k, wmean = a.wmean;
    // (z0 + rho_k z1) sqrt(dt) = rw1 dWx + rw2 dWy for dWx = L00 z0 sqrt(dt),
    // dWy = (L10 z0 + L11 z1) sqrt(dt): the rho derivative's increment
    const float rw2 = rho_grad ? rho_k / L11 : 0.f;
    const float rw1 = rho_grad ? (1.f - rw2 * L10) / L00 : 0.f;
    const float hsg2 = -0.5f * sg * sg, nkk = -kk;   // loop constants of the backward step
    const int n_strikes = a.n_strikes;
#pragma unroll
    for (int i = 0; i < SDE_MAX_STRIKES; ++i)   // constant indices: no parameter address
        if (threadIdx.x == i) {
            ks[i] = a.strikes[i];
            kw[i] = a.weights[i];
        }
    __syncthreads();
    auto fval = [&](float X) {
        float v = wmean * X;
        for (int s = 0; s < n_strikes; ++s) v += kw[s] * fmaxf(X - ks[s], 0.f);
        return v;
    };
    auto fder = [&](float X) {
        float d = wmean;
        for (int s = 0; s < n_strikes; ++s)
            if (X > ks[s]) d += kw[s];
        return d;
    };
    // the correlated increments of a step from its normals (correlate()'s
    // operations)
    auto incr = [&](float z0, float z1, float sq, float &dWx, float &dWy) {
        if (corr) {
            dWx = A::mul(A::mul(L00, z0), sq);
            dWy = A::mul(A::add(A::mul(L10, z0), A::mul(L11, z1)), sq);
        } else {
            dWx = z0 * sq;
            dWy = z1 * sq;
        }
    };
    // one Euler step (fwd_step<float, HESTON, 2>)
    auto step = [&](float dt, float dWx, float dWy, float &x, float &y) {
        const float yp = fmaxf(y, 0.f);
        const float sqy = A::sqrt_(yp);
        const float adt = A::sub(mu, A::mul(A::mul(A::mul(sg, sg), yp), 0.5f));
        const float nx = A::add(x, A::add(A::mul(adt, dt), A::mul(A::mul(sg, sqy), dWx)));
        const float bdt = A::mul(kk, A::sub(th, yp));
        const float ny = A::add(y, A::add(A::mul(bdt, dt), A::mul(A::mul(xi, sqy), dWy)));
        x = nx;
        y = ny;
    };

    // Kahan sums of the slots: x0, mu, sigma, rho | y0, k, theta, xi, and the value
    float acc[9], cmp[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) acc[i] = cmp[i] = 0.f;
    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    for (int64_t p = (int64_t)blockIdx.x * BLOCK + threadIdx.x; p < a.paths; p += stride) {
        const PathPre<1> pre(key, (uint32_t)p + a.path_offset, (uint32_t)g, a.stream);
        PairedSteps<float, 2> pair;
        float ck[ADJ_MAXSEG][2];
        float val = 0.f, xbx = 0.f, xby = 0.f;
        // terminal adjoint (HESTON_X: f(exp(x)); HESTON_XY adds f(y))
        auto terminal = [&](float x, float y) {
            const float X = A::exp_(x);
            val = fval(X);
            xbx = fder(X) * X;
            xby = 0.f;
            if (out_xy) {
                val += fval(y);
                xby = fder(y);
            }
        };
        // checkpoints every seg steps: this sweep, or the forward's (device
        // memory; the terminal adjoint then follows the last segment's
        // recomputation)
        constexpr bool fromck = CK;
        // steps [k0, k1) from (x, y), dt and sqrt(dt) from DT(k), SQ(k); BUF:
        // each step's variance and increments to the segment buffer
        auto sweep = [&](int k0, int k1, float &x, float &y, auto BUF, auto DT, auto SQ) {
            for (int k = k0; k < k1; ++k) {
                float z0, z1, dWx, dWy;
                pair.get(key, pre, k, step_offset, z0, z1);
                incr(z0, z1, SQ(k), dWx, dWy);
                if constexpr (decltype(BUF)::value) {
                    float *b = hbuf + (k - k0) * 3 * BLOCK + threadIdx.x;
                    b[0] = y;
                    b[BLOCK] = dWx;
                    b[2 * BLOCK] = dWy;
                }
                step(DT(k), dWx, dWy, x, y);
            }
        };
        // f(DT, SQ) for segment s: its one dt as constants (the usual case),
        // else the per-step tables
        auto with_dt = [&](int s, auto &&f) {
            const float2 ds = __ldg(reinterpret_cast<const float2 *>(a.segdt) + s);
            if (ds.x == ds.x) f([=](int) { return ds.x; }, [=](int) { return ds.y; });
            else f([&](int k) { return __ldg(a.dt + k); }, [&](int k) { return __ldg(a.sqdt + k); });
        };
        if constexpr (!fromck) {
            float x = x0a, y = x0b;
            for (int s = 0; s < nseg; ++s) {
                ck[s][0] = x;
                ck[s][1] = y;
                const int k0 = s * seg, k1 = min(k0 + seg, n_steps);
                with_dt(s, [&](auto DT, auto SQ) { sweep(k0, k1, x, y, std::false_type(), DT, SQ); });
            }
            terminal(x, y);
        }
        float gmu = 0.f, gsg = 0.f, grho = 0.f, gk = 0.f, gth = 0.f, gxi = 0.f;
        for (int s = nseg - 1; s >= 0; --s) {
            const int k0 = s * seg, k1 = min(k0 + seg, n_steps);
            float sx, sy;
            if constexpr (fromck) {
                sx = a.ckpt[((int64_t)s * W + g * 2) * a.paths + p];
                sy = a.ckpt[((int64_t)s * W + g * 2 + 1) * a.paths + p];
            } else {
                sx = ck[s][0];
                sy = ck[s][1];
            }
            with_dt(s, [&](auto DT, auto SQ) { sweep(k0, k1, sx, sy, std::true_type(), DT, SQ); });
            if constexpr (fromck)
                if (s == nseg - 1) terminal(sx, sy);
            with_dt(s, [&](auto DT, auto) {
            for (int k = k1 - 1; k >= k0; --k) {
                const float *b = hbuf + (k - k0) * 3 * BLOCK + threadIdx.x;
                const float yv = b[0], dWx = b[BLOCK], dWy = b[2 * BLOCK];
                const float dt = DT(k);
                const float yp = fmaxf(yv, 0.f);
                const float sr = A::sqrt_(yp);
                const float ab = xbx, ybn = xby;
                const float ys = ybn * sr;
                gmu += ab * dt;
                gsg += ab * (sr * dWx - sg * yp * dt);
                gk += ybn * (th - yp) * dt;
                gth += ybn * dt;   // (times k at the path's end)
                gxi += ys * dWy;
                // (z0 + rho_k z1) sqrt(dt) from the increments
                if (rho_grad) grho += (ys * xi) * fmaf(rw1, dWx, rw2 * dWy);
                float ny = ybn;
                if (yv > 0.f && sr > 0.f) {
                    const float inv = __fdividef(0.5f, sr);   // (approximate: a gradient term)
                    const float dadyp = fmaf(sg * dWx, inv, hsg2 * dt);
                    const float dydyp = fmaf(xi * dWy, inv, nkk * dt);
                    ny = fmaf(ab, dadyp, fmaf(ybn, dydyp, ybn));
                }
                xby = ny;
            }
            });
        }
        gth *= kk;
        kahan_add(acc[0], cmp[0], xbx);
        kahan_add(acc[1], cmp[1], gmu);
        kahan_add(acc[2], cmp[2], gsg);
        kahan_add(acc[3], cmp[3], grho);
        kahan_add(acc[4], cmp[4], xby);
        kahan_add(acc[5], cmp[5], gk);
        kahan_add(acc[6], cmp[6], gth);
        kahan_add(acc[7], cmp[7], gxi);
        kahan_add(acc[8], cmp[8], val);
    }
    // block reduction into sde_adj_kernel's partial layout: slot j of state
    // m at m * NGV + j, the value at 2 * NGV, then a zero
    const int slot[9] = {0, 1, 2, 7, NGV + 0, NGV + 1, NGV + 2, NGV + 3, 2 * NGV};
    double *dst = a.partials + ((int64_t)g * gridDim.x + blockIdx.x) * NPA;
    if (threadIdx.x < NPA) dst[threadIdx.x] = 0.0;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const float v = block_sum<float>(acc[i] - cmp[i], red);
        if (threadIdx.x == 0) dst[slot[i]] = (double)v;
    }
}

#ifndef __CUDACC_RTC__
// the segment buffer's bytes: 3 floats per step and thread
static inline size_t adj_heston_smem(int seg) { return sizeof(float) * 3 * (size_t)seg * BLOCK; }

static inline void launch_adj_heston(const AdjArgs<float> &a, dim3 grid, cudaStream_t s) {
    const size_t smem = adj_heston_smem(a.seg);
    if (a.ckpt) {
        cudaFuncSetAttribute(sde_adj_heston_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        sde_adj_heston_kernel<true><<<grid, BLOCK, smem, s>>>(a);
    } else {
        cudaFuncSetAttribute(sde_adj_heston_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        sde_adj_heston_kernel<false><<<grid, BLOCK, smem, s>>>(a);
    }
}

static inline int adj_heston_max_blocks_per_sm(int seg) {
    int n = 0, n1 = 0;
    const size_t smem = adj_heston_smem(seg);
    cudaFuncSetAttribute(sde_adj_heston_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(sde_adj_heston_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sde_adj_heston_kernel<false>, BLOCK, smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, sde_adj_heston_kernel<true>, BLOCK, smem);
    return n < n1 ? n : n1;
}
#endif

}  // namespace sdegpu
