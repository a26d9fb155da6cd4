// The adjoint of a user SDE whose program is compiled at run time (sdepy's
// integrate decorator, sdepy/integration.py:1843-1955): single equations and
// systems, with any of the dt, dw, dn and dj terms.
//
// The checkpoints and recomputed segments are those of sde_adj_kernel (one
// level of ceil(sqrt(steps)) steps, or two).  What differs:
//  * the backward step is the program's reverse-mode derivative, generated
//    per program (UserJitAdj<R>::back, sde_jit.cu): one value pass of the
//    program and one pass over its instructions in reverse order, instead of
//    a tangent for each of the seven inputs;
//  * each recomputed step leaves the group's states before the step and the
//    step's increments (those of the dw, dn and dj terms the program has) in
//    shared memory, [seg2][NV * MG][BLOCK] values, so the backward pass
//    neither draws nor touches local memory;
//  * the group width MG, the equations, the terms and their sources are
//    compile-time constants: every state index is a register.
// The Euler step is the forward kernel's (the same rounded operations in
// the same order, the same Philox counters), so the recomputed paths are the
// forward's paths bit for bit.
//
// Gradient slots (the partial layout of sde_adj_kernel): slot 0 of state m
// is d/dx0 of that state; slot 1 + j of state h is d/dp_j of the group's
// component h (a system's parameters are shared along its equations: the
// forward kernel reads component h's from state h).  The functional reads
// every state of a single-equation group, and the first equation's
// components of a system (the process a scalar expectation is taken of).
// Integer Poisson counts, intensities and jump-size laws are not
// differentiated.
#pragma once

#include "sde_adjoint.cuh"

namespace sdegpu {

// generated per program (sde_jit.cu): NEQ equations, NT terms, NP
// parameters read, HAS_DW / HAS_DN / HAS_DJ, and back(): the reverse-mode
// step (UserJitFn<R>::src(i) gives the source of term i)
template <typename R>
struct UserJitAdj;

template <typename R, int MAXM, int MG, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) sde_adj_user_kernel(const __grid_constant__ AdjArgs<R> a) {
    typedef Ar<R> A;
    typedef UserJitAdj<R> U;
    constexpr int Q = U::NEQ;
    static_assert(MG % Q == 0, "a system's group holds whole components");
    constexpr int NCP = MG / Q;                  // components of each equation in the group
    constexpr int NP = U::NP;                    // parameters the program reads
    constexpr int NT = U::NT;                    // terms per equation
    constexpr bool DW = U::HAS_DW, DN = U::HAS_DN, DJ = U::HAS_DJ;
    constexpr bool JUMPS = DN || DJ;
    constexpr int IW = 1, IN = 1 + (DW ? 1 : 0), IJ = IN + (DN ? 1 : 0);   // buffer rows of dw, dn, dj
    constexpr int NV = 1 + (DW ? 1 : 0) + (DN ? 1 : 0) + (DJ ? 1 : 0);
    constexpr int NCMAX = NoiseShape<MAXM, JUMPS>::NCMAX;
    constexpr int PP = (MG + 1) >> 1;                          // Box-Muller pairs of a step
    constexpr int NCALL = (2 * PP + (JUMPS ? MG : 0) + 3) >> 2;   // Philox calls of a step
    constexpr int NZ = Paired<MAXM, JUMPS>::NZ;
    constexpr int NF = Q > 1 ? NCP : MG;          // states the functional reads
    constexpr int NS = MG + NCP * NP + 1;        // accumulated slots: x0's, parameters, the value
    constexpr int NPA = MAXM * NGV + 2;
    extern __shared__ unsigned char ub_raw[];
    R *ub = reinterpret_cast<R *>(ub_raw);
    __shared__ R red[BLOCK / 32];

    const int g = blockIdx.y;
    const int W = a.W;
    const PhiloxKey key = a.key;
    const int n_steps = a.n_steps, seg = a.seg, nseg = a.nseg, seg2 = a.seg2;
    const bool two = seg2 < seg;
    R x0[MG], pv[NCP][6];
#pragma unroll
    for (int m = 0; m < MG; ++m) x0[m] = a.x0[g * MG + m];
#pragma unroll
    for (int h = 0; h < NCP; ++h)
#pragma unroll
        for (int j = 0; j < 6; ++j) pv[h][j] = a.prm[j * W + g * MG + h];
    R acc[NS], cmp[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) acc[i] = cmp[i] = R(0);

    // the increment multiplying term i of state m (the forward's user_dz)
    auto dz_of = [&](int i, int m, R dt, const R (&dW)[MAXM], const R (&dN)[MAXM], const R (&dJ)[MAXM]) -> R {
        const int s = UserJitFn<R>::src(i);
        return s == SDE_SRC_DT ? dt : s == SDE_SRC_DW ? dW[m] : s == SDE_SRC_DJ ? dJ[m] : s == SDE_SRC_DN ? dN[m] : R(0);
    };
    // one Euler step of the group, in the forward kernel's order:
    // x + (A_1 dZ_1 + ... + A_n dZ_n) per state
    auto step = [&](int k, const R dt, R (&st)[MG], const R (&dW)[MAXM], const R (&dN)[MAXM], const R (&dJ)[MAXM]) {
        const R t = a.tk[k];
#pragma unroll
        for (int h = 0; h < NCP; ++h) {
            R xs[Q];
#pragma unroll
            for (int e = 0; e < Q; ++e) xs[e] = st[e * NCP + h];
            R A2[Q][SDE_USER_MAX_TERMS];
            UserJitFn<R>::coefs(xs, t, pv[h], A2);
#pragma unroll
            for (int e = 0; e < Q; ++e) {
                const int m = e * NCP + h;
                R s = R(0);
#pragma unroll
                for (int i = 0; i < NT; ++i) {
                    const R term = A::mul(A2[e][i], dz_of(i, m, dt, dW, dN, dJ));
                    s = i == 0 ? term : A::add(s, term);
                }
                st[m] = A::add(xs[e], s);
            }
        }
    };

    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    for (int64_t p = (int64_t)blockIdx.x * BLOCK + threadIdx.x; p < a.paths; p += stride) {
        const uint32_t pc = (uint32_t)p + a.path_offset;   // counter word 0 of this path
        const PathPre<NCMAX> pre(key, pc, (uint32_t)g, a.stream);
        PairedSteps<R, NZ == 0 ? 1 : NZ> pair;
        // a user jump term's increments of state m from Poisson word `word`
        // (the forward kernel's add_jumps)
        auto jumps = [&](int m, uint32_t word, int k, uint32_t c1w, R (&dN)[MAXM], R (&dJ)[MAXM]) {
            const int w = g * MG + m;
            const int64_t tix = (int64_t)k * W + w;
            auto count = [&](uint32_t u) -> int {
                if ((long long)u <= a.thr[tix]) return 0;
                return (long long)u <= a.thr1[tix] ? 1 : poisson_tail(u, a.p0[tix], a.lamdt[tix], a.err);
            };
            int cnt = count(word);
            if constexpr (DJ) {
                if (cnt) {
                    const R ja = a.jprm[w], jb = a.jprm[W + w], jpa = a.jprm[2 * W + w];
                    R S = R(0);
                    for (int j = 0; j < cnt; ++j) {
                        const uint4 r = philox4x32_10(
                            make_uint4(pc, c1w, 0x80000000u | ((uint32_t)w << 12) | (uint32_t)j, a.stream), key);
                        const R y = jump_size<R>(a.jump_law, r, ja, jb, jpa);
                        S = (j == 0) ? y : A::add(S, y);
                    }
                    dJ[m] = S;   // (the forward multiplies by the grid's sign, +1 here)
                }
                if constexpr (DN) cnt = count(philox4x32_10(make_uint4(pc, c1w, 0x40000000u | (uint32_t)w, a.stream), key).x);
            }
            if constexpr (DN)
                if (cnt) dN[m] = (R)cnt;
        };
        // the increments of step k, drawn as the forward kernel draws them
        auto noise = [&](int k, const R sq, R (&dW)[MAXM], R (&dN)[MAXM], R (&dJ)[MAXM]) {
            const uint32_t c1w = (uint32_t)k + a.step_offset;
#pragma unroll
            for (int m = 0; m < MAXM; ++m) dN[m] = dJ[m] = R(0);
            if constexpr (NZ == 1) {
                R z;
                uint32_t pw;
                pair.get(key, pre, k, a.step_offset, z, pw);
                dW[0] = A::mul(z, sq);
                if constexpr (JUMPS) jumps(0, pw, k, c1w, dN, dJ);
            } else if constexpr (NZ == 2) {
                R z[MAXM];
                pair.get(key, pre, k, a.step_offset, z[0], z[1]);
                with_step_chol(a, k, [&](const R *chol) { correlate<R, MAXM>(chol, a.has_corr, z, sq, dW); });
            } else if constexpr (!JUMPS) {
                with_step_chol(a, k, [&](const R *chol) {
                    step_increments<R, MAXM, false>(key, pre, c1w, NCALL, chol, a.has_corr, sq, dW);
                });
            } else {
                uint32_t u[4 * NCMAX];
                step_words<MAXM, JUMPS>(key, pre, c1w, NCALL, u);
                R z[MAXM];
                words_to_normals<R, MAXM, 4 * NCMAX, false>(u, z);
                with_step_chol(a, k, [&](const R *chol) { correlate<R, MAXM>(chol, a.has_corr, z, sq, dW); });
#pragma unroll
                for (int m = 0; m < MG; ++m) jumps(m, pick_word(u, 2 * PP + m), k, c1w, dN, dJ);
            }
        };
        // steps [k0, k1) from state st, with level-2 checkpoints every seg2
        // steps when ck2 is given
        auto sweep = [&](int k0, int k1, R (&st)[MG], R (*ck2)[MG], auto DT, auto SQ) {
            for (int k = k0, kc = 0, ci = 0; k < k1; ++k) {
                if (ck2 && kc == 0) {
#pragma unroll
                    for (int m = 0; m < MG; ++m) ck2[ci][m] = st[m];
                    ++ci;
                }
                kc = kc + 1 == seg2 ? 0 : kc + 1;
                R dW[MAXM], dN[MAXM], dJ[MAXM];
                noise(k, SQ(k), dW, dN, dJ);
                step(k, DT(k), st, dW, dN, dJ);
            }
        };
        // f(DT, SQ) for level-1 segment s1: its one dt as constants (the
        // usual case), else the per-step tables
        auto with_dt = [&](int s1, auto &&f) {
            const R d = a.segdt[2 * s1], q = a.segdt[2 * s1 + 1];
            if (d == d) f([=](int) { return d; }, [=](int) { return q; });
            else f([&](int k) { return a.dt[k]; }, [&](int k) { return a.sqdt[k]; });
        };

        // ---- terminal adjoint of the final states st ---------------------------
        R xb[MG], val = R(0);
        R st[MG];
        auto terminal = [&]() {
            const bool ex = a.out_mode == SDE_OUT_EXP;
            val = R(0);
#pragma unroll
            for (int m = 0; m < MG; ++m) {
                xb[m] = R(0);
                if (m < NF) {
                    const R X = ex ? A::exp_(st[m]) : st[m];
                    val += f_value(a, X);
                    xb[m] = ex ? f_prime(a, X) * X : f_prime(a, X);
                }
            }
        };
        // ---- level-1 checkpoints every seg steps: this forward sweep, or the
        // forward run's (device memory; the terminal adjoint then follows the
        // recomputation of the last steps) ------------------------------------
        R ck[ADJ_MAXSEG][MG];
        const bool fromck = a.ckpt != nullptr;
        auto ck_load = [&](int s1) {
#pragma unroll
            for (int m = 0; m < MG; ++m)
                st[m] = fromck ? a.ckpt[((int64_t)s1 * W + g * MG + m) * a.paths + p] : ck[s1][m];
        };
        if (!fromck) {
#pragma unroll
            for (int m = 0; m < MG; ++m) st[m] = x0[m];
            for (int s1 = 0; s1 < nseg; ++s1) {
#pragma unroll
                for (int m = 0; m < MG; ++m) ck[s1][m] = st[m];
                const int l0 = s1 * seg, l1 = min(l0 + seg, n_steps);
                with_dt(s1, [&](auto DT, auto SQ) { sweep(l0, l1, st, (R(*)[MG]) nullptr, DT, SQ); });
            }
            terminal();
        }
        R gp[NCP][NP > 0 ? NP : 1];
#pragma unroll
        for (int h = 0; h < NCP; ++h)
#pragma unroll
            for (int j = 0; j < (NP > 0 ? NP : 1); ++j) gp[h][j] = R(0);
        // ---- segments from the last: recompute into the buffer, then reverse ----
        R ck2[ADJ_MAXSEG][MG];
        for (int s1 = nseg - 1; s1 >= 0; --s1) {
            const int l0 = s1 * seg, l1 = min(l0 + seg, n_steps);
            if (two) {
                ck_load(s1);
                with_dt(s1, [&](auto DT, auto SQ) { sweep(l0, l1, st, ck2, DT, SQ); });
                if (fromck && s1 == nseg - 1) terminal();
            }
            const int nseg2 = two ? (l1 - l0 + seg2 - 1) / seg2 : 1;
            for (int s2 = nseg2 - 1; s2 >= 0; --s2) {
                const int k0 = two ? l0 + s2 * seg2 : l0;
                const int k1 = two ? min(k0 + seg2, l1) : l1;
                if (two) {
#pragma unroll
                    for (int m = 0; m < MG; ++m) st[m] = ck2[s2][m];
                } else {
                    ck_load(s1);
                }
                with_dt(s1, [&](auto DT, auto SQ) {
                for (int k = k0; k < k1; ++k) {
                    R dW[MAXM], dN[MAXM], dJ[MAXM];
                    noise(k, SQ(k), dW, dN, dJ);
                    R *b = ub + (size_t)(k - k0) * NV * MG * BLOCK + threadIdx.x;
#pragma unroll
                    for (int m = 0; m < MG; ++m) {
                        b[m * BLOCK] = st[m];
                        if constexpr (DW) b[(IW * MG + m) * BLOCK] = dW[m];
                        if constexpr (DN) b[(IN * MG + m) * BLOCK] = dN[m];
                        if constexpr (DJ) b[(IJ * MG + m) * BLOCK] = dJ[m];
                    }
                    step(k, DT(k), st, dW, dN, dJ);
                }
                if (fromck && !two && s1 == nseg - 1) terminal();
                for (int k = k1 - 1; k >= k0; --k) {
                    const R *b = ub + (size_t)(k - k0) * NV * MG * BLOCK + threadIdx.x;
                    R xv[MG], dW[MAXM], dN[MAXM], dJ[MAXM];
#pragma unroll
                    for (int m = 0; m < MAXM; ++m) dW[m] = dN[m] = dJ[m] = R(0);
#pragma unroll
                    for (int m = 0; m < MG; ++m) {
                        xv[m] = b[m * BLOCK];
                        if constexpr (DW) dW[m] = b[(IW * MG + m) * BLOCK];
                        if constexpr (DN) dN[m] = b[(IN * MG + m) * BLOCK];
                        if constexpr (DJ) dJ[m] = b[(IJ * MG + m) * BLOCK];
                    }
                    const R t = a.tk[k], dt = DT(k);
#pragma unroll
                    for (int h = 0; h < NCP; ++h) {
                        R xs[Q], xbv[Q], dz[Q][SDE_USER_MAX_TERMS];
#pragma unroll
                        for (int e = 0; e < Q; ++e) {
                            const int m = e * NCP + h;
                            xs[e] = xv[m];
                            xbv[e] = xb[m];
#pragma unroll
                            for (int i = 0; i < SDE_USER_MAX_TERMS; ++i)
                                dz[e][i] = i < NT ? dz_of(i, m, dt, dW, dN, dJ) : R(0);
                        }
                        R pb[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};
                        U::back(xs, t, pv[h], dz, xbv, pb);
#pragma unroll
                        for (int e = 0; e < Q; ++e) xb[e * NCP + h] = xbv[e];
#pragma unroll
                        for (int j = 0; j < NP; ++j) gp[h][j] += pb[j];
                    }
                }
                });
            }
        }
        // ---- this path's contributions -------------------------------------------
#pragma unroll
        for (int m = 0; m < MG; ++m) kahan_add(acc[m], cmp[m], xb[m]);
#pragma unroll
        for (int h = 0; h < NCP; ++h)
#pragma unroll
            for (int j = 0; j < NP; ++j) kahan_add(acc[MG + h * NP + j], cmp[MG + h * NP + j], gp[h][j]);
        kahan_add(acc[NS - 1], cmp[NS - 1], val);
    }
    // ---- block reduction into sde_adj_kernel's partial layout ---------------------
    double *dst = a.partials + ((int64_t)g * gridDim.x + blockIdx.x) * NPA;
    for (int i = threadIdx.x; i < NPA; i += BLOCK) dst[i] = 0.0;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NS; ++i) {
        const R v = block_sum<R>(acc[i] - cmp[i], red);
        const int slot = i < MG ? i * NGV : i < NS - 1 ? ((i - MG) / (NP > 0 ? NP : 1)) * NGV + 1 + (i - MG) % (NP > 0 ? NP : 1)
                                                        : MAXM * NGV;
        if (threadIdx.x == 0) dst[slot] = (double)v;
    }
}

}  // namespace sdegpu
