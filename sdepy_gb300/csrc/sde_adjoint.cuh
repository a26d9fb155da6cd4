// Adjoint (reverse-mode) kernel of the Euler recursion: pathwise gradients
// of L = sum_o mean_paths f(X_o(T)),  f(X) = w0*X + sum_s w_s max(X - K_s, 0),
// with respect to the initial state and the SDE coefficients of every state
// variable (and rho for a 2-variable Heston group).
//
// * LINEAR models (wiener, lognorm, jump-diffusions): dx'/dx = 1, so the
//   adjoint is constant along the path and one forward sweep accumulating
//   sum dt, sum dW and the jump-size derivatives gives the exact gradient.
// * OU, CIR, Heston and user SDEs: the path is swept forward once storing the state every
//   `seg` steps (checkpoints, seg ~ sqrt(N)); then, segment by segment from
//   the last, the segment's states and increments are recomputed from their
//   Philox counters and the adjoint is propagated backwards through it.
//   Nothing per step is ever written to global memory.
//
// Integer Poisson counts are not differentiated (their intensity gets no
// gradient); the full-truncation kink of Heston's variance and of CIR
// contributes its one-sided derivative (zero where the state is <= 0).
// User SDEs interpreted on the device (single equations driven by dt /
// dw): the program is run in tangent mode for dA/dx and dA/dp
// (user_coefs_tan); slot 1 + j of a state is the gradient of its parameter
// p_j.  Compiled user programs have their own kernel (sde_adj_user.cuh).
#pragma once
#include "sde_kernels.cuh"

namespace sdegpu {

constexpr int NGV = 8;          // gradient slots per state variable
constexpr int ADJ_MAXSEG = 64;  // checkpoints and steps per segment
// the per-step gradient table of the kernels with time-dependent
// parameters lives in shared memory: at most this many bytes per block
// (steps x 3 x group width x sizeof(R)), and the SM's share for the table
constexpr size_t ADJ_TD_SMEM = 160 * 1024;
constexpr size_t ADJ_TD_SMEM_SM = 220 * 1024;
// steps per segment of the FP32 Heston adjoint that keep three 256-thread
// blocks per SM (3 floats per step and thread in shared memory)
constexpr int ADJ_HESTON_SEG = 24;
// the same for the scalar FP32 OU adjoint (2 floats per step and thread)
constexpr int ADJ_OU_SEG = 32;
// shared-memory bytes per block for the segment buffer of the compiled
// user-SDE adjoint (sde_adj_user.cuh)
constexpr size_t UADJ_SMEM = 96 * 1024;

template <typename R>
struct AdjArgs {
    int64_t paths;
    // checkpoints: level 1 every `seg` steps (nseg of them); within a
    // level-1 segment, level 2 every `seg2` steps (seg2 == seg: one level)
    int32_t groups, M, W, n_steps, seg, nseg, seg2;
    uint32_t step_offset;
    int32_t out_mode, jump_law, has_corr, rho_grad;
    uint64_t seed;
    uint32_t stream;
    uint32_t path_offset;   // added to the path index in counter word 0
    PhiloxKey key;
    const R *dt, *sqdt;
    const double *lamdt, *p0;
    const long long *thr, *thr1;
    const R *x0, *prm;
    R chol[NCHOL];
    R rho_k;  // -rho / sqrt(1 - rho^2) for the rho gradient (2-variable Heston)
    int32_t n_strikes;
    R strikes[SDE_MAX_STRIKES], weights[SDE_MAX_STRIKES];
    R wmean;
    double *partials;  // [groups][gridDim.x][MAXM*NGV + 2]
    int32_t *err;
    // SDE_MODEL_USER: the coefficient program and each step's start time
    SdeUserProgram uprog;
    const R *tk;
    // time-dependent parameters (kernels compiled with TD): slots 0..2 of
    // each step, [n_steps][3][W]; the gradients of those slots, per step,
    // go to tdpart [groups][gridDim.x][n_steps][3][MAXM] instead of the
    // per-variable slots 1..3
    const R *prm_t;
    double *tdpart;
    // a user SDE's jump terms (sde_adj_user_kernel): the jump-size law's a,
    // b, pa per state ([3][W]), and the terms present (bit 0 dj, bit 1 dn)
    const R *jprm;
    int32_t user_jsrc;
    // level-1 checkpoints written by the forward run, [nseg][W][paths], or
    // NULL (the kernel's own checkpoint sweep)
    const R *ckpt;
    // time-dependent correlation: [steps][NCHOL] packed Cholesky factors of
    // each step's correlation matrix, or NULL (chol applies throughout)
    const R *chol_t;
    // [nseg][2]: a level-1 segment's dt and sqrt(dt) when all its steps
    // share them, else NaN (read by the FP32 Heston kernel)
    const R *segdt;
};

// f(the Cholesky factor of step k): the per-step table's row (uniform
// test), else the constant factor of the parameter block -- two copies of
// f, so that the constant one keeps its constant-bank loads
template <typename R, typename F>
__device__ __forceinline__ void with_step_chol(const AdjArgs<R> &a, int k, F &&f) {
    if (a.chol_t) f(a.chol_t + (int64_t)k * NCHOL);
    else f(a.chol);
}

// Tangent-mode run of a user program (single equation): the terms' values
// A[i] and their derivatives dA[i][0] = dA_i/dx, dA[i][1 + j] = dA_i/dp_j.
// Derivative rules per instruction (d = the operands' tangents): sums and
// products by the chain rule; abs, maximum and minimum take the selected
// branch (maximum(x, 0) has derivative 0 where x < 0); sqrt has derivative 0
// at 0 (the one-sided value of the truncated models); a ** b adds the b
// term v log a only where a > 0.
constexpr int UTAN = 7;

// the seeds of a tangent-mode run: r0 = x (d/dx = 1), r1 = t, r2..r7 = p
// (d/dp_j = 1)
template <typename R>
__device__ __forceinline__ void tan_inputs(R x, R t, const R (&p)[6], R (&r)[SDE_USER_MAX_REGS],
                                           R (&d)[SDE_USER_MAX_REGS][UTAN]) {
    r[0] = x;
    r[1] = t;
#pragma unroll
    for (int i = 0; i < 6; ++i) r[2 + i] = p[i];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < UTAN; ++j) d[i][j] = R(0);
    d[0][0] = R(1);
#pragma unroll
    for (int i = 0; i < 6; ++i) d[2 + i][1 + i] = R(1);
}

// one instruction (not SDE_UOP_CONST) in tangent mode: value and tangents
template <typename R>
__device__ __forceinline__ void tan_op(uint32_t op, R (&r)[SDE_USER_MAX_REGS], R (&d)[SDE_USER_MAX_REGS][UTAN]) {
    typedef Ar<R> Ao;
    typedef UFn<R> F;
    const int dst = (op >> 8) & 0xff, ia = (op >> 16) & 0xff, ib = op >> 24;
    const int code = op & 0xff;
    const R va = r[ia], vb = r[ib];
    R v, da = R(0), db = R(0);   // the result and its partials in a and b
    switch (code) {
    case SDE_UOP_ADD: v = Ao::add(va, vb); da = R(1); db = R(1); break;
    case SDE_UOP_SUB: v = Ao::sub(va, vb); da = R(1); db = R(-1); break;
    case SDE_UOP_MUL: v = Ao::mul(va, vb); da = vb; db = va; break;
    case SDE_UOP_DIV: v = va / vb; da = R(1) / vb; db = -v / vb; break;
    case SDE_UOP_NEG: v = -va; da = R(-1); break;
    case SDE_UOP_ABS: v = fabs(va); da = va < R(0) ? R(-1) : R(1); break;
    case SDE_UOP_EXP: v = F::exp_(va); da = v; break;
    case SDE_UOP_LOG: v = F::log_(va); da = R(1) / va; break;
    case SDE_UOP_SQRT: v = Ao::sqrt_(va); da = v > R(0) ? R(0.5) / v : R(0); break;
    case SDE_UOP_MAX: v = np_max(va, vb); if (va >= vb) da = R(1); else db = R(1); break;
    case SDE_UOP_MIN: v = np_min(va, vb); if (va <= vb) da = R(1); else db = R(1); break;
    case SDE_UOP_SIN: v = F::sin_(va); da = F::cos_(va); break;
    case SDE_UOP_COS: v = F::cos_(va); da = -F::sin_(va); break;
    case SDE_UOP_TAN: v = F::tan_(va); da = R(1) + v * v; break;
    case SDE_UOP_TANH: v = F::tanh_(va); da = R(1) - v * v; break;
    case SDE_UOP_POW:
        v = F::pow_(va, vb);
        da = vb * F::pow_(va, vb - R(1));
        db = va > R(0) ? v * F::log_(va) : R(0);
        break;
    case SDE_UOP_EXPM1: v = F::expm1_(va); da = v + R(1); break;
    case SDE_UOP_LOG1P: v = F::log1p_(va); da = R(1) / (R(1) + va); break;
    case SDE_UOP_ARCTAN: v = F::atan_(va); da = R(1) / (R(1) + va * va); break;
    default: v = va; da = R(1); break;   // SDE_UOP_COPY
    }
    R nd[UTAN];
#pragma unroll
    for (int j = 0; j < UTAN; ++j) {
        // a zero tangent contributes nothing (no 0 * inf)
        const R ta = d[ia][j], tb = d[ib][j];
        R s = ta != R(0) ? da * ta : R(0);
        if (tb != R(0) && db != R(0)) s = s + db * tb;
        nd[j] = s;
    }
    r[dst] = v;
#pragma unroll
    for (int j = 0; j < UTAN; ++j) d[dst][j] = nd[j];
}

// a constant in tangent mode
template <typename R>
__device__ __forceinline__ void tan_const(int dst, R c, R (&r)[SDE_USER_MAX_REGS], R (&d)[SDE_USER_MAX_REGS][UTAN]) {
    r[dst] = c;
#pragma unroll
    for (int j = 0; j < UTAN; ++j) d[dst][j] = R(0);
}

// the terms' values and tangents from the registers
template <typename R>
__device__ __forceinline__ void tan_outputs(const SdeUserProgram &u, const R (&r)[SDE_USER_MAX_REGS],
                                            const R (&d)[SDE_USER_MAX_REGS][UTAN], R (&A)[SDE_USER_MAX_TERMS],
                                            R (&dA)[SDE_USER_MAX_TERMS][UTAN]) {
#pragma unroll
    for (int i = 0; i < SDE_USER_MAX_TERMS; ++i) {
        const int reg = i < u.n_terms ? u.term_register[0][i] : 0;
        A[i] = i < u.n_terms ? r[reg] : R(0);
#pragma unroll
        for (int j = 0; j < UTAN; ++j) dA[i][j] = i < u.n_terms ? d[reg][j] : R(0);
    }
}

template <typename R>
__device__ __noinline__ void user_coefs_tan(const SdeUserProgram &u, R x, R t, const R (&p)[6],
                                            R (&A)[SDE_USER_MAX_TERMS], R (&dA)[SDE_USER_MAX_TERMS][UTAN]) {
    R r[SDE_USER_MAX_REGS];
    R d[SDE_USER_MAX_REGS][UTAN];
    tan_inputs<R>(x, t, p, r, d);
    for (int i = 0; i < u.n_ops; ++i) {
        const uint32_t op = u.ops[i];
        if ((op & 0xff) == SDE_UOP_CONST) tan_const<R>((op >> 8) & 0xff, (R)u.consts[(op >> 16) & 0xff], r, d);
        else tan_op<R>(op, r, d);
    }
    tan_outputs<R>(u, r, d, A, dA);
}

// one forward Euler step of a user SDE (the forward kernel's arithmetic):
// x + (A_1 dZ_1 + A_2 dZ_2), dZ = dt or dW
template <typename R, int MAXM, int MODEL = SDE_MODEL_USER>
__device__ __forceinline__ void user_step(const SdeUserProgram &u, const R (&c0)[MAXM], const R (&c1)[MAXM],
                                          const R (&c2)[MAXM], const R (&c3)[MAXM], const R (&c4)[MAXM],
                                          const R (&c5)[MAXM], R t, R dt, const R (&dW)[MAXM], R (&st)[MAXM]) {
    typedef Ar<R> A;
#pragma unroll
    for (int m = 0; m < MAXM; ++m) {
        const R pv[6] = {c0[m], c1[m], c2[m], c3[m], c4[m], c5[m]};
        R A2[1][SDE_USER_MAX_TERMS];
        const R xm[1] = {st[m]};
        user_eval<R, MODEL>(u, xm, t, pv, A2);
        R s = R(0);
        for (int i = 0; i < u.n_terms; ++i) {
            const R term = A::mul(A2[0][i], u.term_source[i] == SDE_SRC_DT ? dt : dW[m]);
            s = i == 0 ? term : A::add(s, term);
        }
        st[m] = A::add(st[m], s);
    }
}

template <typename R>
__device__ __forceinline__ R f_value(const AdjArgs<R> &a, R X) {
    R v = a.wmean * X;
    for (int s = 0; s < a.n_strikes; ++s) v += a.weights[s] * fmax(X - a.strikes[s], R(0));
    return v;
}
template <typename R>
__device__ __forceinline__ R f_prime(const AdjArgs<R> &a, R X) {
    R d = a.wmean;
    for (int s = 0; s < a.n_strikes; ++s)
        if (X > a.strikes[s]) d += a.weights[s];
    return d;
}

template <typename R>
__device__ __forceinline__ void kahan_add(R &s, R &c, R v) {
    const R y = v - c;
    const R t = s + y;
    c = (t - s) - y;
    s = t;
}

// terminal adjoint of the states from the functional of the outputs;
// returns the functional's value for this path
template <typename R, int MAXM>
__device__ __forceinline__ R terminal_adjoint(const AdjArgs<R> &a, const R (&st)[MAXM], R (&xb)[MAXM]) {
    const int M = a.M;
    R val = R(0);
#pragma unroll
    for (int m = 0; m < MAXM; ++m) xb[m] = R(0);
    switch (a.out_mode) {
    case SDE_OUT_EXP:
#pragma unroll
        for (int m = 0; m < MAXM; ++m)
            if (m < M) {
                const R X = Ar<R>::exp_(st[m]);
                val += f_value(a, X);
                xb[m] = f_prime(a, X) * X;
            }
        break;
    case SDE_OUT_SUM: {
        R X = st[0];
#pragma unroll
        for (int m = 1; m < MAXM; ++m)
            if (m < M) X = X + st[m];
        val = f_value(a, X);
        const R d = f_prime(a, X);
#pragma unroll
        for (int m = 0; m < MAXM; ++m)
            if (m < M) xb[m] = d;
        break;
    }
    case SDE_OUT_HESTON_X:
    case SDE_OUT_HESTON_XY:
#pragma unroll
        for (int m = 0; m < MAXM / 2; ++m) {
            const R X = Ar<R>::exp_(st[m]);
            val += f_value(a, X);
            xb[m] = f_prime(a, X) * X;
        }
        if (a.out_mode == SDE_OUT_HESTON_XY) {
#pragma unroll
            for (int m = MAXM / 2; m < MAXM; ++m) {
                val += f_value(a, st[m]);
                xb[m] = f_prime(a, st[m]);
            }
        }
        break;
    default:
#pragma unroll
        for (int m = 0; m < MAXM; ++m)
            if (m < M) {
                val += f_value(a, st[m]);
                xb[m] = f_prime(a, st[m]);
            }
    }
    return val;
}

// one forward Euler step of the OU / CIR / Heston models (same arithmetic as
// the forward kernel); z: uncorrelated normals, dW: correlated increments
template <typename R, int MODEL, int MAXM>
__device__ __forceinline__ void fwd_step(const R (&c0)[MAXM], const R (&c1)[MAXM], const R (&c2)[MAXM],
                                         R dt, const R (&dW)[MAXM], R (&st)[MAXM]) {
    typedef Ar<R> A;
    if (MODEL == SDE_MODEL_OU) {
#pragma unroll
        for (int m = 0; m < MAXM; ++m) {
            const R drift = A::mul(c0[m], A::sub(c1[m], st[m]));
            st[m] = A::add(st[m], A::add(A::mul(drift, dt), A::mul(c2[m], dW[m])));
        }
    } else if (MODEL == SDE_MODEL_CIR) {
#pragma unroll
        for (int m = 0; m < MAXM; ++m) {
            const R xp = fmax(st[m], R(0));
            const R drift = A::mul(c0[m], A::sub(c1[m], xp));
            const R vol = A::mul(c2[m], A::sqrt_(xp));
            st[m] = A::add(st[m], A::add(A::mul(drift, dt), A::mul(vol, dW[m])));
        }
    } else {
        constexpr int h = MAXM / 2;
        R nx[MAXM];
#pragma unroll
        for (int i = 0; i < h; ++i) {
            const R y = st[h + i];
            const R yp = fmax(y, R(0));
            const R sqy = A::sqrt_(yp);
            const R adt = A::sub(c0[i], A::mul(A::mul(A::mul(c1[i], c1[i]), yp), R(0.5)));
            nx[i] = A::add(st[i], A::add(A::mul(adt, dt), A::mul(A::mul(c1[i], sqy), dW[i])));
            const R bdt = A::mul(c0[h + i], A::sub(c1[h + i], yp));
            nx[h + i] = A::add(y, A::add(A::mul(bdt, dt), A::mul(A::mul(c2[h + i], sqy), dW[h + i])));
        }
#pragma unroll
        for (int m = 0; m < MAXM; ++m) st[m] = nx[m];
    }
}

// FP32 kernels of one or two states are held to 80 registers: 3 resident
// blocks per SM (measured 2.4 % faster for Heston than 2 blocks at 90)
// TD: time-dependent parameter slots 0..2 (AdjArgs::prm_t), reloaded at every
// step of every sweep, with per-step gradients: each warp sums a step's
// contributions over its paths and adds them to a block table in shared
// memory (n_steps * 3 * MAXM values of R), written out at the block's end.
// Every lane of a warp walks a path in every round (the last round's spare
// lanes contribute zero), so the warp sums see whole warps.
template <typename R, int MODEL, int MAXM, bool JUMPS, bool TD = false>
__global__ void __launch_bounds__(BLOCK, (sizeof(R) == 4 && MAXM <= 2) ? 3 : 1)
sde_adj_kernel(const __grid_constant__ AdjArgs<R> a) {
    // a user SDE interpreted on the device
    constexpr bool UJ = MODEL == SDE_MODEL_USER;
    typedef Ar<R> A;
    constexpr int NCMAX = NoiseShape<MAXM, JUMPS>::NCMAX;
    constexpr int NPA = MAXM * NGV + 2;
    __shared__ R red[BLOCK / 32];

    const int g = blockIdx.y;
    const int M = a.M;
    const int W = a.W;
    const int P = (M + 1) >> 1;
    const int NC = (2 * P + (JUMPS ? M : 0) + 3) >> 2;
    const PhiloxKey key = a.key;  // by value: uniform registers, not indexed parameter loads

    R x0[MAXM], c0[MAXM], c1[MAXM], c2[MAXM], c3[MAXM], c4[MAXM], c5[MAXM];
#pragma unroll
    for (int m = 0; m < MAXM; ++m) {
        const int w = g * M + (m < M ? m : 0);
        x0[m] = a.x0[w];
        c0[m] = a.prm[0 * W + w];
        c1[m] = a.prm[1 * W + w];
        c2[m] = a.prm[2 * W + w];
        c3[m] = a.prm[3 * W + w];
        c4[m] = a.prm[4 * W + w];
        c5[m] = a.prm[5 * W + w];
    }
    // per-thread Kahan accumulators of the gradient slots and the value
    R acc[NPA], cmp[NPA];
#pragma unroll
    for (int i = 0; i < NPA; ++i) acc[i] = cmp[i] = R(0);
    extern __shared__ unsigned char td_raw[];
    R *tdtab = reinterpret_cast<R *>(td_raw);
    const int ntd = TD ? a.n_steps * 3 * MAXM : 0;
    if constexpr (TD) {
        for (int i = threadIdx.x; i < ntd; i += BLOCK) tdtab[i] = R(0);
        __syncthreads();
    }
    // a step's coefficients (TD): slots 0..2 from the table
    auto load_step = [&](int k) {
        if constexpr (TD) {
            const R *pk = a.prm_t + (int64_t)k * 3 * W;
#pragma unroll
            for (int m = 0; m < MAXM; ++m) {
                const int w = g * M + (m < M ? m : 0);
                c0[m] = pk[w];
                c1[m] = pk[W + w];
                c2[m] = pk[2 * W + w];
            }
        }
    };

    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    const int64_t rounds = (a.paths + stride - 1) / stride;
    for (int64_t rd = 0; rd < rounds; ++rd) {
        const int64_t pr = rd * stride + (int64_t)blockIdx.x * BLOCK + threadIdx.x;
        const bool act = pr < a.paths;
        if (!TD && !act) continue;   // TD: spare lanes walk path 0 and contribute zero
        const int64_t p = act ? pr : 0;
        // d L / d (slot j of state m at step k) += v
        auto addp = [&](int k, int m, int j, R v) {
            if constexpr (TD) {
                v = warp_sum<R>(act ? v : R(0));
                if ((threadIdx.x & 31) == 0) atomicAdd(&tdtab[(k * 3 + j) * MAXM + m], v);
            }
        };
        R gr[MAXM][NGV];
#pragma unroll
        for (int m = 0; m < MAXM; ++m)
#pragma unroll
            for (int j = 0; j < NGV; ++j) gr[m][j] = R(0);
        const uint32_t pc = (uint32_t)p + a.path_offset;   // counter word 0 of this path
        const PathPre<NCMAX> pre(key, pc, (uint32_t)g, a.stream);
        constexpr int NZ = Paired<MAXM, JUMPS>::NZ;
        PairedSteps<R, NZ == 0 ? 1 : NZ> pair;   // groups of one or two variables
        // the words, normals and increments of step k, exactly as the
        // forward kernel draws them
        auto noise = [&](int k, R sq, uint32_t (&u)[4 * NCMAX], R (&z)[MAXM], R (&dW)[MAXM]) {
            if constexpr (NZ == 1) {
                uint32_t pw;
                pair.get(key, pre, k, a.step_offset, z[0], pw);
                u[0] = u[1] = u[3] = 0u;
                u[2] = pw;   // the Poisson word, index 2P + m with P = 1, m = 0
            } else if constexpr (NZ == 2) {
                pair.get(key, pre, k, a.step_offset, z[0], z[1]);
                for (int i = 0; i < 4 * NCMAX; ++i) u[i] = 0u;
            } else {
                step_words<MAXM, JUMPS>(key, pre, (uint32_t)k + a.step_offset, NC, u);
                words_to_normals<R, MAXM>(u, z);
            }
            with_step_chol(a, k, [&](const R *chol) { correlate<R, MAXM>(chol, a.has_corr, z, sq, dW); });
        };
        R val = R(0);
        if (MODEL == SDE_MODEL_LINEAR) {
            // ---- constant adjoint: one forward sweep ------------------------------
            R st[MAXM], sdw[MAXM], sja[MAXM], sjb[MAXM];
            R sdt = R(0);
#pragma unroll
            for (int m = 0; m < MAXM; ++m) { st[m] = x0[m]; sdw[m] = sja[m] = sjb[m] = R(0); }
            for (int k = 0; k < a.n_steps; ++k) {
                const R dt = a.dt[k], sq = a.sqdt[k];
                const uint32_t c1w = (uint32_t)k + a.step_offset;
                uint32_t u[4 * NCMAX];
                R z[MAXM], dW[MAXM];
                noise(k, sq, u, z, dW);
                load_step(k);
                sdt = sdt + dt;
#pragma unroll
                for (int m = 0; m < MAXM; ++m) {
                    R inc = A::add(A::mul(c0[m], dt), A::mul(c1[m], dW[m]));
                    sdw[m] = sdw[m] + dW[m];
                    if (JUMPS && m < M) {
                        const uint32_t word = pick_word(u, 2 * P + m);
                        const int w = g * M + m;
                        const int64_t tix = (int64_t)k * W + w;
                        if ((long long)word > a.thr[tix]) {
                            const int cnt = (long long)word <= a.thr1[tix]
                                                ? 1 : poisson_tail(word, a.p0[tix], a.lamdt[tix], a.err);
                            R S = R(0);
                            for (int j = 0; j < cnt; ++j) {
                                const uint4 r = philox4x32_10(
                                    make_uint4(pc, c1w, 0x80000000u | ((uint32_t)w << 12) | (uint32_t)j,
                                               a.stream), key);
                                const R y = jump_size<R>(a.jump_law, r, c3[m], c4[m], c5[m]);
                                R da, db;
                                jump_size_grad<R>(a.jump_law, r, c3[m], c4[m], c5[m], da, db);
                                sja[m] = sja[m] + da;
                                sjb[m] = sjb[m] + db;
                                S = (j == 0) ? y : A::add(S, y);
                            }
                            inc = A::add(inc, S);
                        }
                    }
                    st[m] = A::add(st[m], inc);
                }
            }
            R xb[MAXM];
            val = terminal_adjoint<R, MAXM>(a, st, xb);
#pragma unroll
            for (int m = 0; m < MAXM; ++m) {
                gr[m][0] = xb[m];
                gr[m][1] = xb[m] * sdt;
                gr[m][2] = xb[m] * sdw[m];
                gr[m][4] = xb[m] * sja[m];
                gr[m][5] = xb[m] * sjb[m];
            }
            if constexpr (TD) {
                // the constant adjoint xb times each step's dt and dW: the
                // increments are drawn again (the kernels with TD take no jumps)
                for (int k = 0; k < a.n_steps; ++k) {
                    const R dt = a.dt[k], sq = a.sqdt[k];
                    uint32_t u[4 * NCMAX];
                    R z[MAXM], dW[MAXM];
                    noise(k, sq, u, z, dW);
#pragma unroll
                    for (int m = 0; m < MAXM; ++m) {
                        addp(k, m, 0, xb[m] * dt);
                        addp(k, m, 1, xb[m] * dW[m]);
                    }
                }
            }
        } else {
            // ---- checkpointed reverse sweep (OU, Heston) ----------------------------
            R ck[ADJ_MAXSEG][MAXM];
            R st[MAXM];
            R xb[MAXM];
            // level-1 checkpoints: this sweep, or the forward's (device
            // memory; the terminal adjoint then follows the recomputation
            // of the last steps)
            const bool fromck = a.ckpt != nullptr;
            auto ck_load = [&](int s1) {
#pragma unroll
                for (int m = 0; m < MAXM; ++m)
                    st[m] = fromck ? a.ckpt[((int64_t)s1 * W + g * M + (m < M ? m : 0)) * a.paths + p] : ck[s1][m];
            };
            if (!fromck) {
#pragma unroll
                for (int m = 0; m < MAXM; ++m) st[m] = x0[m];
                for (int k = 0; k < a.n_steps; ++k) {
                    if (k % a.seg == 0) {
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) ck[k / a.seg][m] = st[m];
                    }
                    const R sq = a.sqdt[k];
                    uint32_t u[4 * NCMAX];
                    R z[MAXM], dW[MAXM];
                    noise(k, sq, u, z, dW);
                    load_step(k);
                    if constexpr (UJ) user_step<R, MAXM, MODEL>(a.uprog, c0, c1, c2, c3, c4, c5, a.tk[k], a.dt[k], dW, st);
                    else fwd_step<R, MODEL, MAXM>(c0, c1, c2, a.dt[k], dW, st);
                }
                val = terminal_adjoint<R, MAXM>(a, st, xb);
            }
            R bx[ADJ_MAXSEG][MAXM], bw[ADJ_MAXSEG][MAXM], bz[ADJ_MAXSEG][2];
            // level-2 checkpoints of the current level-1 segment (two levels
            // only: runs longer than ADJ_MAXSEG^2 steps)
            R ck2[ADJ_MAXSEG][MAXM];
            const bool two = a.seg2 < a.seg;
            for (int s1 = a.nseg - 1; s1 >= 0; --s1) {
              const int l0 = s1 * a.seg;
              const int l1 = min(l0 + a.seg, a.n_steps);
              if (two) {
                  ck_load(s1);
                  for (int k = l0; k < l1; ++k) {
                      if ((k - l0) % a.seg2 == 0) {
#pragma unroll
                          for (int m = 0; m < MAXM; ++m) ck2[(k - l0) / a.seg2][m] = st[m];
                      }
                      const R sq = a.sqdt[k];
                      uint32_t u[4 * NCMAX];
                      R z[MAXM], dW[MAXM];
                      noise(k, sq, u, z, dW);
                      load_step(k);
                      if constexpr (UJ) user_step<R, MAXM, MODEL>(a.uprog, c0, c1, c2, c3, c4, c5, a.tk[k], a.dt[k], dW, st);
                      else fwd_step<R, MODEL, MAXM>(c0, c1, c2, a.dt[k], dW, st);
                  }
                  if (fromck && s1 == a.nseg - 1) val = terminal_adjoint<R, MAXM>(a, st, xb);
              }
              const int nseg2 = two ? (l1 - l0 + a.seg2 - 1) / a.seg2 : 1;
              for (int sidx = nseg2 - 1; sidx >= 0; --sidx) {
                const int k0 = two ? l0 + sidx * a.seg2 : l0;
                const int k1 = two ? min(k0 + a.seg2, l1) : l1;
                if (two) {
#pragma unroll
                    for (int m = 0; m < MAXM; ++m) st[m] = ck2[sidx][m];
                } else {
                    ck_load(s1);
                }
                for (int k = k0; k < k1; ++k) {
                    const R sq = a.sqdt[k];
                    uint32_t u[4 * NCMAX];
                    R z[MAXM], dW[MAXM];
                    noise(k, sq, u, z, dW);
#pragma unroll
                    for (int m = 0; m < MAXM; ++m) {
                        bx[k - k0][m] = st[m];
                        bw[k - k0][m] = dW[m];
                    }
                    bz[k - k0][0] = z[0];
                    bz[k - k0][1] = MAXM > 1 ? z[MAXM > 1 ? 1 : 0] : R(0);
                    load_step(k);
                    if constexpr (UJ) user_step<R, MAXM, MODEL>(a.uprog, c0, c1, c2, c3, c4, c5, a.tk[k], a.dt[k], dW, st);
                    else fwd_step<R, MODEL, MAXM>(c0, c1, c2, a.dt[k], dW, st);
                }
                if (fromck && !two && s1 == a.nseg - 1) val = terminal_adjoint<R, MAXM>(a, st, xb);
                for (int k = k1 - 1; k >= k0; --k) {
                    const R dt = a.dt[k], sq = a.sqdt[k];
                    load_step(k);
                    if constexpr (UJ) {
                        // x' = x + sum_i A_i(t, x, p) dZ_i: dx'/dx = 1 + sum_i dA_i/dx dZ_i,
                        // dx'/dp_j = sum_i dA_i/dp_j dZ_i
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) {
                            const R pv[6] = {c0[m], c1[m], c2[m], c3[m], c4[m], c5[m]};
                            R Av[SDE_USER_MAX_TERMS], dA[SDE_USER_MAX_TERMS][UTAN];
                            user_coefs_tan<R>(a.uprog, bx[k - k0][m], a.tk[k], pv, Av, dA);
                            R gx = R(0), gp[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};
                            for (int i = 0; i < a.uprog.n_terms; ++i) {
                                const R dz = a.uprog.term_source[i] == SDE_SRC_DT ? dt : bw[k - k0][m];
                                gx += dA[i][0] * dz;
#pragma unroll
                                for (int j = 0; j < 6; ++j) gp[j] += dA[i][1 + j] * dz;
                            }
                            const R xbn = xb[m];
#pragma unroll
                            for (int j = 0; j < 6; ++j) gr[m][1 + j] += xbn * gp[j];
                            xb[m] = xbn * (R(1) + gx);
                        }
                    } else if (MODEL == SDE_MODEL_OU) {
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) {
                            const R x = bx[k - k0][m];
                            const R xbn = xb[m];
                            if constexpr (TD) {
                                addp(k, m, 0, xbn * (c1[m] - x) * dt);
                                addp(k, m, 1, xbn * c0[m] * dt);
                                addp(k, m, 2, xbn * bw[k - k0][m]);
                            } else {
                                gr[m][1] += xbn * (c1[m] - x) * dt;   // k
                                gr[m][2] += xbn * c0[m] * dt;         // theta
                                gr[m][3] += xbn * bw[k - k0][m];      // sigma
                            }
                            xb[m] = xbn * (R(1) - c0[m] * dt);
                        }
                    } else if (MODEL == SDE_MODEL_CIR) {
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) {
                            const R x = bx[k - k0][m];
                            const R xp = fmax(x, R(0));
                            const R s = A::sqrt_(xp);
                            const R xbn = xb[m], dw = bw[k - k0][m];
                            if constexpr (TD) {
                                addp(k, m, 0, xbn * (c1[m] - xp) * dt);
                                addp(k, m, 1, xbn * c0[m] * dt);
                                addp(k, m, 2, xbn * s * dw);
                            } else {
                                gr[m][1] += xbn * (c1[m] - xp) * dt;   // k
                                gr[m][2] += xbn * c0[m] * dt;          // theta
                                gr[m][3] += xbn * s * dw;              // xi
                            }
                            // dx'/dx = 1 + (-k dt + xi dW / (2 sqrt x)) where x > 0
                            R d = R(1);
                            if (x > R(0) && s > R(0)) d = R(1) - c0[m] * dt + c2[m] * dw * (R(0.5) / s);
                            xb[m] = xbn * d;
                        }
                    } else {
                        constexpr int h = MAXM / 2;
#pragma unroll
                        for (int i = 0; i < h; ++i) {
                            const R y = bx[k - k0][h + i];
                            const R yp = fmax(y, R(0));
                            const R s = A::sqrt_(yp);
                            const R ab = xb[i], ybn = xb[h + i];
                            const R mu = c0[i], sg = c1[i];
                            const R kk = c0[h + i], th = c1[h + i], xi = c2[h + i];
                            const R dWx = bw[k - k0][i], dWy = bw[k - k0][h + i];
                            if constexpr (TD) {
                                addp(k, i, 0, ab * dt);
                                addp(k, i, 1, ab * (s * dWx - sg * yp * dt));
                                addp(k, h + i, 0, ybn * (th - yp) * dt);
                                addp(k, h + i, 1, ybn * kk * dt);
                                addp(k, h + i, 2, ybn * s * dWy);
                            } else {
                                gr[i][1] += ab * dt;                              // mu
                                gr[i][2] += ab * (s * dWx - sg * yp * dt);         // sigma
                                gr[h + i][1] += ybn * (th - yp) * dt;              // k
                                gr[h + i][2] += ybn * kk * dt;                     // theta
                                gr[h + i][3] += ybn * s * dWy;                     // xi
                            }
                            if (MAXM == 2 && a.rho_grad) {
                                // dW_y = (rho z0 + sqrt(1 - rho^2) z1) sq
                                const R ddw = (bz[k - k0][0] + a.rho_k * bz[k - k0][1]) * sq;
                                gr[0][7] += ybn * xi * s * ddw;
                            }
                            R ny = ybn;
                            if (y > R(0) && s > R(0)) {
                                const R inv = R(0.5) / s;
                                const R dadyp = -sg * sg * dt * R(0.5) + sg * dWx * inv;
                                const R dydyp = -kk * dt + xi * dWy * inv;
                                ny = ybn + ab * dadyp + ybn * dydyp;
                            }
                            xb[h + i] = ny;
                        }
                    }
                }
              }
            }
#pragma unroll
            for (int m = 0; m < MAXM; ++m) gr[m][0] = xb[m];
        }
        // accumulate this path
        if (act) {
#pragma unroll
            for (int m = 0; m < MAXM; ++m)
#pragma unroll
                for (int j = 0; j < NGV; ++j) kahan_add(acc[m * NGV + j], cmp[m * NGV + j], gr[m][j]);
            kahan_add(acc[MAXM * NGV], cmp[MAXM * NGV], val);
        }
    }
    // block reduction, FP64 partial per block
#pragma unroll
    for (int i = 0; i < NPA - 1; ++i) {
        const R s = block_sum<R>(acc[i] - cmp[i], red);
        if (threadIdx.x == 0)
            a.partials[(((int64_t)g * gridDim.x + blockIdx.x) * NPA) + i] = (double)s;
    }
    if (threadIdx.x == 0) a.partials[(((int64_t)g * gridDim.x + blockIdx.x) * NPA) + NPA - 1] = 0.0;
    if constexpr (TD) {
        __syncthreads();
        double *dst = a.tdpart + ((int64_t)g * gridDim.x + blockIdx.x) * ntd;
        for (int i = threadIdx.x; i < ntd; i += BLOCK) dst[i] = (double)tdtab[i];
    }
}

#ifndef __CUDACC_RTC__
template <typename R>
using AdjLauncher = void (*)(const AdjArgs<R> &, dim3, cudaStream_t);

template <typename R, int MODEL, int MAXM, bool JUMPS, bool TD = false>
void launch_adj(const AdjArgs<R> &a, dim3 grid, cudaStream_t s) {
    if constexpr (TD) {
        // the block's per-step table; the bytes were checked by the caller
        const size_t smem = sizeof(R) * (size_t)a.n_steps * 3 * MAXM;
        cudaFuncSetAttribute(sde_adj_kernel<R, MODEL, MAXM, JUMPS, TD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        sde_adj_kernel<R, MODEL, MAXM, JUMPS, TD><<<grid, BLOCK, smem, s>>>(a);
    } else {
        sde_adj_kernel<R, MODEL, MAXM, JUMPS><<<grid, BLOCK, 0, s>>>(a);
    }
}

template <typename R, int MODEL, int MAXM, bool JUMPS, bool TD = false>
int adj_max_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sde_adj_kernel<R, MODEL, MAXM, JUMPS, TD>, BLOCK, 0);
    return n;
}

AdjLauncher<float> find_adj_f32(int model, int maxm, bool jumps, int *bps);
AdjLauncher<double> find_adj_f64(int model, int maxm, bool jumps, int *bps);
// the FP32 2-variable Heston adjoint with its segment in shared memory
// (sde_adj_heston.cuh, in adj_f32.cu): constant parameters, no jumps, one
// checkpoint level of at most ADJ_HESTON_SEG steps per segment
AdjLauncher<float> find_adj_heston_f32(int seg, int *bps);
// the scalar FP32 OU adjoint with its segment in shared memory
// (sde_adj_ou.cuh, in adj_f32.cu): constant parameters, the state output,
// one checkpoint level of at most ADJ_OU_SEG steps per segment
AdjLauncher<float> find_adj_ou_f32(int seg, int *bps);
// time-dependent parameter slots, no jumps (adj_td.cu); the occupancy
// returned is for the kernel without its per-step table
AdjLauncher<float> find_adj_td_f32(int model, int maxm, int *bps);
AdjLauncher<double> find_adj_td_f64(int model, int maxm, int *bps);
// user SDEs (adj_user.cu)
AdjLauncher<float> find_adj_user_f32(int maxm, int *bps);
AdjLauncher<double> find_adj_user_f64(int maxm, int *bps);
#endif  // !__CUDACC_RTC__

}  // namespace sdegpu
