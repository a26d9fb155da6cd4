// Euler-Maruyama path integration of the sdepy preset SDEs.
//
// One thread owns one path of one group (the state variables that share a
// correlated Wiener increment) and walks the whole integration grid with the
// state in registers.  Per step it draws the group's normals (and Poisson
// uniforms / jump sizes) from Philox counters, or reads injected increments,
// applies the Euler step and, at output points, stores the group's outputs
// with paths innermost (a warp writes 32 consecutive paths: 128 B for f32,
// 256 B for f64).  Nothing else touches HBM.
//
// FP64 follows the operation order of sdepy's integrator.euler_next
// (sdepy/integration.py:707-718):  x + ((A_dt*dt + A_dw*dw) + A_dj*dj),
// with the coefficients of SDE.sde for each preset, using _rn intrinsics so
// that no multiply-add is contracted.  FP32 lets the compiler fuse.
#pragma once
#ifdef __CUDACC_RTC__
// runtime compilation of user SDE programs (sde_jit.cu): no host headers
typedef signed char int8_t;
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;
#define INFINITY __int_as_float(0x7f800000)
#else
#include <cstdint>
#include <cuda_runtime.h>
#endif

#include "../../include/sdepy_gb300.h"
#include "rng.cuh"

namespace sdegpu {

constexpr int BLOCK = 256;
constexpr int NCHOL = SDE_MAX_GROUP * (SDE_MAX_GROUP + 1) / 2;
constexpr int NPART = 8 + SDE_MAX_STRIKES;  // n, mean, M2, M3, M4, min, max, -, payoffs

// error flags (bitwise) reported by kernels
constexpr int ERRF_JUMP_CAP = 1;
constexpr int ERRF_ARGS = 4;  // a kernel was launched without a table it needs

template <typename R>
struct FwdArgs {
    int64_t paths;
    int32_t groups, M, W, n_pts;
    uint32_t step_offset;
    int32_t jump_law, out_mode, opg, has_corr;
    uint64_t seed;
    uint32_t stream;
    uint32_t path_offset;   // added to the path index in counter word 0
    PhiloxKey key;  // round keys of seed
    R sgn;  // sign of dt on this leg (+1 forward, -1 backward)
    // per-step tables
    const R *dt, *sqdt;
    const int32_t *out_row;
    const double *lamdt, *p0;
    const long long *thr, *thr1;   // Poisson count >= 1 / >= 2 thresholds (poisson_thresholds)
    // per-variable inputs
    const R *x0, *prm;  // prm[p*W + w]
    // FP32 LINEAR / OU with device RNG: coefficient rows [row][groups][2][MAXM],
    // padded to the kernel's MAXM, with normals z' = z / sqrt(2 ln 2):
    //   OU      (d, c): y' = (y - d y) + c (L z'),  y = x - theta,
    //                   d = k dt, c = sigma sqrt|dt| sqrt(2 ln 2);
    //   LINEAR  (b, c): x' = (x + b) + c (L z') (+ jumps),
    //                   b = c_dt dt, c = c_dw sqrt|dt| sqrt(2 ln 2)
    // (FP64 products rounded to FP32).  The OU state is held as the
    // deviation from theta, so the update is two fused multiply-adds and
    // rounds relative to the deviation; d is kept small (not 1 - k dt) so
    // that its rounding does not bias the decay over many steps.
    // With a time-dependent theta an OU row carries a third vector
    // b = k dt (theta_k - theta0) and the state is the deviation from the
    // first step's theta0: y' = ((y - d y) + c (L z')) + b (kernels
    // compiled with TDB, rows [row][groups][3][MAXM]).
    const float *coef;
    // OU: [groups][2][MAXM] = (theta0, x0 - theta0) in FP32
    const float *tshift;
    // the other kernels with time-dependent parameters: [steps][3][W] =
    // parameter slots 0..2 of each step, or NULL (prm applies throughout)
    const R *prm_t;
    // time-dependent correlation: [steps][NCHOL] packed Cholesky factors of
    // each step's correlation matrix (rows as chol below), or NULL; read
    // only by the kernels that reload per-step coefficients (STEPCORR)
    const R *chol_t;
    // SDE_MODEL_USER: the coefficient program, and each step's start time;
    // with dn / dj terms (user_jsrc bit 0: a dj term, bit 1: a dn term) the
    // jump-size law's a, b, pa per state, [3][W]
    SdeUserProgram uprog;
    const R *tk;
    const R *jprm;
    int32_t user_jsrc;
    // and the grid as runs of steps sharing one coefficient row:
    // (first step, end step, output row stored after the run or -1, coef row);
    // for the other kernels, runs of steps with one dt, w = 1 where an
    // adjoint checkpoint falls before the run's first step, or NULL
    const int4 *runs;
    int32_t n_runs;
    R chol[NCHOL];      // packed lower triangle, row m at m*(m+1)/2
    // injected increments (FP64, device)
    const double *dw, *dj;
    const long long *dn;
    // adjoint checkpoints (the general kernels): the state before every
    // ckpt_seg-th step, [ceil(n_steps / ckpt_seg)][W][paths], or NULL
    R *ckpt;
    int32_t ckpt_seg;
    // outputs
    R *xx;
    int64_t n_out_vars;
    int32_t *neg_count, *jump_count;
    unsigned long long *row_jumps;
    // the output row of the grid's first point (out_row[0], read on the
    // host), which the FP32 LINEAR / OU launcher fills with x0 by a separate
    // launch; -1: none
    int32_t tab_row0;
    // fused statistics
    int32_t stats_row, n_strikes;
    R strikes[SDE_MAX_STRIKES];
    R *stats_vals;     // [n_out_vars][paths] copy of the stats row, or NULL
    double *partials;  // [groups][gridDim.x][opg][NPART], or NULL
    int32_t *err;
};

// exact-order arithmetic for FP64, fusable for FP32
template <typename R> struct Ar;
template <> struct Ar<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double sqrt_(double a) { return __dsqrt_rn(a); }
    static __device__ __forceinline__ double exp_(double a) { return exp(a); }
};
template <> struct Ar<float> {
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
    static __device__ __forceinline__ float sqrt_(float a) { return approx_sqrt(a); }
    static __device__ __forceinline__ float exp_(float a) { return __expf(a); }
};

// ---------------------------------------------------------------------------
// block-level summary of one value per thread and output variable:
// count, mean, central sums M2..M4 (two-pass inside the block), min, max,
// payoff sums; merged into a running per-block partial in FP64 (Pebay's
// pairwise update), so each block's partial is exact to FP64 merge order.
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <typename R>
__device__ __forceinline__ R warp_min(R v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <typename R>
__device__ __forceinline__ R warp_max(R v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// block sum of one value (all threads must call; result valid in all threads)
template <typename R>
__device__ __forceinline__ R block_sum(R v, R *red) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    R s = (lane < BLOCK / 32) ? red[lane] : R(0);
    s = warp_sum(s);
    return s;
}
template <typename R>
__device__ __forceinline__ R block_min(R v, R *red) {
    v = warp_min(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    R s = (lane < BLOCK / 32) ? red[lane] : R(INFINITY);
    return warp_min(s);
}
template <typename R>
__device__ __forceinline__ R block_max(R v, R *red) {
    v = warp_max(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    R s = (lane < BLOCK / 32) ? red[lane] : R(-INFINITY);
    return warp_max(s);
}

// merge (nb, mb, M2b, M3b, M4b) into (na, ma, ...) -- Pebay 2008, eq. 2.1-2.3
__device__ __forceinline__ void moments_merge(double *A, const double *B) {
    const double na = A[0], nb = B[0];
    if (nb == 0.0) return;
    if (na == 0.0) {
        for (int i = 0; i < 5; ++i) A[i] = B[i];
        return;
    }
    const double n = na + nb;
    const double d = B[1] - A[1];
    const double dn = d / n;
    const double dn2 = dn * dn;
    const double t1 = d * dn * na * nb;
    const double M2 = A[2] + B[2] + t1;
    const double M3 = A[3] + B[3] + t1 * dn * (na - nb) +
                      3.0 * dn * (na * B[2] - nb * A[2]);
    const double M4 = A[4] + B[4] + t1 * dn2 * (na * na - na * nb + nb * nb) +
                      6.0 * dn2 * (na * na * B[2] + nb * nb * A[2]) +
                      4.0 * dn * (na * B[3] - nb * A[3]);
    A[0] = n;
    A[1] = A[1] + dn * nb;
    A[2] = M2;
    A[3] = M3;
    A[4] = M4;
}

// One round: every thread of the block offers value v (valid if act) for
// one output variable; the block's summary is merged into part (smem,
// NPART doubles) by thread 0.  All threads must call.
template <typename R>
__device__ void block_round_stats(R v, bool act, const R *strikes, int n_strikes,
                                  double *part, R *red) {
    const R one = act ? R(1) : R(0);
    const R n = block_sum<R>(one, red);
    if (n == R(0)) return;  // uniform across the block
    const R s1 = block_sum<R>(act ? v : R(0), red);
    const R mean = s1 / n;
    const R d = act ? (v - mean) : R(0);
    const R d2 = d * d;
    const R r1 = block_sum<R>(d, red);
    const R m2 = block_sum<R>(d2, red);
    const R m3 = block_sum<R>(d2 * d, red);
    const R m4 = block_sum<R>(d2 * d2, red);
    const R mn = block_min<R>(act ? v : R(INFINITY), red);
    const R mx = block_max<R>(act ? v : R(-INFINITY), red);
    R pay[SDE_MAX_STRIKES];
#pragma unroll
    for (int s = 0; s < SDE_MAX_STRIKES; ++s) {
        if (s < n_strikes) {
            const R x = act ? fmax(v - strikes[s], R(0)) : R(0);
            pay[s] = block_sum<R>(x, red);
        }
    }
    if (threadIdx.x == 0) {
        // recentre on the refined mean (mean + sum(d)/n) in FP64:
        // sum (d - e)^k with e = r/n, r = sum(d)
        const double nn = (double)n, r = (double)r1;
        const double a2 = (double)m2, a3 = (double)m3, a4 = (double)m4;
        const double e = r / nn;
        double B[5];
        B[0] = nn;
        B[1] = (double)mean + e;
        B[2] = a2 - r * e;
        B[3] = a3 - 3.0 * e * a2 + 2.0 * r * e * e;
        B[4] = a4 - 4.0 * e * a3 + 6.0 * e * e * a2 - 3.0 * r * e * e * e;
        moments_merge(part, B);
        part[5] = fmin(part[5], (double)mn);
        part[6] = fmax(part[6], (double)mx);
#pragma unroll
        for (int s = 0; s < SDE_MAX_STRIKES; ++s)
            if (s < n_strikes) part[8 + s] += (double)pay[s];
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// output transform of one group's state
// ---------------------------------------------------------------------------
template <typename R, int MAXM>
__device__ __forceinline__ int group_outputs(const R (&st)[MAXM], int M, int out_mode,
                                             R (&ov)[MAXM]) {
    switch (out_mode) {
    case SDE_OUT_EXP:
#pragma unroll
        for (int m = 0; m < MAXM; ++m) ov[m] = Ar<R>::exp_(st[m]);
        return M;
    case SDE_OUT_SUM: {
        R s = st[0];
#pragma unroll
        for (int m = 1; m < MAXM; ++m)
            if (m < M) s = Ar<R>::add(s, st[m]);
        ov[0] = s;
        return 1;
    }
    case SDE_OUT_HESTON_X:
#pragma unroll
        for (int m = 0; m < MAXM; ++m) ov[m] = (m < M / 2) ? Ar<R>::exp_(st[m]) : st[m];
        return M / 2;
    case SDE_OUT_HESTON_XY:
#pragma unroll
        for (int m = 0; m < MAXM; ++m) ov[m] = (m < M / 2) ? Ar<R>::exp_(st[m]) : st[m];
        return M;
    default:
#pragma unroll
        for (int m = 0; m < MAXM; ++m) ov[m] = st[m];
        return M;
    }
}

// Poisson count by inversion of the CDF, in FP64 (bit-exact given the
// uniform word): smallest k with u <= F(k).  Called only when u > p0.
// Integer thresholds of the inversion for uniform word w, u = (w + 0.5) 2^-32:
// count >= 1 <=> w > thr0 (u > p0), count >= 2 <=> w > thr1 (u > F(1)), with
// F(1) = p0 + (p0 lam) / 1 formed by the same rounded FP64 operations as
// poisson_tail (the temporaries keep the host compiler from fusing them).
// F * 2^32 is exact and so is subtracting 0.5 (F < 1), so each comparison
// is exactly the FP64 one; a step with one event needs no FP64 arithmetic.
#ifndef __CUDACC_RTC__
static inline void poisson_thresholds(double p0, double lam, long long &thr0, long long &thr1) {
    thr0 = (long long)floor(p0 * 4294967296.0 - 0.5);
    volatile double pk = p0 * lam;
    volatile double pk1 = pk / 1.0;
    volatile double F1 = p0 + pk1;
    thr1 = (long long)floor(F1 * 4294967296.0 - 0.5);
}
#endif

__device__ __forceinline__ int poisson_tail(uint32_t word, double p0, double lam, int32_t *err) {
    const double u = u01_f64(word);
    int k = 0;
    double pk = p0, F = p0;
    while (u > F) {
        ++k;
        pk = __ddiv_rn(__dmul_rn(pk, lam), (double)k);
        F = __dadd_rn(F, pk);
        if (k >= SDE_MAX_JUMPS_PER_STEP) {
            atomicOr(err, ERRF_JUMP_CAP);
            break;
        }
    }
    return k;
}

// one jump size of law `law` from the 4 words of its Philox call
template <typename R>
__device__ __forceinline__ R jump_size(int law, uint4 r, R ja, R jb, R jpa) {
    typedef Ar<R> A;
    switch (law) {
    case SDE_JUMP_NORM: {
        R z0, z1;
        Rng<R>::normal2(r.x, r.y, z0, z1);
        return A::add(ja, A::mul(jb, z0));
    }
    case SDE_JUMP_DOUBLE_EXP: {
        const R e = Rng<R>::expo(r.x);
        const R us = Rng<R>::unif(r.z);
        return (us <= jpa) ? A::mul(ja, e) : -A::mul(jb, e);
    }
    case SDE_JUMP_UNIFORM:
        return A::add(ja, A::mul(A::sub(jb, ja), Rng<R>::unif(r.z)));
    case SDE_JUMP_EXP:
        return A::mul(ja, Rng<R>::expo(r.x));
    default:
        return R(0);
    }
}

// ---------------------------------------------------------------------------
// per-step noise of one group, shared by the forward and adjoint kernels so
// that both see identical increments
// ---------------------------------------------------------------------------
template <int MAXM, bool JUMPS>
struct NoiseShape {
    static constexpr int NCMAX = (2 * ((MAXM + 1) / 2) + (JUMPS ? MAXM : 0) + 3) / 4;
};

// first Philox rounds of a path's per-step calls (counter (p, step,
// (g << 8) | call, stream) for call < NCALLS), which do not depend on the
// step (see philox_round0)
template <int NCALLS>
struct PathPre {
    uint4 r0[NCALLS];
    __device__ __forceinline__ PathPre(const PhiloxKey &key, uint32_t p, uint32_t g, uint32_t stream) {
#pragma unroll
        for (int c = 0; c < NCALLS; ++c) r0[c] = philox_round0(p, (g << 8) | (uint32_t)c, stream, key);
    }
};

// Groups of one or two state variables draw one Philox call per two
// steps, the call of even step k (counter (p, k + leg offset, g << 8,
// stream)):
//   one variable  -- its Box-Muller pair gives z0 to step k and z1 to step
//                    k + 1; words z and w are the Poisson uniforms of steps
//                    k and k + 1;
//   two variables (no jumps) -- the pair of words (x, y) gives the normals
//                    of step k, the pair of words (z, w) those of step k + 1.
// (With jumps, two-variable groups draw one call per step: words z, w are
// their Poisson uniforms.)  The cache holds the last call's values; any
// step order works (the adjoint starts segments at odd steps).  SC as for
// words_to_normals.
template <typename R, int NZ, bool SC = false>
struct PairedSteps;

template <typename R, bool SC>
struct PairedSteps<R, 1, SC> {
    int k0 = -2;          // even step of the cached call
    R z0, z1;
    uint32_t w0, w1;
    __device__ __forceinline__ void get(const PhiloxKey &key, const PathPre<1> &pre, int k, uint32_t offset,
                                        R &z, uint32_t &pword) {
        const int ke = k & ~1;
        if (ke != k0) {
            const uint4 r = philox_from_round0(pre.r0[0], (uint32_t)ke + offset, key);
            if (SC) Rng<R>::normal2_s(r.x, r.y, z0, z1);
            else Rng<R>::normal2(r.x, r.y, z0, z1);
            w0 = r.z;
            w1 = r.w;
            k0 = ke;
        }
        const bool odd = (k & 1) != 0;
        z = odd ? z1 : z0;
        pword = odd ? w1 : w0;
    }
};

template <typename R, bool SC>
struct PairedSteps<R, 2, SC> {
    int k0 = -2;
    R z[4];
    __device__ __forceinline__ void get(const PhiloxKey &key, const PathPre<1> &pre, int k, uint32_t offset,
                                        R &za, R &zb) {
        const int ke = k & ~1;
        if (ke != k0) {
            const uint4 r = philox_from_round0(pre.r0[0], (uint32_t)ke + offset, key);
            if (SC) {
                Rng<R>::normal2_s(r.x, r.y, z[0], z[1]);
                Rng<R>::normal2_s(r.z, r.w, z[2], z[3]);
            } else {
                Rng<R>::normal2(r.x, r.y, z[0], z[1]);
                Rng<R>::normal2(r.z, r.w, z[2], z[3]);
            }
            k0 = ke;
        }
        const bool odd = (k & 1) != 0;
        za = odd ? z[2] : z[0];
        zb = odd ? z[3] : z[1];
    }
};

// the paired-step scheme applies to groups of width MAXM == 1, and to
// MAXM == 2 without jumps
template <int MAXM, bool JUMPS>
struct Paired {
    static constexpr int NZ = (MAXM == 1) ? 1 : ((MAXM == 2 && !JUMPS) ? 2 : 0);
};

// Philox words of step k (c1w = step + leg offset): u[0 .. 2P) feed the
// Box-Muller pairs, u[2P + m] is the Poisson uniform of state m (jump models)
template <int MAXM, bool JUMPS>
__device__ __forceinline__ void step_words(const PhiloxKey &key,
                                           const PathPre<NoiseShape<MAXM, JUMPS>::NCMAX> &pre, uint32_t c1w,
                                           int NC, uint32_t (&u)[4 * NoiseShape<MAXM, JUMPS>::NCMAX]) {
    constexpr int NCMAX = NoiseShape<MAXM, JUMPS>::NCMAX;
#pragma unroll
    for (int c = 0; c < NCMAX; ++c) {
        if (c < NC) {
            const uint4 r = philox_from_round0(pre.r0[c], c1w, key);
            u[4 * c + 0] = r.x;
            u[4 * c + 1] = r.y;
            u[4 * c + 2] = r.z;
            u[4 * c + 3] = r.w;
        } else {
            u[4 * c + 0] = u[4 * c + 1] = u[4 * c + 2] = u[4 * c + 3] = 0u;
        }
    }
}

// SC: normals divided by sqrt(2 ln 2) (Rng::normal2_s), for the FP32 table
// kernels whose coefficients carry that factor
template <typename R, int MAXM, int NW, bool SC = false>
__device__ __forceinline__ void words_to_normals(const uint32_t (&u)[NW], R (&z)[MAXM]) {
#pragma unroll
    for (int q = 0; q < (MAXM + 1) / 2; ++q) {
        R z0, z1;
        if (SC) Rng<R>::normal2_s(u[2 * q], u[2 * q + 1], z0, z1);
        else Rng<R>::normal2(u[2 * q], u[2 * q + 1], z0, z1);
        z[2 * q] = z0;
        if (2 * q + 1 < MAXM) z[2 * q + 1] = z1;
    }
}

// dW = (L z) * sqrt|dt| (or z * sqrt|dt| without correlation)
template <typename R, int MAXM>
__device__ __forceinline__ void correlate(const R *chol, bool has_corr, const R (&z)[MAXM], R sq,
                                          R (&dW)[MAXM]) {
    typedef Ar<R> A;
    if (has_corr) {
#pragma unroll
        for (int m = 0; m < MAXM; ++m) {
            const int base = m * (m + 1) / 2;
            R acc = A::mul(chol[base], z[0]);
#pragma unroll
            for (int j = 1; j <= m; ++j) acc = A::add(acc, A::mul(chol[base + j], z[j]));
            dW[m] = A::mul(acc, sq);
        }
    } else {
#pragma unroll
        for (int m = 0; m < MAXM; ++m) dW[m] = A::mul(z[m], sq);
    }
}

template <typename R, bool SC>
__device__ __forceinline__ void normals4(uint4 r, R (&zc)[4]) {
    if (SC) {
        Rng<R>::normal2_s(r.x, r.y, zc[0], zc[1]);
        Rng<R>::normal2_s(r.z, r.w, zc[2], zc[3]);
    } else {
        Rng<R>::normal2(r.x, r.y, zc[0], zc[1]);
        Rng<R>::normal2(r.z, r.w, zc[2], zc[3]);
    }
}

// Same increments as step_words + words_to_normals + correlate, produced one
// Philox call (4 normals) at a time so that only 4 normals are live; the
// mat-vec accumulates in the same order (j ascending), so FP64 rounding is
// identical.  Used by the kernels without jumps.
template <typename R, int MAXM, bool SC = false>
__device__ __forceinline__ void step_increments(const PhiloxKey &key, const PathPre<(MAXM + 3) / 4> &pre,
                                                uint32_t c1w, int NC, const R *chol, bool has_corr,
                                                R sq, R (&dW)[MAXM]) {
    typedef Ar<R> A;
    constexpr int NCN = (MAXM + 3) / 4;  // calls carrying normals
    if (!has_corr) {  // tested once per step, not per normal
#pragma unroll
        for (int c = 0; c < NCN; ++c) {
            if (c < NC) {
                const uint4 r = philox_from_round0(pre.r0[c], c1w, key);
                R zc[4];
                normals4<R, SC>(r, zc);
#pragma unroll
                for (int l = 0; l < 4; ++l)
                    if (4 * c + l < MAXM) dW[4 * c + l] = A::mul(zc[l], sq);
            }
        }
        return;
    }
#pragma unroll
    for (int c = 0; c < NCN; ++c) {
        if (c < NC) {
            const uint4 r = philox_from_round0(pre.r0[c], c1w, key);
            R zc[4];
            normals4<R, SC>(r, zc);
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const int j = 4 * c + l;
                if (j < MAXM) {
#pragma unroll
                    for (int m = 0; m < MAXM; ++m) {
                        if (m >= j) {
                            const R t = A::mul(chol[m * (m + 1) / 2 + j], zc[l]);
                            dW[m] = (j == 0) ? t : A::add(dW[m], t);
                        }
                    }
                }
            }
        }
    }
#pragma unroll
    for (int m = 0; m < MAXM; ++m) dW[m] = A::mul(dW[m], sq);
}

template <int NW>
__device__ __forceinline__ uint32_t pick_word(const uint32_t (&u)[NW], int idx) {
    uint32_t word = u[0];
#pragma unroll
    for (int i = 0; i < NW; ++i)
        if (i == idx) word = u[i];
    return word;
}

// derivatives of one jump size with respect to the law's a and b
template <typename R>
__device__ __forceinline__ void jump_size_grad(int law, uint4 r, R ja, R jb, R jpa, R &da, R &db) {
    switch (law) {
    case SDE_JUMP_NORM: {
        R z0, z1;
        Rng<R>::normal2(r.x, r.y, z0, z1);
        da = R(1);
        db = z0;
        return;
    }
    case SDE_JUMP_DOUBLE_EXP: {
        const R e = Rng<R>::expo(r.x);
        const R us = Rng<R>::unif(r.z);
        if (us <= jpa) { da = e; db = R(0); }
        else { da = R(0); db = -e; }
        return;
    }
    case SDE_JUMP_UNIFORM: {
        const R u = Rng<R>::unif(r.z);
        da = R(1) - u;
        db = u;
        return;
    }
    case SDE_JUMP_EXP:
        da = Rng<R>::expo(r.x);
        db = R(0);
        return;
    default:
        da = db = R(0);
    }
}

// ---------------------------------------------------------------------------
// user SDEs: the coefficient program (SdeUserProgram), interpreted per state
// variable and step.  Every thread runs the same instruction sequence (no
// divergence); the register file lives in local memory (L1).  Register and
// constant indices are checked on the host before launch.  FP64 arithmetic
// is explicitly rounded (no contraction), so that the sequence of roundings
// is numpy's; the elementary functions are CUDA's.
// ---------------------------------------------------------------------------
template <typename R> struct UFn;
template <> struct UFn<double> {
    __device__ static double exp_(double x) { return exp(x); }
    __device__ static double log_(double x) { return log(x); }
    __device__ static double sin_(double x) { return sin(x); }
    __device__ static double cos_(double x) { return cos(x); }
    __device__ static double tan_(double x) { return tan(x); }
    __device__ static double tanh_(double x) { return tanh(x); }
    __device__ static double pow_(double x, double y) { return pow(x, y); }
    __device__ static double expm1_(double x) { return expm1(x); }
    __device__ static double log1p_(double x) { return log1p(x); }
    __device__ static double atan_(double x) { return atan(x); }
};
template <> struct UFn<float> {
    __device__ static float exp_(float x) { return expf(x); }
    __device__ static float log_(float x) { return logf(x); }
    __device__ static float sin_(float x) { return sinf(x); }
    __device__ static float cos_(float x) { return cosf(x); }
    __device__ static float tan_(float x) { return tanf(x); }
    __device__ static float tanh_(float x) { return tanhf(x); }
    __device__ static float pow_(float x, float y) { return powf(x, y); }
    __device__ static float expm1_(float x) { return expm1f(x); }
    __device__ static float log1p_(float x) { return log1pf(x); }
    __device__ static float atan_(float x) { return atanf(x); }
};

// numpy's maximum / minimum: NaN if either operand is NaN
template <typename R>
__device__ __forceinline__ R np_max(R a, R b) { return (a != a) ? a : (b != b) ? b : (a >= b ? a : b); }
template <typename R>
__device__ __forceinline__ R np_min(R a, R b) { return (a != a) ? a : (b != b) ? b : (a <= b ? a : b); }

// xs[0..q-1]: the states of one component in the q equations (q = 1 for a
// single SDE); out[e][j]: the coefficient of term j of equation e
template <typename R>
__device__ __noinline__ void user_coefs(const SdeUserProgram &u, const R *xs, R t, const R (&p)[6],
                                        R (*out)[SDE_USER_MAX_TERMS]) {
    typedef Ar<R> A;
    typedef UFn<R> F;
    R r[SDE_USER_MAX_REGS];
    r[0] = xs[0];
    r[1] = t;
#pragma unroll
    for (int i = 0; i < 6; ++i) r[2 + i] = p[i];
    for (int e = 1; e < u.n_eq; ++e) r[7 + e] = xs[e];
    for (int i = 0; i < u.n_ops; ++i) {
        const uint32_t op = u.ops[i];
        const int d = (op >> 8) & 0xff, ia = (op >> 16) & 0xff, ib = op >> 24;
        const int code = op & 0xff;
        if (code == SDE_UOP_CONST) {
            r[d] = (R)u.consts[ia];
            continue;
        }
        const R va = r[ia], vb = r[ib];
        R v;
        switch (code) {
        case SDE_UOP_ADD: v = A::add(va, vb); break;
        case SDE_UOP_SUB: v = A::sub(va, vb); break;
        case SDE_UOP_MUL: v = A::mul(va, vb); break;
        case SDE_UOP_DIV: v = va / vb; break;   // IEEE division, correctly rounded
        case SDE_UOP_NEG: v = -va; break;
        case SDE_UOP_ABS: v = fabs(va); break;
        case SDE_UOP_EXP: v = F::exp_(va); break;
        case SDE_UOP_LOG: v = F::log_(va); break;
        case SDE_UOP_SQRT: v = A::sqrt_(va); break;
        case SDE_UOP_MAX: v = np_max(va, vb); break;
        case SDE_UOP_MIN: v = np_min(va, vb); break;
        case SDE_UOP_SIN: v = F::sin_(va); break;
        case SDE_UOP_COS: v = F::cos_(va); break;
        case SDE_UOP_TAN: v = F::tan_(va); break;
        case SDE_UOP_TANH: v = F::tanh_(va); break;
        case SDE_UOP_POW: v = F::pow_(va, vb); break;
        case SDE_UOP_EXPM1: v = F::expm1_(va); break;
        case SDE_UOP_LOG1P: v = F::log1p_(va); break;
        case SDE_UOP_ARCTAN: v = F::atan_(va); break;
        default: v = va; break;   // SDE_UOP_COPY
        }
        r[d] = v;
    }
    for (int e = 0; e < u.n_eq; ++e)
#pragma unroll
        for (int j = 0; j < SDE_USER_MAX_TERMS; ++j) out[e][j] = j < u.n_terms ? r[u.term_register[e][j]] : R(0);
}

// the internal kernel model of user SDE systems (q > 1: SdeSpec.model is
// SDE_MODEL_USER, the program's n_eq selects these instantiations)
constexpr int SDE_MODEL_USER_SYS = 16;
// user SDEs compiled at run time (sde_jit.cu): the program becomes the
// straight-line function UserJitFn<R>::coefs of a runtime-compiled unit,
// which instantiates the forward kernel with these models
constexpr int SDE_MODEL_USER_JIT = 32;
constexpr int SDE_MODEL_USER_SYS_JIT = 48;
template <typename R>
struct UserJitFn;   // defined only in runtime-compiled units

// a user program's coefficients: compiled, or interpreted
template <typename R, int MODEL>
__device__ __forceinline__ void user_eval(const SdeUserProgram &u, const R *xs, R t, const R (&p)[6],
                                          R (*out)[SDE_USER_MAX_TERMS]) {
    if constexpr (MODEL == SDE_MODEL_USER_JIT || MODEL == SDE_MODEL_USER_SYS_JIT)
        UserJitFn<R>::coefs(xs, t, p, out);
    else
        user_coefs<R>(u, xs, t, p, out);
}

// a user program's shape: the equations, the terms and each term's source
// (SDE_SRC_*), compile-time constants of a compiled program (UserJitFn's
// NEQ, NT, src), else read from the program
template <typename R, int MODEL>
__device__ __forceinline__ int user_neq(const SdeUserProgram &u) {
    if constexpr (MODEL == SDE_MODEL_USER_JIT || MODEL == SDE_MODEL_USER_SYS_JIT) return UserJitFn<R>::NEQ;
    else return u.n_eq;
}
template <typename R, int MODEL>
__device__ __forceinline__ int user_nt(const SdeUserProgram &u) {
    if constexpr (MODEL == SDE_MODEL_USER_JIT || MODEL == SDE_MODEL_USER_SYS_JIT) return UserJitFn<R>::NT;
    else return u.n_terms;
}
template <typename R, int MODEL>
__device__ __forceinline__ int user_src(const SdeUserProgram &u, int i) {
    if constexpr (MODEL == SDE_MODEL_USER_JIT || MODEL == SDE_MODEL_USER_SYS_JIT) return UserJitFn<R>::src(i);
    else return u.term_source[i];
}

// ---------------------------------------------------------------------------
// the forward kernel
// ---------------------------------------------------------------------------
// FP32 device-RNG kernels without jumps, up to 8 states per thread (4 for
// Heston, whose step keeps more values live; half that for antithetic
// kernels, which carry two paths), are held to 80 registers: 3 resident
// blocks (24 warps) per SM
template <typename R, int MODEL, int MAXM, bool INJECT, bool JUMPS, bool ANTI = false>
struct FwdOccupancy {
    static constexpr int CAP_M = (MODEL == SDE_MODEL_HESTON || MODEL == SDE_MODEL_CIR ? 4 : 8) / (ANTI ? 2 : 1);
    // the other FP32 kernels of up to 4 states: at least two blocks per SM
    // (128 registers; one more register halves the resident warps; wider
    // groups would spill)
    static constexpr int MIN_BLOCKS =
        (sizeof(R) == 4 && MAXM <= CAP_M && !INJECT && !JUMPS && MODEL != SDE_MODEL_USER && MODEL < 8) ? 3
        : (sizeof(R) == 4 && MAXM <= 4) ? 2 : 1;
};

// TDEP: time-dependent-coefficient instantiations of the FP32 device-noise
// kernels whose common form carries no trace of the extra code (even code
// that never runs changes how the hot loop compiles): OU run tables with
// the theta term, Heston with per-step coefficient reloads.
// ANTI: antithetic paths (device noise): paths q and q + K (K = paths / 2)
// share their draws, the second with the opposite Wiener increments and
// the same jumps (sdepy's odd_wiener_source / even_cpoisson_source,
// sdepy/infrastructure.py:2047-2150); one thread integrates both, drawing
// once.
template <typename R, int MODEL, int MAXM, bool INJECT, bool JUMPS, bool TDEP = false, bool ANTI = false>
__global__ void __launch_bounds__(BLOCK, (FwdOccupancy<R, MODEL, MAXM, INJECT, JUMPS, ANTI>::MIN_BLOCKS))
sde_fwd_kernel(const __grid_constant__ FwdArgs<R> a) {
    typedef Ar<R> A;
    constexpr int NCMAX = NoiseShape<MAXM, JUMPS>::NCMAX;
    constexpr bool TAB = sizeof(R) == 4 && (MODEL == SDE_MODEL_LINEAR || MODEL == SDE_MODEL_OU) && !INJECT;
    constexpr bool SHIFT = TAB && MODEL == SDE_MODEL_OU;  // state held as x - theta
    constexpr int NA = ANTI ? 2 : 1;   // paths per thread
    constexpr bool TDB = TDEP && SHIFT;   // OU rows with the time-dependent-theta term
    // per-step coefficient reloads compiled in (the non-table kernels but
    // the common FP32 Heston and CIR ones)
    constexpr bool USER = MODEL == SDE_MODEL_USER || MODEL == SDE_MODEL_USER_SYS ||
                          MODEL == SDE_MODEL_USER_JIT || MODEL == SDE_MODEL_USER_SYS_JIT;
    constexpr bool RELOAD = !TAB && (sizeof(R) == 8 || INJECT || TDEP || USER);
    // per-step correlation factors compiled in (the same kernels, TAB ones
    // included, with device noise)
    constexpr bool STEPCORR = !INJECT && (sizeof(R) == 8 || TDEP || USER);
    // parameter slots of a time-dependent table row (all six for USER)
    constexpr int NPT = USER ? 6 : 3;
    // steps per iteration of the step loops: two, so that the next step's
    // draws overlap this step's arithmetic (5-12% on the FP32 kernels), but
    // one for the 8- and 16-wide time-dependent forms, which would spill
    constexpr int UNROLL = (TDEP && MAXM >= 8) ? 1 : 2;
    // the kernels other than the FP32 run-table ones step through runs of
    // one dt (FwdArgs::runs, when the host gives them)
    constexpr bool RUNS = !TAB;
    __shared__ R red[BLOCK / 32];
    __shared__ double part[MAXM][NPART];
    __shared__ R svs[NA][MAXM][BLOCK];   // this round's value of each output at the stats row

    const int g = blockIdx.y;
    const int M = a.M;
    const int W = a.W;
    const int P = (M + 1) >> 1;
    const int NC = (2 * P + (JUMPS ? M : 0) + 3) >> 2;
    const int n_steps = a.n_pts - 1;
    const bool do_stats = a.partials != nullptr;
    const PhiloxKey key = a.key;  // by value: uniform registers, not indexed parameter loads
    if (((TAB && (a.coef == nullptr || a.runs == nullptr || (SHIFT && a.tshift == nullptr))) ||
         (!TAB && !RELOAD && a.prm_t != nullptr) || (!STEPCORR && a.chol_t != nullptr)) &&
        n_steps > 0) {  // uniform: the grid returns
        if (threadIdx.x == 0 && blockIdx.x == 0 && blockIdx.y == 0) atomicOr(a.err, ERRF_ARGS);
        return;
    }

    // this group's coefficients, in registers
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
    if (do_stats && threadIdx.x < MAXM) {
        for (int i = 0; i < NPART; ++i) part[threadIdx.x][i] = 0.0;
        part[threadIdx.x][5] = INFINITY;
        part[threadIdx.x][6] = -INFINITY;
    }

    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    const int64_t npath = ANTI ? a.paths / 2 : a.paths;   // paths (pairs with ANTI) over threads
    const int64_t rounds = (npath + stride - 1) / stride;
    for (int64_t rd = 0; rd < rounds; ++rd) {
        const int64_t p = rd * stride + (int64_t)blockIdx.x * BLOCK + threadIdx.x;
        const bool act = p < npath;
        if (do_stats) {
#pragma unroll
            for (int i = 0; i < NA; ++i)
#pragma unroll
                for (int m = 0; m < MAXM; ++m) svs[i][m][threadIdx.x] = R(0);
        }
        if (act) {
            R st[MAXM];
            R st1[ANTI ? MAXM : 1];   // the antithetic path p + npath
#pragma unroll
            for (int m = 0; m < MAXM; ++m) st[m] = x0[m];
            if constexpr (ANTI) {
#pragma unroll
                for (int m = 0; m < MAXM; ++m) st1[m] = x0[m];
            }
            int negc[MAXM], negc1[ANTI ? MAXM : 1];
            int jcnt[MAXM];
#pragma unroll
            for (int m = 0; m < MAXM; ++m) { negc[m] = 0; jcnt[m] = 0; }
            if constexpr (ANTI) {
#pragma unroll
                for (int m = 0; m < MAXM; ++m) negc1[m] = 0;
            }
            unsigned int row_jc = 0;
            // a user SDE's Poisson increments dn of the step (dJ holds dj)
            R dN[(USER && JUMPS) ? MAXM : 1] = {};
            // the increment of a user SDE's term: dt, dw, dn or dj of state m
            auto user_dz = [&](int src, R dt, R dw, R dj, int m) -> R {
                if (src == SDE_SRC_DT) return dt;
                if (src == SDE_SRC_DW) return dw;
                if constexpr (USER && JUMPS) return src == SDE_SRC_DJ ? dj : dN[m];
                return R(0);
            };

            // store helper (lambda keeps the loop body readable): state s of
            // path pth, stats values in slot i; sh: the state is the
            // deviation from theta
            auto store1 = [&](int row, bool sh, const R (&s)[MAXM], int64_t pth, int i) {
                R ov[MAXM];
                int no;
                if (SHIFT && sh) {
                    R sx[MAXM];
#pragma unroll
                    for (int m = 0; m < MAXM; ++m) sx[m] = s[m] + (R)__ldg(a.tshift + g * 2 * MAXM + m);
                    no = group_outputs<R, MAXM>(sx, M, a.out_mode, ov);
                } else {
                    no = group_outputs<R, MAXM>(s, M, a.out_mode, ov);
                }
                if (a.xx) {
#pragma unroll
                    for (int m = 0; m < MAXM; ++m)
                        if (m < no)
                            // streaming store: the path output must not evict
                            // the per-step tables from L2
                            __stcs(&a.xx[((int64_t)row * a.n_out_vars + (int64_t)g * a.opg + m) * a.paths + pth], ov[m]);
                }
                if (row == a.stats_row) {
#pragma unroll
                    for (int m = 0; m < MAXM; ++m) svs[i][m][threadIdx.x] = ov[m];
                    if (a.stats_vals) {
#pragma unroll
                        for (int m = 0; m < MAXM; ++m)
                            if (m < no)
                                __stcs(&a.stats_vals[((int64_t)g * a.opg + m) * a.paths + pth], ov[m]);
                    }
                }
            };
            auto store = [&](int row, bool sh) {
                store1(row, sh, st, p, 0);
                if constexpr (ANTI) store1(row, sh, st1, p + npath, 1);
                if (JUMPS && a.row_jumps) {
                    if (row_jc) atomicAdd(&a.row_jumps[row], (unsigned long long)row_jc);
                    row_jc = 0;
                }
            };

            {
                const int r0 = a.out_row[0];
                if (r0 >= 0) store(r0, false);
            }
            if (SHIFT && n_steps > 0) {
#pragma unroll
                for (int m = 0; m < MAXM; ++m) st[m] = (R)__ldg(a.tshift + (g * 2 + 1) * MAXM + m);
                if constexpr (ANTI) {
#pragma unroll
                    for (int m = 0; m < MAXM; ++m) st1[m] = st[m];
                }
            }
            const uint32_t pc = (uint32_t)p + a.path_offset;   // counter word 0 of this path
            const PathPre<NCMAX> pre(key, pc, (uint32_t)g, a.stream);
            constexpr int NZ = Paired<MAXM, JUMPS>::NZ;
            PairedSteps<R, NZ == 0 ? 1 : NZ, TAB> pair;   // groups of one or two variables
            // Poisson count of state m at step k from uniform word `word`, and
            // the sum of its jump sizes
            auto add_jumps = [&](int m, uint32_t word, int k, uint32_t c1w, R (&dJ)[MAXM]) {
                const int w = g * M + m;
                const int64_t tix = (int64_t)k * W + w;
                if constexpr (USER) {
                    // dj: the count of `word` and as many jump sizes; dn: that
                    // count, or with a dj term too, the count of an
                    // independent word (counter (p, step, 2^30 | w, stream))
                    auto count = [&](uint32_t u) -> int {
                        if ((long long)u <= a.thr[tix]) return 0;
                        return (long long)u <= a.thr1[tix] ? 1 : poisson_tail(u, a.p0[tix], a.lamdt[tix], a.err);
                    };
                    int cnt = count(word);
                    if (a.user_jsrc & 1) {
                        if (cnt) {
                            const R ja = a.jprm[w], jb = a.jprm[W + w], jpa = a.jprm[2 * W + w];
                            R S = R(0);
                            for (int j = 0; j < cnt; ++j) {
                                const uint4 r = philox4x32_10(
                                    make_uint4(pc, c1w, 0x80000000u | ((uint32_t)w << 12) | (uint32_t)j,
                                               a.stream),
                                    key);
                                const R y = jump_size<R>(a.jump_law, r, ja, jb, jpa);
                                S = (j == 0) ? y : A::add(S, y);
                            }
                            dJ[m] = A::mul(a.sgn, S);
                        }
                        if (a.user_jsrc & 2)
                            cnt = count(philox4x32_10(make_uint4(pc, c1w, 0x40000000u | (uint32_t)w, a.stream),
                                                      key).x);
                    }
                    if constexpr (JUMPS)
                        if ((a.user_jsrc & 2) && cnt) dN[m] = A::mul(a.sgn, (R)cnt);
                    return;
                }
                if ((long long)word > a.thr[tix]) {
                    const int cnt = (long long)word <= a.thr1[tix] ? 1 : poisson_tail(word, a.p0[tix], a.lamdt[tix], a.err);
                    R S = R(0);
                    for (int j = 0; j < cnt; ++j) {
                        const uint4 r = philox4x32_10(
                            make_uint4(pc, c1w, 0x80000000u | ((uint32_t)w << 12) | (uint32_t)j, a.stream),
                            key);
                        const R y = jump_size<R>(a.jump_law, r, c3[m], c4[m], c5[m]);
                        S = (j == 0) ? y : A::add(S, y);
                    }
                    dJ[m] = A::mul(a.sgn, S);
                    const int sc = a.sgn < R(0) ? -cnt : cnt;
                    jcnt[m] += sc;
                    row_jc += (unsigned int)(NA * cnt);   // the antithetic path jumps alike
                }
            };
            // increments of step k: injected, or drawn from Philox counters
            // (normals, correlated; Poisson counts and jump sums)
            auto draw = [&](int k, R sq, R (&dW)[MAXM], R (&dJ)[MAXM]) {
#pragma unroll
                for (int m = 0; m < MAXM; ++m) dJ[m] = R(0);
                if constexpr (USER && JUMPS) {
#pragma unroll
                    for (int m = 0; m < MAXM; ++m) dN[m] = R(0);
                }
                // f(the step's correlation factor): the per-step table's row
                // (uniform test), else the constant factor of the parameter
                // block -- two copies of f, so that the constant one keeps
                // its constant-bank loads
                auto with_chol = [&](auto &&f) {
                    if constexpr (STEPCORR)
                        if (a.chol_t) {
                            f(a.chol_t + (int64_t)k * NCHOL);
                            return;
                        }
                    f(a.chol);
                };
                if (INJECT) {
#pragma unroll
                    for (int m = 0; m < MAXM; ++m) {
                        if (m < M) {
                            const int64_t idx = ((int64_t)k * W + g * M + m) * a.paths + p;
                            if constexpr (USER) dW[m] = a.dw ? (R)a.dw[idx] : R(0);   // a program without dw
                            else dW[m] = (R)a.dw[idx];
                            if constexpr (USER && JUMPS) {   // the program's own dj / dn sources
                                if (a.dj) dJ[m] = (R)a.dj[idx];
                                if (a.dn) dN[m] = (R)a.dn[idx];
                            } else if (JUMPS) {
                                dJ[m] = (R)a.dj[idx];
                                if (a.dn) {
                                    const int c = (int)a.dn[idx];
                                    jcnt[m] += c;
                                    row_jc += (unsigned int)(c < 0 ? -c : c);
                                }
                            }
                        } else {
                            dW[m] = R(0);
                        }
                    }
                    return;
                }
                const uint32_t c1w = (uint32_t)k + a.step_offset;
                if constexpr (NZ == 1) {
                    R z;
                    uint32_t pword;
                    pair.get(key, pre, k, a.step_offset, z, pword);
                    dW[0] = A::mul(z, sq);   // a 1x1 correlation factor is 1
                    if (JUMPS) add_jumps(0, pword, k, c1w, dJ);
                    return;
                } else if constexpr (NZ == 2) {
                    R z[MAXM];
                    pair.get(key, pre, k, a.step_offset, z[0], z[1]);
                    with_chol([&](const R *chol) { correlate<R, MAXM>(chol, a.has_corr, z, sq, dW); });
                    return;
                }
                if constexpr (!JUMPS) {
                    with_chol([&](const R *chol) {
                        step_increments<R, MAXM, TAB>(key, pre, c1w, NC, chol, a.has_corr, sq, dW);
                    });
                    return;
                }
                uint32_t u[4 * NCMAX];
                step_words<MAXM, JUMPS>(key, pre, c1w, NC, u);
                R z[MAXM];
                words_to_normals<R, MAXM, 4 * NCMAX, TAB>(u, z);
                with_chol([&](const R *chol) { correlate<R, MAXM>(chol, a.has_corr, z, sq, dW); });
#pragma unroll
                for (int m = 0; m < MAXM; ++m)
                    if (m < M) add_jumps(m, pick_word(u, 2 * P + m), k, c1w, dJ);
            };

            if constexpr (TAB) {
                // runs of steps sharing one coefficient row: no per-step
                // output-row test or table indexing
#pragma unroll 1
                for (int ri = 0; ri < a.n_runs; ++ri) {
                    const int4 run = __ldg(a.runs + ri);
                    // rows padded to MAXM (d = b = c = 0 beyond M); read every step
                    // from L1 rather than held in registers across the run
                    constexpr int NB = TDB ? 3 : 2;   // coefficient vectors per row
                    const float *tb = a.coef + ((int64_t)run.w * a.groups + g) * NB * MAXM;
#pragma unroll UNROLL
                    for (int k = run.x; k < run.y; ++k) {
                        R dW[MAXM], dJ[MAXM];
                        // sqrt|dt| sqrt(2 ln 2) is folded into c
                        draw(k, R(1), dW, dJ);
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
                        // one state array, increments dW times sgn
                        auto tab_update = [&](R (&s)[MAXM], float sgn) {
#pragma unroll
                            for (int m = 0; m < MAXM; ++m) {
                                float x = (float)s[m];
                                if (SHIFT) x = fmaf(-ca[m], x, x);   // y - d y
                                else x = x + ca[m];                  // x + b
                                x = fmaf(sgn * cc[m], (float)dW[m], x);
                                if (JUMPS) x = x + (float)dJ[m];
                                s[m] = (R)x;
                            }
                            if constexpr (SHIFT && TDB) {   // a time-dependent theta
#pragma unroll
                                for (int m = 0; m < MAXM; ++m) s[m] = s[m] + __ldg(tb + 2 * MAXM + m);
                            }
                        };
                        tab_update(st, 1.0f);
                        if constexpr (ANTI) tab_update(st1, -1.0f);
                    }
                    if (run.z >= 0) store(run.z, true);
                }
            } else {
                // adjoint checkpoints: the state before steps 0, ckpt_seg, ...
                int ci = 0;
                auto ck_store = [&]() {
#pragma unroll
                    for (int m = 0; m < MAXM; ++m)
                        if (m < M) a.ckpt[((int64_t)ci * W + g * M + m) * a.paths + p] = st[m];
                    ++ci;
                };
                // one Euler step, k from tt[k] (dt, sq = sqrt|dt|)
                auto step_k = [&](int k, const R dt, const R sq) {
                    // time-dependent coefficients of step k (uniform test; not
                    // compiled into the FP32 Heston kernels' common form)
                    if (RELOAD && a.prm_t) {
                        const R *pk = a.prm_t + (int64_t)k * NPT * W;
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) {
                            const int w = g * M + (m < M ? m : 0);
                            c0[m] = __ldg(pk + w);
                            c1[m] = __ldg(pk + W + w);
                            c2[m] = __ldg(pk + 2 * W + w);
                            if constexpr (USER) {
                                c3[m] = __ldg(pk + 3 * W + w);
                                c4[m] = __ldg(pk + 4 * W + w);
                                c5[m] = __ldg(pk + 5 * W + w);
                            }
                        }
                    }
                    const R tk = USER ? a.tk[k] : R(0);   // the step's start (user SDEs)
                    R dW[MAXM], dJ[MAXM];
                    draw(k, sq, dW, dJ);
                    // ---- Euler step, sdepy's operation order ----------------------
                    auto euler = [&](R (&st)[MAXM], const R (&dW)[MAXM], int (&negc)[MAXM]) {
                    if (MODEL == SDE_MODEL_LINEAR) {
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) {
                            R inc = A::add(A::mul(c0[m], dt), A::mul(c1[m], dW[m]));
                            if (JUMPS) inc = A::add(inc, dJ[m]);
                            st[m] = A::add(st[m], inc);
                        }
                    } else if (MODEL == SDE_MODEL_OU) {
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) {
                            const R drift = A::mul(c0[m], A::sub(c1[m], st[m]));
                            st[m] = A::add(st[m], A::add(A::mul(drift, dt), A::mul(c2[m], dW[m])));
                        }
                    } else if (MODEL == SDE_MODEL_USER || MODEL == SDE_MODEL_USER_JIT) {
                        // x + (A_1 dZ_1 + ... + A_n dZ_n), the terms in the order of
                        // the SDE function's dict (sdepy sums from 0: 0 + v == v)
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) {
                            const R pv[6] = {c0[m], c1[m], c2[m], c3[m], c4[m], c5[m]};
                            R A2[1][SDE_USER_MAX_TERMS];
                            const R xm[1] = {st[m]};
                            user_eval<R, MODEL>(a.uprog, xm, tk, pv, A2);
                            R s = R(0);
#pragma unroll
                            for (int i = 0; i < SDE_USER_MAX_TERMS; ++i)
                                if (i < user_nt<R, MODEL>(a.uprog)) {
                                    const R dz = user_dz(user_src<R, MODEL>(a.uprog, i), dt, dW[m], dJ[m], m);
                                    const R term = A::mul(A2[0][i], dz);
                                    s = i == 0 ? term : A::add(s, term);
                                }
                            st[m] = A::add(st[m], s);
                        }
                    } else if (MODEL == SDE_MODEL_USER_SYS || MODEL == SDE_MODEL_USER_SYS_JIT) {
                        // the group is one last-axis slice: equation e's component
                        // h at e * nc + h; the program runs per component on the
                        // states of every equation, then all states step at once.
                        // States are gathered and scattered by unrolled selects
                        // (compile-time indices: registers, not local memory).
                        const int q = user_neq<R, MODEL>(a.uprog), nc = M / q;
                        R nx[MAXM];
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) nx[m] = st[m];
#pragma unroll
                        for (int h = 0; h < MAXM; ++h) {
                            if (h >= nc) break;
                            R xs[SDE_USER_MAX_EQ], A2[SDE_USER_MAX_EQ][SDE_USER_MAX_TERMS];
#pragma unroll
                            for (int e = 0; e < SDE_USER_MAX_EQ; ++e) {
                                xs[e] = R(0);
#pragma unroll
                                for (int m = 0; m < MAXM; ++m)
                                    if (e < q && m == e * nc + h) xs[e] = st[m];
                            }
                            // parameters broadcast along the equations: component h's
                            const R pv[6] = {c0[h], c1[h], c2[h], c3[h], c4[h], c5[h]};
                            user_eval<R, MODEL>(a.uprog, xs, tk, pv, A2);
#pragma unroll
                            for (int e = 0; e < SDE_USER_MAX_EQ; ++e) {
                                if (e >= q) break;
                                const int mm = e * nc + h;
                                R dwv = R(0), djv = R(0), dnv = R(0);
#pragma unroll
                                for (int m = 0; m < MAXM; ++m)
                                    if (m == mm) {
                                        dwv = dW[m];
                                        djv = dJ[m];
                                        if constexpr (USER && JUMPS) dnv = dN[m];
                                    }
                                R s = R(0);
#pragma unroll
                                for (int i = 0; i < SDE_USER_MAX_TERMS; ++i)
                                    if (i < user_nt<R, MODEL>(a.uprog)) {
                                        const int src = user_src<R, MODEL>(a.uprog, i);
                                        const R dz = src == SDE_SRC_DT ? dt : src == SDE_SRC_DW ? dwv
                                                     : src == SDE_SRC_DJ ? djv : src == SDE_SRC_DN ? dnv : R(0);
                                        const R term = A::mul(A2[e][i], dz);
                                        s = i == 0 ? term : A::add(s, term);
                                    }
                                const R v = A::add(xs[e], s);
#pragma unroll
                                for (int m = 0; m < MAXM; ++m)
                                    if (m == mm) nx[m] = v;
                            }
                        }
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) st[m] = nx[m];
                    } else if (MODEL == SDE_MODEL_CIR) {   // k*(theta - x+), xi*sqrt(x+)
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) {
                            const R xp = fmax(st[m], R(0));
                            const R drift = A::mul(c0[m], A::sub(c1[m], xp));
                            const R vol = A::mul(c2[m], A::sqrt_(xp));
                            st[m] = A::add(st[m], A::add(A::mul(drift, dt), A::mul(vol, dW[m])));
                        }
                    } else {  // HESTON: first half log-price, second half variance
                        // Heston kernels run with group_size == MAXM exactly
                        constexpr int h = MAXM / 2;
                        R nx[MAXM];
#pragma unroll
                        for (int i = 0; i < h; ++i) {
                            const R y = st[h + i];
                            if (y < R(0)) negc[i] += 1;
                            const R yp = fmax(y, R(0));
                            const R sqy = A::sqrt_(yp);
                            // x part: mu - sigma*sigma*y+/2, sigma*sqrt(y+)
                            const R mu = c0[i], sg = c1[i];
                            const R adt = A::sub(mu, A::mul(A::mul(A::mul(sg, sg), yp), R(0.5)));
                            const R adw = A::mul(sg, sqy);
                            nx[i] = A::add(st[i], A::add(A::mul(adt, dt), A::mul(adw, dW[i])));
                            // y part: k*(theta - y+), xi*sqrt(y+)
                            const R kk = c0[h + i], th = c1[h + i], xi = c2[h + i];
                            const R bdt = A::mul(kk, A::sub(th, yp));
                            const R bdw = A::mul(xi, sqy);
                            nx[h + i] = A::add(y, A::add(A::mul(bdt, dt), A::mul(bdw, dW[h + i])));
                        }
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) st[m] = nx[m];
                    }
                    };
                    euler(st, dW, negc);
                    if constexpr (ANTI) {   // the antithetic path: exactly opposite increments
                        R dWn[MAXM];
#pragma unroll
                        for (int m = 0; m < MAXM; ++m) dWn[m] = -dW[m];
                        euler(st1, dWn, negc1);
                    }
                };
                if (RUNS && a.runs) {
                    // runs of steps with one dt, ending where a row is stored
                    // and split where a checkpoint falls (bit 0 of run.w): no
                    // per-step row test or dt load
#pragma unroll 1
                    for (int ri = 0; ri < a.n_runs; ++ri) {
                        const int4 run = __ldg(a.runs + ri);
                        if (a.ckpt && (run.w & 1)) ck_store();
                        const R dt = a.dt[run.x], sq = a.sqdt[run.x];
#pragma unroll UNROLL
                        for (int k = run.x; k < run.y; ++k) step_k(k, dt, sq);
                        if (run.z >= 0) store(run.z, false);
                    }
                } else {
                    int kc = 0;   // steps to the next checkpoint
#pragma unroll UNROLL
                    for (int k = 0; k < n_steps; ++k) {
                        if (a.ckpt) {
                            if (kc == 0) {
                                ck_store();
                                kc = a.ckpt_seg;
                            }
                            --kc;
                        }
                        step_k(k, a.dt[k], a.sqdt[k]);
                        const int r = a.out_row[k + 1];
                        if (r >= 0) store(r, false);
                    }
                }
            }
            if (MODEL == SDE_MODEL_HESTON && a.neg_count) {
                constexpr int h = MAXM / 2;
#pragma unroll
                for (int i = 0; i < h; ++i) {
                    a.neg_count[((int64_t)g * h + i) * a.paths + p] = negc[i];
                    if constexpr (ANTI) a.neg_count[((int64_t)g * h + i) * a.paths + p + npath] = negc1[i];
                }
            }
            if (JUMPS && a.jump_count) {
#pragma unroll
                for (int m = 0; m < MAXM; ++m)
                    if (m < M) {
                        a.jump_count[((int64_t)g * M + m) * a.paths + p] = jcnt[m];
                        if constexpr (ANTI) a.jump_count[((int64_t)g * M + m) * a.paths + p + npath] = jcnt[m];
                    }
            }
        }
        if (do_stats) {
#pragma unroll
            for (int i = 0; i < NA; ++i)
#pragma unroll
                for (int m = 0; m < MAXM; ++m) {
                    if (m < a.opg)
                        block_round_stats<R>(svs[i][m][threadIdx.x], act, a.strikes, a.n_strikes, part[m], red);
                }
        }
    }
    if (do_stats) {
        __syncthreads();
        if (threadIdx.x < a.opg && threadIdx.x < MAXM) {
            double *dst = a.partials +
                          (((int64_t)g * gridDim.x + blockIdx.x) * a.opg + threadIdx.x) * NPART;
            for (int i = 0; i < NPART; ++i) dst[i] = part[threadIdx.x][i];
        }
    }
}

// sqrt(2 ln 2), carried by the c coefficients of the FP32 table kernels
#define SDE_SQRT_2LN2 1.1774100225154747

// per-step coefficients of the FP32 LINEAR / OU kernels, [steps][groups][2][MAXM]
// (see FwdArgs::coef), from the FP64 grid and parameters with explicitly
// rounded FP64 operations (the host builds the same rows with the same
// operations); OU also writes the shift table FwdArgs::tshift
static __global__ void __launch_bounds__(BLOCK)
coef_table_kernel(const double *tt, int n_steps, const double *x0, const double *prm, int groups, int M,
                  int maxm, int model, float *coef, float *tshift) {
    const int64_t i = (int64_t)blockIdx.x * BLOCK + threadIdx.x;
    const int64_t n = (int64_t)n_steps * groups * maxm;
    if (i >= n) return;
    const int m = (int)(i % maxm);
    const int64_t kg = i / maxm;
    const int g = (int)(kg % groups);
    const int k = (int)(kg / groups);
    float *t = coef + kg * 2 * maxm;
    const int W = groups * M, w = g * M + m;
    if (k == 0 && model == SDE_MODEL_OU) {
        tshift[g * 2 * maxm + m] = m < M ? (float)prm[W + w] : 0.0f;
        tshift[(g * 2 + 1) * maxm + m] = m < M ? (float)__dsub_rn(x0[w], prm[W + w]) : 0.0f;
    }
    if (m >= M) {
        t[m] = 0.0f;
        t[maxm + m] = 0.0f;
        return;
    }
    const double dt = __dsub_rn(tt[k + 1], tt[k]);
    const double sq = __dsqrt_rn(fabs(dt));
    const int ip = model == SDE_MODEL_OU ? 2 : 1;   // sigma
    t[m] = (float)__dmul_rn(prm[w], dt);
    t[maxm + m] = (float)__dmul_rn(__dmul_rn(prm[ip * W + w], sq), SDE_SQRT_2LN2);
}

#ifndef __CUDACC_RTC__
// launcher signature shared by the instantiation units
template <typename R>
using FwdLauncher = void (*)(const FwdArgs<R> &, dim3, cudaStream_t);

template <typename R, int MODEL, int MAXM, bool INJECT, bool JUMPS, bool TDEP = false, bool ANTI = false>
void launch_fwd(const FwdArgs<R> &a, dim3 grid, cudaStream_t s) {
    sde_fwd_kernel<R, MODEL, MAXM, INJECT, JUMPS, TDEP, ANTI><<<grid, BLOCK, 0, s>>>(a);
}

template <typename R, int MODEL, int MAXM, bool INJECT, bool JUMPS, bool TDEP = false, bool ANTI = false>
int fwd_max_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sde_fwd_kernel<R, MODEL, MAXM, INJECT, JUMPS, TDEP, ANTI>,
                                                  BLOCK, 0);
    return n;
}

// The FP32 LINEAR / OU kernels of device noise without jumps, antithetic
// paths or time-dependent coefficients (sde_fwd_tab_kernel, sde_tab.cuh)
// store the summarised row and reduce it in a second launch: a summary
// needs FwdArgs::stats_vals, or xx in device memory
inline bool fwd_summary_from_row(bool fp32, int model, bool inject, bool jumps, bool anti, bool tdep, bool user) {
    return fp32 && !inject && !jumps && !anti && !tdep && !user &&
           (model == SDE_MODEL_LINEAR || model == SDE_MODEL_OU);
}

// dispatch lookup implemented in the instantiation units (fwd_*.cu)
FwdLauncher<double> find_fwd_f64_linear(int model, int maxm, bool inject, bool jumps, int *bps);
FwdLauncher<double> find_fwd_f64_ou_heston(int model, int maxm, bool inject, bool jumps, int *bps);
FwdLauncher<float> find_fwd_f32_linear(int model, int maxm, bool inject, bool jumps, int *bps);
FwdLauncher<float> find_fwd_f32_ou_heston(int model, int maxm, bool inject, bool jumps, int *bps);
// FP32 device-noise kernels with time-dependent coefficients: OU with a
// time-dependent theta, Heston
FwdLauncher<float> find_fwd_f32_tdep(int model, int maxm, int *bps);
// CIR kernels (fwd_cir.cu): plain, time-dependent (FP32), antithetic
FwdLauncher<float> find_fwd_f32_cir(int maxm, bool inject, bool tdep, bool anti, int *bps);
FwdLauncher<double> find_fwd_f64_cir(int maxm, bool inject, bool anti, int *bps);
// user-SDE kernels (fwd_user_*.cu): device or injected noise; sys: systems
// of equations (SDE_MODEL_USER_SYS)
FwdLauncher<float> find_fwd_f32_user(int maxm, bool inject, bool sys, bool jumps, int *bps);
FwdLauncher<double> find_fwd_f64_user(int maxm, bool inject, bool sys, bool jumps, int *bps);
// the same with dn / dj terms (fwd_user_jump_*.cu: single equations;
// fwd_user_jump_sys_*.cu: systems)
FwdLauncher<float> find_fwd_f32_user_jump(int maxm, bool inject, bool sys, int *bps);
FwdLauncher<double> find_fwd_f64_user_jump(int maxm, bool inject, bool sys, int *bps);
FwdLauncher<float> find_fwd_f32_user_jump_sys(int maxm, bool inject, int *bps);
FwdLauncher<double> find_fwd_f64_user_jump_sys(int maxm, bool inject, int *bps);
// antithetic kernels (device noise, groups of up to 8 states)
FwdLauncher<float> find_fwd_f32_anti(int model, int maxm, bool jumps, int *bps);
// FP32 antithetic kernels with per-step coefficients and correlation factors
// (fwd_anti_tdep_f32.cu)
FwdLauncher<float> find_fwd_f32_anti_tdep(int model, int maxm, bool jumps, int *bps);
FwdLauncher<double> find_fwd_f64_anti(int model, int maxm, bool jumps, int *bps);
#endif  // !__CUDACC_RTC__

}  // namespace sdegpu
