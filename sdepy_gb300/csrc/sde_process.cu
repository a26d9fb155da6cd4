// Process post-processing on the device: summaries across paths of written
// process values (process.pmin / pmax / psum / pmean / pvar / pstd,
// sdepy/infrastructure.py:833-889), the empirical cdf (process.cdf,
// :1169-1212) and the empirical characteristic function (process.chf,
// :1125-1167) at timeline points or at time points interpolated as
// process.interp does (:544-613).
//
// Data: x [n_rows][n_vars][paths], paths innermost, f64 or f32, in device
// memory, in page-locked host memory (read in place over the host link) or
// in pageable host memory (copied to the device first).  A *series* is one
// (time point, value component): n_t * n_vars series of `paths` values.
//
// Kernels (each value read once):
//   moments: FP64 sums about a per-series shift (the mean of the first
//     finite values), per-block partials merged in fixed order --
//     deterministic for a given launch geometry;
//   cdf: each value finds by binary search the first threshold it does not
//     exceed (thresholds sorted on the host, in shared memory), a
//     shared-memory histogram of those positions, and a prefix sum per
//     series gives the counts -- exact integers;
//   chf: chunks of values staged in shared memory as FP64, FP64 sincos of
//     u_j * v for tiles of u, per-block sums in shared memory, partials
//     merged in fixed order.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <type_traits>
#include <vector>

#include "fp64_tables.h"
#include "sdepy_gb300.h"
#include "sde_runtime.h"

using namespace sdegpu;

namespace {

constexpr int PB = 256;           // threads per block
constexpr int SHIFT_N = 64;       // leading values averaged into a series' shift
constexpr int CHF_CHUNK = 4096;   // values staged per chf block iteration
constexpr int CHF_UT = 8;         // u values per chf register tile (at most)
constexpr int CDF_SMEM_MAX = 8192;  // thresholds held in shared memory
constexpr int CDF_ILP = 4;          // values searched side by side per thread

#define PCU(call)                                                                        \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            char m_[512];                                                                \
            snprintf(m_, sizeof m_, "%s failed: %s", #call, cudaGetErrorString(e_));      \
            return rt_fail(SDE_ERR_CUDA, m_);                                            \
        }                                                                                \
    } while (0)

__device__ __forceinline__ bool nan_bits(float v) {
    return (__float_as_uint(v) & 0x7fffffffu) > 0x7f800000u;
}
__device__ __forceinline__ bool nan_bits(double v) {
    return ((unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}
__device__ __forceinline__ bool finite_bits(float v) {
    return (__float_as_uint(v) & 0x7f800000u) != 0x7f800000u;
}
__device__ __forceinline__ bool finite_bits(double v) {
    return ((unsigned long long)__double_as_longlong(v) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}

// one time point of the read: row lo, or the interpolation of rows lo / hi
struct TimePoint {
    int64_t lo, hi;
    double wl, wh;
};

// value p of series (time point tp, component var): row lo itself, or
// (INTERP) the FP64 value wh * x_hi + wl * x_lo (no contraction) rounded to
// R.  Callers branch on tp.hi once per series, so that the value loop of a
// timeline read carries no interpolation arithmetic.
template <bool INTERP, typename R>
__device__ __forceinline__ R read_value(const R *__restrict__ xl_row, const R *__restrict__ xh_row,
                                        const TimePoint &tp, int64_t p) {
    const R xl = __ldg(xl_row + p);
    if (!INTERP) return xl;
    const R xh = __ldg(xh_row + p);
    return (R)__dadd_rn(__dmul_rn(tp.wh, (double)xh), __dmul_rn(tp.wl, (double)xl));
}

// order-preserving integer key of a double (the IEEE bit pattern with the
// magnitude bits of negative numbers flipped; -0 maps to +0's key): key
// comparisons agree with FP64 comparisons of non-NaN values and run on the
// integer pipes (GB300 issues FP64 at 1/64 of the FP32 rate)
__host__ __device__ __forceinline__ long long order_key(long long b) {
    if ((b & 0x7fffffffffffffffLL) == 0) return 0;
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ long long order_key(double v) { return order_key(__double_as_longlong(v)); }
__device__ __forceinline__ double key_value(long long k) {
    return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL));
}

// Knuth's TwoSum in FP32: s + e == a + b exactly (round-to-nearest, no
// overflow)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// ---------------------------------------------------------------------------
// moments
// ---------------------------------------------------------------------------
// shift[s] = mean of the finite values among the first SHIFT_N of series s,
// rounded to R (0 when none is finite); one warp per series, fixed
// reduction order
template <typename R>
__global__ void __launch_bounds__(PB) pmom_shift_kernel(const R *__restrict__ x, int64_t n_series,
                                                        int64_t paths, double *__restrict__ shift) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (PB / 32);
    for (int64_t s = (int64_t)blockIdx.x * (PB / 32) + threadIdx.x / 32; s < n_series; s += warps) {
        double sum = 0.0;
        int cnt = 0;
        for (int k = lane; k < SHIFT_N && k < paths; k += 32) {
            const R v = __ldg(x + s * paths + k);
            if (finite_bits(v)) {
                sum += (double)v;
                ++cnt;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            sum += __shfl_xor_sync(0xffffffffu, sum, o);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        if (lane == 0) shift[s] = cnt ? (double)(R)(sum / cnt) : 0.0;
    }
}

// Per-thread accumulation of one series' values about the shift sh: sums of
// d = w - sh and d^2 where w is the value, or sh itself for a non-finite
// value (infinities and NaN are accounted for through min / max and the NaN
// count); min, max (NaN ignored) and the NaN count.
//
// FP32 values: d is formed exactly as dh + dl (TwoSum), d^2 as p + q (the
// FMA product error, dl^2 dropped: below 2^-48 d^2); the sums are carried
// as FP32 pairs (compensated with TwoSum) over runs of 32 values and then
// added to FP64 totals -- FP64-class accuracy from FP32 instructions
// (differences of squares above FLT_MAX, |v - sh| > 1.8e19, overflow).
// FP64 values: three FP64 operations per value; min / max on order keys.
template <typename R> struct MomAcc;

template <> struct MomAcc<float> {
    double S1 = 0.0, S2 = 0.0;
    float a1 = 0.f, c1 = 0.f, a2 = 0.f, c2 = 0.f;
    float mn = INFINITY, mx = -INFINITY;
    unsigned int nan = 0;
    float sh;
    __device__ explicit MomAcc(double shift) : sh((float)shift) {}
    __device__ __forceinline__ void add(float v) {
        nan += nan_bits(v);
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
        const float w = finite_bits(v) ? v : sh;
        float dh, dl, t, e;
        two_sum(w, -sh, dh, dl);
        two_sum(a1, dh, t, e);
        a1 = t;
        c1 = __fadd_rn(c1, __fadd_rn(e, dl));
        const float pr = __fmul_rn(dh, dh);
        const float q = __fmaf_rn(__fmul_rn(2.f, dh), dl, __fmaf_rn(dh, dh, -pr));
        two_sum(a2, pr, t, e);
        a2 = t;
        c2 = __fadd_rn(c2, __fadd_rn(e, q));
    }
    __device__ __forceinline__ void flush() {
        S1 += (double)a1 + (double)c1;
        S2 += (double)a2 + (double)c2;
        a1 = c1 = a2 = c2 = 0.f;
    }
    __device__ __forceinline__ double vmin() const { return (double)mn; }
    __device__ __forceinline__ double vmax() const { return (double)mx; }
};

template <> struct MomAcc<double> {
    double S1 = 0.0, S2 = 0.0;
    long long kmn = 0x7fffffffffffffffLL, kmx = (long long)0x8000000000000000ULL;
    unsigned int nan = 0;
    double sh;
    __device__ explicit MomAcc(double shift) : sh(shift) {}
    __device__ __forceinline__ void add(double v) {
        const long long b = __double_as_longlong(v);
        const bool isnan = (b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
        nan += isnan;
        const long long k = order_key(b);
        if (!isnan) {
            kmn = k < kmn ? k : kmn;
            kmx = k > kmx ? k : kmx;
        }
        const double w = finite_bits(v) ? v : sh;
        const double d = __dsub_rn(w, sh);
        S1 = __dadd_rn(S1, d);
        S2 = __fma_rn(d, d, S2);
    }
    __device__ __forceinline__ void flush() {}
    __device__ __forceinline__ double vmin() const {
        return kmn == 0x7fffffffffffffffLL ? (double)INFINITY : key_value(kmn);
    }
    __device__ __forceinline__ double vmax() const {
        return kmx == (long long)0x8000000000000000ULL ? -(double)INFINITY : key_value(kmx);
    }
};

// per-block partials [n_series][nch][6] = (n, S1, S2, min, max, NaN count)
// of the chunk [bx * chunk, min(paths, (bx + 1) * chunk)) of each series
template <typename R>
__global__ void __launch_bounds__(PB) pmom_kernel(const R *__restrict__ x, int64_t n_series, int64_t paths,
                                                  int64_t chunk, int nch, const double *__restrict__ shift,
                                                  double *__restrict__ part) {
    __shared__ double red[4][PB / 32];
    __shared__ unsigned int redn[PB / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t c0 = (int64_t)blockIdx.x * chunk;
    const int64_t c1 = c0 + chunk < paths ? c0 + chunk : paths;
    for (int64_t s = blockIdx.y; s < n_series; s += gridDim.y) {
        const R *__restrict__ p = x + s * paths;
        MomAcc<R> acc(shift[s]);
        int run = 0;
        int64_t i = c0 + threadIdx.x;
        for (; i + 3 * PB < c1; i += 4 * PB) {   // whole groups of 4 values per thread
            R v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = __ldg(p + i + u * PB);
#pragma unroll
            for (int u = 0; u < 4; ++u) acc.add(v[u]);
            if (++run == 8) {   // 32 values
                acc.flush();
                run = 0;
            }
        }
        for (; i < c1; i += PB) acc.add(__ldg(p + i));   // at most 3 more
        acc.flush();
        double s1 = acc.S1, s2 = acc.S2, m = acc.vmin(), M = acc.vmax();
        unsigned int nan = acc.nan;
        for (int o = 16; o > 0; o >>= 1) {
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
            m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
            M = fmax(M, __shfl_xor_sync(0xffffffffu, M, o));
            nan += __shfl_xor_sync(0xffffffffu, nan, o);
        }
        if (lane == 0) {
            red[0][warp] = s1;
            red[1][warp] = s2;
            red[2][warp] = m;
            red[3][warp] = M;
            redn[warp] = nan;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double a = 0.0, b = 0.0, lo = INFINITY, hi = -INFINITY;
            unsigned long long nn = 0;
            for (int w = 0; w < PB / 32; ++w) {
                a += red[0][w];
                b += red[1][w];
                lo = fmin(lo, red[2][w]);
                hi = fmax(hi, red[3][w]);
                nn += redn[w];
            }
            double *o = part + (s * nch + blockIdx.x) * 6;
            o[0] = (double)(c1 > c0 ? c1 - c0 : 0);
            o[1] = a;
            o[2] = b;
            o[3] = lo;
            o[4] = hi;
            o[5] = (double)nn;
        }
        __syncthreads();
    }
}

// out[s][6] = (sum, mean, M2, min, max, NaN count) from the partials, in
// fixed order.  Non-finite values: any NaN makes every statistic NaN;
// otherwise +inf (-inf) makes the sum and mean +inf (-inf), both NaN, and
// M2 NaN -- numpy's results for such samples.
__global__ void pmom_final_kernel(const double *__restrict__ part, int64_t n_series, int nch,
                                  const double *__restrict__ shift, double *__restrict__ out) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_series) return;
    double n = 0.0, s1 = 0.0, s2 = 0.0, lo = INFINITY, hi = -INFINITY, nan = 0.0;
    for (int b = 0; b < nch; ++b) {
        const double *q = part + (s * nch + b) * 6;
        n += q[0];
        s1 += q[1];
        s2 += q[2];
        lo = fmin(lo, q[3]);
        hi = fmax(hi, q[4]);
        nan += q[5];
    }
    const double sh = shift[s];
    double *o = out + s * SDE_PMOM_STRIDE;
    const double qnan = (double)NAN;
    const bool pinf = hi == (double)INFINITY, ninf = lo == -(double)INFINITY;
    if (nan > 0.0) {
        o[0] = o[1] = o[2] = o[3] = o[4] = qnan;
    } else if (pinf || ninf) {
        o[0] = o[1] = pinf && ninf ? qnan : pinf ? (double)INFINITY : -(double)INFINITY;
        o[2] = qnan;
        o[3] = lo;
        o[4] = hi;
    } else {
        o[0] = sh * n + s1;
        o[1] = sh + s1 / n;
        const double m2 = s2 - s1 * (s1 / n);
        o[2] = m2 < 0.0 ? 0.0 : m2;
        o[3] = lo;
        o[4] = hi;
    }
    o[5] = nan;
}

// ---------------------------------------------------------------------------
// cdf
// ---------------------------------------------------------------------------
// thresholds as the kernels compare them: FP32 data against floats (the
// largest float not above each FP64 threshold: v <= x exactly when v <= that
// float), FP64 data against order keys
template <typename R> struct Thr;
template <> struct Thr<float> {
    using T = float;
    __device__ static __forceinline__ float key(float v) { return v; }
};
template <> struct Thr<double> {
    using T = long long;
    __device__ static __forceinline__ long long key(double v) { return order_key(v); }
};

// counts[s][k] += number of values of series s whose first threshold not
// below them is thr[k].  thr holds the n_thr sorted NaN-free thresholds
// followed by sentinels (above every value) up to n_pad = 2^m - 1 entries,
// so that the position is found by m halving steps without branches.
// Values above every threshold and NaN values are not counted.  Each thread
// runs the searches of CDF_ILP values side by side (independent chains of
// shared-memory loads).  SMEM: thresholds and counters in shared memory,
// shared atomics; else (n_thr above CDF_SMEM_MAX) thresholds in global
// memory and global atomics.
template <typename R, bool SMEM>
__global__ void __launch_bounds__(PB) cdf_kernel(const R *__restrict__ x, int64_t n_vars, int64_t paths,
                                                 const TimePoint *__restrict__ tps, int64_t n_series,
                                                 const typename Thr<R>::T *__restrict__ thr_g, int n_thr,
                                                 int n_pad, int64_t chunk,
                                                 unsigned long long *__restrict__ counts) {
    using T = typename Thr<R>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned int *hist = reinterpret_cast<unsigned int *>(smem_raw);
    T *thr_s = reinterpret_cast<T *>(smem_raw + (((size_t)n_thr * 4 + 15) & ~(size_t)15));
    const T *thr = SMEM ? thr_s : thr_g;
    if (SMEM)
        for (int k = threadIdx.x; k < n_pad; k += PB) thr_s[k] = thr_g[k];
    const int top = (n_pad + 1) >> 1;
    const int64_t c0 = (int64_t)blockIdx.x * chunk;
    const int64_t c1 = c0 + chunk < paths ? c0 + chunk : paths;
    for (int64_t s = blockIdx.y; s < n_series; s += gridDim.y) {
        const TimePoint tp = tps[s / n_vars];
        const int64_t var = s % n_vars;
        const R *xl = x + (tp.lo * n_vars + var) * paths;
        const R *xh = tp.hi < 0 ? xl : x + (tp.hi * n_vars + var) * paths;
        if (SMEM) {
            for (int k = threadIdx.x; k < n_thr; k += PB) hist[k] = 0;
            __syncthreads();
        }
        auto tally = [&](int b, bool ok) {
            if (ok && b < n_thr) {
                if (SMEM) atomicAdd(hist + b, 1u);
                else atomicAdd(counts + s * n_thr + b, 1ull);
            }
        };
        auto count = [&](auto interp) {
            constexpr bool IP = decltype(interp)::value;
            int64_t i = c0 + threadIdx.x;
            for (; i + (CDF_ILP - 1) * PB < c1; i += CDF_ILP * PB) {
                T kv[CDF_ILP];
                bool ok[CDF_ILP];
                int b[CDF_ILP];
#pragma unroll
                for (int u = 0; u < CDF_ILP; ++u) {
                    const R v = read_value<IP>(xl, xh, tp, i + u * PB);
                    ok[u] = !nan_bits(v);
                    kv[u] = Thr<R>::key(v);
                    b[u] = 0;   // the number of thresholds below v
                }
                for (int step = top; step > 0; step >>= 1)
#pragma unroll
                    for (int u = 0; u < CDF_ILP; ++u) b[u] += thr[b[u] + step - 1] < kv[u] ? step : 0;
#pragma unroll
                for (int u = 0; u < CDF_ILP; ++u) tally(b[u], ok[u]);
            }
            for (; i < c1; i += PB) {
                const R v = read_value<IP>(xl, xh, tp, i);
                const T kv = Thr<R>::key(v);
                int b = 0;
                for (int step = top; step > 0; step >>= 1) b += thr[b + step - 1] < kv ? step : 0;
                tally(b, !nan_bits(v));
            }
        };
        if (tp.hi < 0) count(std::false_type{});
        else count(std::true_type{});
        if (SMEM) {
            __syncthreads();
            for (int k = threadIdx.x; k < n_thr; k += PB)
                if (hist[k]) atomicAdd(counts + s * n_thr + k, (unsigned long long)hist[k]);
            __syncthreads();
        }
    }
}

// out[t][perm[k]][var] = (counts[s][0] + ... + counts[s][k]) / paths
__global__ void cdf_final_kernel(const unsigned long long *__restrict__ counts, int64_t n_series,
                                 int n_thr, const int64_t *__restrict__ perm, int64_t n_vars, int64_t n_x,
                                 int64_t paths, double *__restrict__ out) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_series) return;
    const int64_t t = s / n_vars, var = s % n_vars;
    unsigned long long run = 0;
    for (int k = 0; k < n_thr; ++k) {
        run += counts[s * n_thr + k];
        out[(t * n_x + perm[k]) * n_vars + var] = (double)run / (double)paths;
    }
}

// ---------------------------------------------------------------------------
// chf
// ---------------------------------------------------------------------------
// sin a and cos a in FP64 (|a| <= 2^20; larger or non-finite a go to CUDA's
// sincos): Cody-Waite reduction a = k pi/64 + r with pi/64 split into two
// doubles (a - k c1 is exact, the c2 term's rounding is below an ulp of r;
// the third part of the split is below 2^-110 k), sin and cos of k pi/64
// from the angle-addition table of the Box-Muller transform (entries
// correctly rounded), the Taylor series of sin r to r^7 and of cos r - 1 to
// r^6 (|r| <= pi/128: the next terms are below 2^-60 relative), and the
// table values added last: s = S + (C sin r + S (cos r - 1)).  About 1 ulp,
// 15 FP64 operations.
__device__ __forceinline__ void sincos_tab(double a, double &s, double &c) {
    if (!(fabs(a) <= 0x1p20)) {
        sincos(a, &s, &c);
        return;
    }
    const double big = 0x1.8p52;   // adding it rounds to an integer
    const double t = __fma_rn(a, F64_INV_PIO64, big);
    const double kd = __dsub_rn(t, big);
    const int idx = (__double2loint(t) + 64) & 127;   // k mod 128 as n + 64, n in [-64, 64)
    double r = __fma_rn(-kd, F64_PIO64_1, a);
    r = __fma_rn(-kd, F64_PIO64_2, r);
    const double r2 = __dmul_rn(r, r);
    double ps = -1.0 / 5040.0;
    ps = __fma_rn(ps, r2, 1.0 / 120.0);
    ps = __fma_rn(ps, r2, -1.0 / 6.0);
    const double sr = __fma_rn(__dmul_rn(r, r2), ps, r);
    double pc = -1.0 / 720.0;
    pc = __fma_rn(pc, r2, 1.0 / 24.0);
    pc = __fma_rn(pc, r2, -0.5);
    const double cm1 = __dmul_rn(r2, pc);
    const double S = __ldg(&F64_SINPI_N[idx]), C = __ldg(&F64_COSPI_N[idx]);
    s = __dadd_rn(S, __fma_rn(C, sr, __dmul_rn(S, cm1)));
    c = __dadd_rn(C, __fma_rn(-S, sr, __dmul_rn(C, cm1)));
}

// part[s][bx][j][2] = sum over the values of series s handled by block bx
// of (cos(u_j v), sin(u_j v)); block bx handles chunks bx, bx + nch, ...;
// UT values of u per register tile (1, 2, 4 or 8: no padding below 8 u)
template <typename R, int UT>
__global__ void __launch_bounds__(PB) chf_kernel(const R *__restrict__ x, int64_t n_vars, int64_t paths,
                                                 const TimePoint *__restrict__ tps, int64_t n_series,
                                                 const double *__restrict__ u, int n_u, int nch,
                                                 double *__restrict__ part) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *vals = reinterpret_cast<double *>(smem_raw);              // [CHF_CHUNK]
    double *acc = vals + CHF_CHUNK;                                     // [n_u][2]
    __shared__ double red[PB / 32][2 * UT];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t s = blockIdx.y; s < n_series; s += gridDim.y) {
        const TimePoint tp = tps[s / n_vars];
        const int64_t var = s % n_vars;
        const R *xl = x + (tp.lo * n_vars + var) * paths;
        const R *xh = tp.hi < 0 ? xl : x + (tp.hi * n_vars + var) * paths;
        for (int k = threadIdx.x; k < 2 * n_u; k += PB) acc[k] = 0.0;
        for (int64_t c0 = (int64_t)blockIdx.x * CHF_CHUNK; c0 < paths; c0 += (int64_t)nch * CHF_CHUNK) {
            const int cn = (int)(paths - c0 < CHF_CHUNK ? paths - c0 : CHF_CHUNK);
            __syncthreads();
            if (tp.hi < 0)
                for (int k = threadIdx.x; k < cn; k += PB) vals[k] = (double)read_value<false>(xl, xh, tp, c0 + k);
            else
                for (int k = threadIdx.x; k < cn; k += PB) vals[k] = (double)read_value<true>(xl, xh, tp, c0 + k);
            __syncthreads();
            for (int j0 = 0; j0 < n_u; j0 += UT) {
                double c[UT], sn[UT], uj[UT];
#pragma unroll
                for (int q = 0; q < UT; ++q) {
                    c[q] = 0.0;
                    sn[q] = 0.0;
                    uj[q] = j0 + q < n_u ? __ldg(u + j0 + q) : 0.0;
                }
                for (int k = threadIdx.x; k < cn; k += PB) {
                    const double v = vals[k];
#pragma unroll
                    for (int q = 0; q < UT; ++q) {
                        double sv, cv;
                        sincos_tab(__dmul_rn(uj[q], v), sv, cv);
                        c[q] += cv;
                        sn[q] += sv;
                    }
                }
#pragma unroll
                for (int q = 0; q < UT; ++q)
                    for (int o = 16; o > 0; o >>= 1) {
                        c[q] += __shfl_xor_sync(0xffffffffu, c[q], o);
                        sn[q] += __shfl_xor_sync(0xffffffffu, sn[q], o);
                    }
                if (lane == 0)
#pragma unroll
                    for (int q = 0; q < UT; ++q) {
                        red[warp][2 * q] = c[q];
                        red[warp][2 * q + 1] = sn[q];
                    }
                __syncthreads();
                if (threadIdx.x < 2 * UT && j0 + threadIdx.x / 2 < n_u) {
                    double a = 0.0;
                    for (int w = 0; w < PB / 32; ++w) a += red[w][threadIdx.x];
                    acc[2 * j0 + threadIdx.x] += a;
                }
                __syncthreads();
            }
        }
        __syncthreads();
        double *o = part + (s * nch + blockIdx.x) * 2 * (int64_t)n_u;
        for (int k = threadIdx.x; k < 2 * n_u; k += PB) o[k] = acc[k];
        __syncthreads();
    }
}

// out[t][j][var][2] = (sum over blocks of part[s][b][j]) / paths, fixed order
__global__ void chf_final_kernel(const double *__restrict__ part, int64_t n_series, int nch, int n_u,
                                 int64_t n_vars, int64_t paths, double *__restrict__ out) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;   // (s, j)
    if (q >= n_series * n_u) return;
    const int64_t s = q / n_u, j = q % n_u;
    const int64_t t = s / n_vars, var = s % n_vars;
    double c = 0.0, sn = 0.0;
    for (int b = 0; b < nch; ++b) {
        const double *p = part + ((s * nch + b) * n_u + j) * 2;
        c += p[0];
        sn += p[1];
    }
    double *o = out + ((t * n_u + j) * n_vars + var) * 2;
    o[0] = c / (double)paths;
    o[1] = sn / (double)paths;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// device address of the input: itself on the device, page-locked host
// memory in place, other host memory through a copy into scratch slot 0
int input_ptr(const RtCall &c, const void *x, size_t bytes, int on_device, const void **dx) {
    if (on_device) {
        *dx = x;
        return SDE_OK;
    }
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, x) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
        pa.devicePointer != nullptr) {
        *dx = pa.devicePointer;
        return SDE_OK;
    }
    cudaGetLastError();
    void *p;
    int rc = rt_scratch(0, bytes, &p);
    if (rc) return rc;
    PCU(cudaMemcpyAsync(p, x, bytes, cudaMemcpyHostToDevice, c.st));
    *dx = p;
    return SDE_OK;
}

int check_dims(const void *x, int64_t n_rows, int64_t n_vars, int64_t paths, const void *out) {
    if (!x || !out) return rt_fail(SDE_ERR_INVALID, "null data or output pointer");
    if (n_rows < 1 || n_vars < 1 || paths < 1)
        return rt_fail(SDE_ERR_INVALID, "process summaries need rows, values and paths >= 1");
    if (n_rows > ((int64_t)1 << 40) / n_vars || n_rows * n_vars > ((int64_t)1 << 40) / paths)
        return rt_fail(SDE_ERR_INVALID, "process too large");
    return SDE_OK;
}

// time points: the rows themselves when at is NULL, else checked copies
int time_points(const SdeTimes *at, int64_t n_rows, std::vector<TimePoint> *tp) {
    if (!at) {
        tp->resize(n_rows);
        for (int64_t i = 0; i < n_rows; ++i) (*tp)[i] = TimePoint{i, -1, 0.0, 0.0};
        return SDE_OK;
    }
    if (at->n_t < 1 || !at->lo || !at->hi || !at->wl || !at->wh)
        return rt_fail(SDE_ERR_INVALID, "bad time points");
    tp->resize(at->n_t);
    for (int64_t i = 0; i < at->n_t; ++i) {
        const int64_t lo = at->lo[i], hi = at->hi[i];
        if (lo < 0 || lo >= n_rows || hi >= n_rows)
            return rt_fail(SDE_ERR_INVALID, "time point row out of range");
        (*tp)[i] = TimePoint{lo, hi < 0 ? -1 : hi, at->wl[i], at->wh[i]};
    }
    return SDE_OK;
}

unsigned grid_y(int64_t n_series) { return (unsigned)(n_series < 65535 ? n_series : 65535); }

template <typename R>
int moments_impl(const void *x, int on_device, int64_t n_series, int64_t paths, double *out) {
    int rc;
    if ((rc = check_dims(x, n_series, 1, paths, out))) return rc;
    std::lock_guard<std::mutex> lk(rt_mutex());
    RtCall c;
    if ((rc = rt_begin(&c))) return rc;
    const void *dx;
    if ((rc = input_ptr(c, x, sizeof(R) * n_series * paths, on_device, &dx))) return rc;
    // blocks per series: enough for 8 per SM in all, chunks of >= 4 * PB values
    const int64_t target = (int64_t)c.sms * 8;
    int64_t nch = (target + n_series - 1) / n_series;
    const int64_t maxch = (paths + 4 * PB - 1) / (4 * PB);
    if (nch > maxch) nch = maxch;
    if (nch < 1) nch = 1;
    const int64_t chunk = (paths + nch - 1) / nch;
    nch = (paths + chunk - 1) / chunk;
    void *part, *res;
    if ((rc = rt_scratch(2, sizeof(double) * (n_series * nch * 6 + n_series), &part))) return rc;
    if ((rc = rt_scratch(3, sizeof(double) * n_series * SDE_PMOM_STRIDE, &res))) return rc;
    double *shift = (double *)part + n_series * nch * 6;
    const R *xr = (const R *)dx;
    if (c.timing) PCU(cudaEventRecord(c.ev0, c.st));
    pmom_shift_kernel<R><<<(unsigned)std::min<int64_t>((n_series + 7) / 8, 65535), PB, 0, c.st>>>(
        xr, n_series, paths, shift);
    pmom_kernel<R><<<dim3((unsigned)nch, grid_y(n_series)), PB, 0, c.st>>>(xr, n_series, paths, chunk, (int)nch,
                                                                           shift, (double *)part);
    pmom_final_kernel<<<(unsigned)((n_series + 255) / 256), 256, 0, c.st>>>((const double *)part, n_series,
                                                                            (int)nch, shift, (double *)res);
    if (c.timing) PCU(cudaEventRecord(c.ev1, c.st));
    PCU(cudaGetLastError());
    PCU(cudaMemcpyAsync(out, res, sizeof(double) * n_series * SDE_PMOM_STRIDE, cudaMemcpyDeviceToHost, c.st));
    PCU(cudaStreamSynchronize(c.st));
    if (c.timing) {
        float ms = 0.f;
        PCU(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
        c.last_ms[0] = ms;
    }
    return SDE_OK;
}

// host form of the thresholds (Thr<R>::T): for f32 data the largest float
// not above each FP64 threshold, for f64 data its order key
template <typename R> typename Thr<R>::T thr_cast(double v);
template <> long long thr_cast<double>(double v) {
    long long b;
    memcpy(&b, &v, sizeof b);
    return order_key(b);
}
template <> float thr_cast<float>(double v) {
    float f = (float)v;
    if ((double)f > v) f = nextafterf(f, -INFINITY);
    return f;
}
// padding above every value's key: +inf (a value of +inf is not below it),
// the largest key (above +inf's)
template <typename R> typename Thr<R>::T thr_sentinel();
template <> float thr_sentinel<float>() { return INFINITY; }
template <> long long thr_sentinel<double>() { return 0x7fffffffffffffffLL; }

template <typename R>
int cdf_impl(const void *x, int on_device, int64_t n_rows, int64_t n_vars, int64_t paths, const SdeTimes *at,
             const double *xv, int64_t n_x, double *out) {
    int rc;
    if ((rc = check_dims(x, n_rows, n_vars, paths, out))) return rc;
    if (n_x < 1 || !xv) return rt_fail(SDE_ERR_INVALID, "cdf needs at least one value");
    if (n_x > ((int64_t)1 << 24)) return rt_fail(SDE_ERR_INVALID, "cdf: at most 2^24 values");
    std::vector<TimePoint> tp;
    if ((rc = time_points(at, n_rows, &tp))) return rc;
    const int64_t n_t = (int64_t)tp.size(), n_series = n_t * n_vars;
    if (n_series > ((int64_t)1 << 40) / n_x) return rt_fail(SDE_ERR_INVALID, "cdf output too large");
    // sorted NaN-free thresholds and their positions in xv
    std::vector<int64_t> perm;
    for (int64_t j = 0; j < n_x; ++j)
        if (!std::isnan(xv[j])) perm.push_back(j);
    std::stable_sort(perm.begin(), perm.end(), [&](int64_t a, int64_t b) { return xv[a] < xv[b]; });
    const int n_thr = (int)perm.size();
    int n_pad = 1;   // 2^m - 1 >= n_thr
    while (n_pad < n_thr) n_pad = 2 * n_pad + 1;
    std::vector<typename Thr<R>::T> thr(n_pad, thr_sentinel<R>());
    for (int k = 0; k < n_thr; ++k) thr[k] = thr_cast<R>(xv[perm[k]]);

    std::lock_guard<std::mutex> lk(rt_mutex());
    RtCall c;
    if ((rc = rt_begin(&c))) return rc;
    void *res;
    const size_t out_bytes = sizeof(double) * n_series * n_x;
    if ((rc = rt_scratch(3, out_bytes, &res))) return rc;
    PCU(cudaMemsetAsync(res, 0, out_bytes, c.st));
    if (n_thr > 0) {
        const void *dx;
        if ((rc = input_ptr(c, x, sizeof(R) * n_rows * n_vars * paths, on_device, &dx))) return rc;
        // tables: time points, thresholds, permutation
        const size_t o_thr = (sizeof(TimePoint) * n_t + 15) & ~(size_t)15;
        const size_t o_perm = o_thr + ((sizeof(typename Thr<R>::T) * n_pad + 15) & ~(size_t)15);
        const size_t tab_bytes = o_perm + sizeof(int64_t) * n_thr;
        std::vector<char> tab(tab_bytes);
        memcpy(tab.data(), tp.data(), sizeof(TimePoint) * n_t);
        memcpy(tab.data() + o_thr, thr.data(), sizeof(typename Thr<R>::T) * n_pad);
        memcpy(tab.data() + o_perm, perm.data(), sizeof(int64_t) * n_thr);
        void *dtab, *cnt;
        if ((rc = rt_scratch(1, tab_bytes, &dtab))) return rc;
        PCU(cudaMemcpyAsync(dtab, tab.data(), tab_bytes, cudaMemcpyHostToDevice, c.st));
        const size_t cnt_bytes = sizeof(unsigned long long) * n_series * n_thr;
        if ((rc = rt_scratch(2, cnt_bytes, &cnt))) return rc;
        PCU(cudaMemsetAsync(cnt, 0, cnt_bytes, c.st));
        const int64_t target = (int64_t)c.sms * 8;
        int64_t nch = (target + n_series - 1) / n_series;
        const int64_t maxch = (paths + 4 * PB - 1) / (4 * PB);
        if (nch > maxch) nch = maxch;
        if (nch < 1) nch = 1;
        const int64_t chunk = (paths + nch - 1) / nch;
        nch = (paths + chunk - 1) / chunk;
        const dim3 grid((unsigned)nch, grid_y(n_series));
        const TimePoint *dtp = (const TimePoint *)dtab;
        const typename Thr<R>::T *dthr = (const typename Thr<R>::T *)((char *)dtab + o_thr);
        if (c.timing) PCU(cudaEventRecord(c.ev0, c.st));
        if (n_thr <= CDF_SMEM_MAX) {
            const size_t smem = (((size_t)n_thr * 4 + 15) & ~(size_t)15) + sizeof(typename Thr<R>::T) * n_pad;
            if (smem > 48 * 1024)
                PCU(cudaFuncSetAttribute(cdf_kernel<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
            cdf_kernel<R, true><<<grid, PB, smem, c.st>>>((const R *)dx, n_vars, paths, dtp, n_series, dthr, n_thr,
                                                          n_pad, chunk, (unsigned long long *)cnt);
        } else {
            cdf_kernel<R, false><<<grid, PB, 0, c.st>>>((const R *)dx, n_vars, paths, dtp, n_series, dthr, n_thr,
                                                        n_pad, chunk, (unsigned long long *)cnt);
        }
        cdf_final_kernel<<<(unsigned)((n_series + 255) / 256), 256, 0, c.st>>>(
            (const unsigned long long *)cnt, n_series, n_thr, (const int64_t *)((char *)dtab + o_perm), n_vars,
            n_x, paths, (double *)res);
        if (c.timing) PCU(cudaEventRecord(c.ev1, c.st));
        PCU(cudaGetLastError());
    }
    PCU(cudaMemcpyAsync(out, res, out_bytes, cudaMemcpyDeviceToHost, c.st));
    PCU(cudaStreamSynchronize(c.st));
    if (c.timing && n_thr > 0) {
        float ms = 0.f;
        PCU(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
        c.last_ms[0] = ms;
    }
    return SDE_OK;
}

template <typename R>
int chf_impl(const void *x, int on_device, int64_t n_rows, int64_t n_vars, int64_t paths, const SdeTimes *at,
             const double *u, int64_t n_u, double *out) {
    int rc;
    if ((rc = check_dims(x, n_rows, n_vars, paths, out))) return rc;
    if (n_u < 1 || !u) return rt_fail(SDE_ERR_INVALID, "chf needs at least one u");
    if (n_u > 4096) return rt_fail(SDE_ERR_INVALID, "chf: at most 4096 values of u per call");
    std::vector<TimePoint> tp;
    if ((rc = time_points(at, n_rows, &tp))) return rc;
    const int64_t n_t = (int64_t)tp.size(), n_series = n_t * n_vars;
    std::lock_guard<std::mutex> lk(rt_mutex());
    RtCall c;
    if ((rc = rt_begin(&c))) return rc;
    const void *dx;
    if ((rc = input_ptr(c, x, sizeof(R) * n_rows * n_vars * paths, on_device, &dx))) return rc;
    const size_t o_u = (sizeof(TimePoint) * n_t + 15) & ~(size_t)15;
    const size_t tab_bytes = o_u + sizeof(double) * n_u;
    std::vector<char> tab(tab_bytes);
    memcpy(tab.data(), tp.data(), sizeof(TimePoint) * n_t);
    memcpy(tab.data() + o_u, u, sizeof(double) * n_u);
    void *dtab, *part, *res;
    if ((rc = rt_scratch(1, tab_bytes, &dtab))) return rc;
    PCU(cudaMemcpyAsync(dtab, tab.data(), tab_bytes, cudaMemcpyHostToDevice, c.st));
    // blocks per series: 8 per SM in all, at most one per chunk
    const int64_t target = (int64_t)c.sms * 8;
    int64_t nch = (target + n_series - 1) / n_series;
    const int64_t maxch = (paths + CHF_CHUNK - 1) / CHF_CHUNK;
    if (nch > maxch) nch = maxch;
    if (nch < 1) nch = 1;
    if ((rc = rt_scratch(2, sizeof(double) * 2 * n_u * n_series * nch, &part))) return rc;
    const size_t out_bytes = sizeof(double) * 2 * n_series * n_u;
    if ((rc = rt_scratch(3, out_bytes, &res))) return rc;
    const size_t smem = sizeof(double) * (CHF_CHUNK + 2 * n_u);
    auto launch = [&](auto kern) -> int {
        PCU(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        if (c.timing) PCU(cudaEventRecord(c.ev0, c.st));
        kern<<<dim3((unsigned)nch, grid_y(n_series)), PB, smem, c.st>>>(
            (const R *)dx, n_vars, paths, (const TimePoint *)dtab, n_series,
            (const double *)((char *)dtab + o_u), (int)n_u, (int)nch, (double *)part);
        return SDE_OK;
    };
    rc = n_u >= CHF_UT ? launch(chf_kernel<R, CHF_UT>)
         : n_u > 2    ? launch(chf_kernel<R, 4>)
         : n_u > 1    ? launch(chf_kernel<R, 2>)
                      : launch(chf_kernel<R, 1>);
    if (rc) return rc;
    chf_final_kernel<<<(unsigned)((n_series * n_u + 255) / 256), 256, 0, c.st>>>(
        (const double *)part, n_series, (int)nch, (int)n_u, n_vars, paths, (double *)res);
    if (c.timing) PCU(cudaEventRecord(c.ev1, c.st));
    PCU(cudaGetLastError());
    PCU(cudaMemcpyAsync(out, res, out_bytes, cudaMemcpyDeviceToHost, c.st));
    PCU(cudaStreamSynchronize(c.st));
    if (c.timing) {
        float ms = 0.f;
        PCU(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
        c.last_ms[0] = ms;
    }
    return SDE_OK;
}

}  // namespace

extern "C" int32_t sde_process_moments(const void *x, int32_t is_fp32, int32_t on_device, int64_t n_series,
                                       int64_t paths, double *out) {
    if (is_fp32) return moments_impl<float>(x, on_device, n_series, paths, out);
    return moments_impl<double>(x, on_device, n_series, paths, out);
}

extern "C" int32_t sde_process_cdf(const void *x, int32_t is_fp32, int32_t on_device, int64_t n_rows,
                                   int64_t n_vars, int64_t paths, const SdeTimes *at, const double *xv,
                                   int64_t n_x, double *out) {
    if (is_fp32) return cdf_impl<float>(x, on_device, n_rows, n_vars, paths, at, xv, n_x, out);
    return cdf_impl<double>(x, on_device, n_rows, n_vars, paths, at, xv, n_x, out);
}

extern "C" int32_t sde_process_chf(const void *x, int32_t is_fp32, int32_t on_device, int64_t n_rows,
                                   int64_t n_vars, int64_t paths, const SdeTimes *at, const double *u,
                                   int64_t n_u, double *out) {
    if (is_fp32) return chf_impl<float>(x, on_device, n_rows, n_vars, paths, at, u, n_u, out);
    return chf_impl<double>(x, on_device, n_rows, n_vars, paths, at, u, n_u, out);
}
