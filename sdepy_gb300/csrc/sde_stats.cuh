// Montecarlo summaries on the device: final deterministic FP64 merge of the
// per-block partials, histogram edges and the histogram itself.
//
// The histogram restates numpy.histogram's uniform-bin rule (numpy 2.x,
// numpy/lib/_histograms_impl.py: _get_outer_edges, the linspace of
// _get_bin_edges, and the block loop of histogram()), which is what
// sdepy's montecarlo._update_histogram calls (sdepy/infrastructure.py:
// 2999-3013):
//   edges   = linspace(lo, hi, bins + 1) evaluated in the sample dtype
//             (float64 when an explicit range is given, then cast);
//   keep    = lo <= x <= hi;
//   i       = int(((x - lo) / (hi - lo)) * bins), i == bins -> bins - 1;
//   i -= x < edges[i];  i += x >= edges[i + 1] and i != bins - 1.
#pragma once
#include "sde_kernels.cuh"

namespace sdegpu {

constexpr int ERRF_RANGE = 2;     // autodetected histogram range not finite
constexpr int HIST_SMEM_BINS = 8192;

// result record per output variable (doubles):
//   [0..6] n, mean, M2, M3, M4, min, max, [7] lo edge, [8] hi edge,
//   [9 .. 9+n_strikes) payoff means
constexpr int RES_STRIDE = 9 + SDE_MAX_STRIKES;

// merge partials [groups][nb][opg][NPART] into res[(g*opg + j)*RES_STRIDE]
// and, when bins > 0, write the histogram edges edges[(o)*(bins+1) + e] in R.
template <typename R>
__global__ void __launch_bounds__(BLOCK)
stats_finalize_kernel(const double *partials, int nb, int opg, int n_strikes, int bins,
                      int has_range, double range_lo, double range_hi,
                      double *res, R *edges, double *edges64, int32_t *err) {
    __shared__ double acc[BLOCK][8];
    __shared__ double pay[BLOCK][SDE_MAX_STRIKES];
    const int o = blockIdx.x;  // output variable g*opg + j
    const int g = o / opg, j = o % opg;
    double A[8] = {0, 0, 0, 0, 0, INFINITY, -INFINITY, 0};
    double P[SDE_MAX_STRIKES];
    for (int s = 0; s < SDE_MAX_STRIKES; ++s) P[s] = 0.0;
    // fixed assignment: thread t merges blocks t, t + BLOCK, ... in order
    for (int b = threadIdx.x; b < nb; b += BLOCK) {
        const double *q = partials + (((int64_t)g * nb + b) * opg + j) * NPART;
        double B[5] = {q[0], q[1], q[2], q[3], q[4]};
        moments_merge(A, B);
        A[5] = fmin(A[5], q[5]);
        A[6] = fmax(A[6], q[6]);
        for (int s = 0; s < n_strikes; ++s) P[s] += q[8 + s];
    }
    for (int i = 0; i < 8; ++i) acc[threadIdx.x][i] = A[i];
    for (int s = 0; s < SDE_MAX_STRIKES; ++s) pay[threadIdx.x][s] = P[s];
    __syncthreads();
    // fixed pairwise tree
    for (int w = BLOCK / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            double *a = acc[threadIdx.x];
            const double *b = acc[threadIdx.x + w];
            double B[5] = {b[0], b[1], b[2], b[3], b[4]};
            moments_merge(a, B);
            a[5] = fmin(a[5], b[5]);
            a[6] = fmax(a[6], b[6]);
            for (int s = 0; s < n_strikes; ++s) pay[threadIdx.x][s] += pay[threadIdx.x + w][s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double *r = res + (int64_t)o * RES_STRIDE;
        for (int i = 0; i < 7; ++i) r[i] = acc[0][i];
        const double n = acc[0][0];
        for (int s = 0; s < n_strikes; ++s) r[9 + s] = n > 0 ? pay[0][s] / n : 0.0;
        if (bins > 0) {
            R lo, hi;
            if (has_range) {
                lo = (R)range_lo;
                hi = (R)range_hi;
            } else {
                lo = (R)acc[0][5];
                hi = (R)acc[0][6];
                if (n == 0.0) {
                    lo = R(0);
                    hi = R(1);
                } else if (!(isfinite((double)lo) && isfinite((double)hi))) {
                    atomicOr(err, ERRF_RANGE);
                    lo = R(0);
                    hi = R(1);
                }
            }
            if (has_range ? (range_lo == range_hi) : (lo == hi)) {
                if (has_range) {
                    range_lo -= 0.5;
                    range_hi += 0.5;
                } else {
                    lo = lo - R(0.5);
                    hi = hi + R(0.5);
                }
            }
            R *e = edges + (int64_t)o * (bins + 1);
            double *e64 = edges64 + (int64_t)o * (bins + 1);
            if (has_range) {
                // linspace in float64 (python float bounds), cast to R
                const double delta = range_hi - range_lo;
                const double step = delta / bins;
                for (int i = 0; i < bins; ++i) {
                    const double y = (step == 0.0) ? __dadd_rn(__dmul_rn(__ddiv_rn((double)i, bins), delta), range_lo)
                                                   : __dadd_rn(__dmul_rn((double)i, step), range_lo);
                    e[i] = (R)y;
                }
                e[bins] = (R)range_hi;
                r[7] = range_lo;
                r[8] = range_hi;
            } else {
                // linspace in the sample dtype
                const R delta = Ar<R>::sub(hi, lo);
                const R step = delta / (R)bins;
                for (int i = 0; i < bins; ++i) {
                    R y;
                    if (step == R(0))
                        y = Ar<R>::add(Ar<R>::mul((R)i / (R)bins, delta), lo);
                    else
                        y = Ar<R>::add(Ar<R>::mul((R)i, step), lo);
                    e[i] = y;
                }
                e[bins] = hi;
                r[7] = (double)lo;
                r[8] = (double)hi;
            }
            for (int i = 0; i <= bins; ++i) e64[i] = (double)e[i];
        }
    }
}

// exact-order float helpers for the bin index
__device__ __forceinline__ float hdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double hdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float hmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double hmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float hsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double hsub(double a, double b) { return __dsub_rn(a, b); }

// numpy bin index of x, or -1 when x is outside [lo, hi] (or NaN)
template <typename R>
__device__ __forceinline__ int np_bin(R x, R lo, R hi, const R *e, int bins, int has_range,
                                      double dlo, double dhi) {
    if (!(x >= lo && x <= hi)) return -1;
    int i;
    if (has_range && sizeof(R) == 4) {
        // float32 sample with python-float range: (x - lo) in float32,
        // divided by the float64 range width, times bins in float64
        const double f = __dmul_rn(__ddiv_rn((double)hsub(x, lo), __dsub_rn(dhi, dlo)), (double)bins);
        i = (int)f;
    } else {
        const R f = hmul(hdiv(hsub(x, lo), hsub(hi, lo)), (R)bins);
        i = (int)f;
    }
    if (i >= bins) i = bins - 1;
    if (i < 0) i = 0;
    if (x < e[i]) i -= 1;
    if (i < bins - 1 && x >= e[i + 1]) i += 1;
    if (i < 0) i = 0;
    return i;
}

// histogram of vals[o*var_stride + p] (p < paths) for o = blockIdx.y
template <typename R>
__global__ void __launch_bounds__(BLOCK)
hist_kernel(const R *vals, int64_t var_stride, int64_t paths, int bins, const R *edges,
            const double *res, int has_range, unsigned long long *counts) {
    extern __shared__ unsigned int sh[];
    const int o = blockIdx.y;
    const R *e = edges + (int64_t)o * (bins + 1);
    const R lo = e[0], hi = e[bins];
    const double dlo = res[(int64_t)o * RES_STRIDE + 7], dhi = res[(int64_t)o * RES_STRIDE + 8];
    const bool use_smem = bins <= HIST_SMEM_BINS;
    unsigned long long *cnt = counts + (int64_t)o * bins;
    if (use_smem)
        for (int b = threadIdx.x; b < bins; b += BLOCK) sh[b] = 0u;
    __syncthreads();
    const R *v = vals + (int64_t)o * var_stride;
    for (int64_t p = (int64_t)blockIdx.x * BLOCK + threadIdx.x; p < paths; p += (int64_t)gridDim.x * BLOCK) {
        const int b = np_bin<R>(v[p], lo, hi, e, bins, has_range, dlo, dhi);
        if (b >= 0) {
            if (use_smem)
                atomicAdd(&sh[b], 1u);
            else
                atomicAdd(&cnt[b], 1ull);
        }
    }
    __syncthreads();
    if (use_smem)
        for (int b = threadIdx.x; b < bins; b += BLOCK)
            if (sh[b]) atomicAdd(&cnt[b], (unsigned long long)sh[b]);
}

// histogram against explicit edges (numpy's cumulative searchsorted rule,
// _search_sorted_inclusive): bin i holds e_i <= x < e_{i+1}, the last bin is
// closed on the right, values outside [e_0, e_bins] are dropped.
template <typename R>
__global__ void __launch_bounds__(BLOCK)
hist_edges_kernel(const R *vals, int64_t var_stride, int64_t paths, int bins, const R *edges,
                  unsigned long long *counts) {
    extern __shared__ unsigned int sh[];
    const int o = blockIdx.y;
    const R *e = edges + (int64_t)o * (bins + 1);
    const bool use_smem = bins <= HIST_SMEM_BINS;
    unsigned long long *cnt = counts + (int64_t)o * bins;
    if (use_smem)
        for (int b = threadIdx.x; b < bins; b += BLOCK) sh[b] = 0u;
    __syncthreads();
    const R *v = vals + (int64_t)o * var_stride;
    const R e0 = e[0], en = e[bins];
    for (int64_t p = (int64_t)blockIdx.x * BLOCK + threadIdx.x; p < paths; p += (int64_t)gridDim.x * BLOCK) {
        const R x = v[p];
        if (!(x >= e0 && x <= en)) continue;
        // number of e[0..bins-1] that are <= x, minus one
        int lo = 0, hi = bins;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (e[mid] <= x) lo = mid + 1;
            else hi = mid;
        }
        const int b = lo - 1;
        if (use_smem)
            atomicAdd(&sh[b], 1u);
        else
            atomicAdd(&cnt[b], 1ull);
    }
    __syncthreads();
    if (use_smem)
        for (int b = threadIdx.x; b < bins; b += BLOCK)
            if (sh[b]) atomicAdd(&cnt[b], (unsigned long long)sh[b]);
}

// block partials of an existing sample [n_vars][paths] (groups = n_vars, opg = 1)
template <typename R>
__global__ void __launch_bounds__(BLOCK)
sample_partials_kernel(const R *vals, int64_t paths, double *partials, const R *strikes_unused) {
    __shared__ R red[BLOCK / 32];
    __shared__ double part[NPART];
    const int o = blockIdx.y;
    if (threadIdx.x == 0) {
        for (int i = 0; i < NPART; ++i) part[i] = 0.0;
        part[5] = INFINITY;
        part[6] = -INFINITY;
    }
    const R *v = vals + (int64_t)o * paths;
    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    const int64_t rounds = (paths + stride - 1) / stride;
    for (int64_t rd = 0; rd < rounds; ++rd) {
        const int64_t p = rd * stride + (int64_t)blockIdx.x * BLOCK + threadIdx.x;
        const bool act = p < paths;
        block_round_stats<R>(act ? v[p] : R(0), act, strikes_unused, 0, part, red);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double *dst = partials + ((int64_t)o * gridDim.x + blockIdx.x) * NPART;
        for (int i = 0; i < NPART; ++i) dst[i] = part[i];
    }
}

}  // namespace sdegpu
