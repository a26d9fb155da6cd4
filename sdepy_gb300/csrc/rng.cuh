// Counter-based random numbers drawn in registers.
//
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with the
// published multipliers and Weyl key increments.  Every draw is a pure
// function of (counter, key), so any thread can regenerate any increment of
// any path -- the adjoint kernel recomputes forward states this way.
//
// Counter words used by the integrator:
//   c0 = path index, c1 = step index + leg offset,
//   c2 = (group << 8) | call      (normals, then Poisson uniforms)
//      = 0x80000000 | (var << 12) | jump   (jump sizes)
//   c3 = stream (call / instance id);  key = 64-bit seed.
// Groups of one state variable use one call per two steps (the even
// step's): see PairedSteps in sde_kernels.cuh.
//
// Uniforms: u = (x + 0.5) * 2^-32 in (0, 1) for a 32-bit word x.
// Normals (Box-Muller) from a word pair (a, b):
//   r = sqrt(-2 log u(a)),  v = (b >> 9) * 2^-22 - 1  in [-1, 1),
//   z0 = r cos(pi v),  z1 = r sin(pi v).
// FP64 evaluates this formula to a few ulp with table-driven logarithm and
// sine / cosine (ln_u01_f64, sincospi_f64 below); FP32 evaluates it with the
// SFU approximations, so both precisions consume identical draws.
#pragma once
#ifndef __CUDACC_RTC__
#include <cstdint>
#endif

#include "fp64_tables.h"

namespace sdegpu {

// The ten round keys (k + i*(0x9E3779B9, 0xBB67AE85)) are computed once on
// the host and read from the kernel parameter block, so a round is two wide
// multiplies and two three-input XORs.
struct PhiloxKey {
    uint32_t k0[10], k1[10];
};

__host__ __device__ inline PhiloxKey philox_schedule(uint64_t seed) {
    PhiloxKey k;
    uint32_t a = (uint32_t)seed, b = (uint32_t)(seed >> 32);
    for (int i = 0; i < 10; ++i) {
        k.k0[i] = a;
        k.k1[i] = b;
        a += 0x9E3779B9u;
        b += 0xBB67AE85u;
    }
    return k;
}

__device__ __forceinline__ void mulwide(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
    unsigned long long p;
    asm("mul.wide.u32 %0, %1, %2;" : "=l"(p) : "r"(a), "r"(b));
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, const PhiloxKey &key) {
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        uint32_t hi0, lo0, hi1, lo1;
        mulwide(0xD2511F53u, c.x, hi0, lo0);
        mulwide(0xCD9E8D57u, c.z, hi1, lo1);
        c = make_uint4(hi1 ^ c.y ^ key.k0[i], lo1, hi0 ^ c.w ^ key.k1[i], lo0);
    }
    return c;
}

// The first round multiplies only c0 and c2; with c1 (the step) left out
// it is invariant along a path, so a path loop computes it once:
//   pre = philox_round0(c0, c2, c3, key),  out = philox_from_round0(pre, c1, key)
// equals philox4x32_10((c0, c1, c2, c3), key) bit for bit.
__device__ __forceinline__ uint4 philox_round0(uint32_t c0, uint32_t c2, uint32_t c3, const PhiloxKey &key) {
    uint32_t hi0, lo0, hi1, lo1;
    mulwide(0xD2511F53u, c0, hi0, lo0);
    mulwide(0xCD9E8D57u, c2, hi1, lo1);
    return make_uint4(hi1 ^ key.k0[0], lo1, hi0 ^ c3 ^ key.k1[0], lo0);
}

__device__ __forceinline__ uint4 philox_from_round0(uint4 c, uint32_t c1, const PhiloxKey &key) {
    c.x ^= c1;
#pragma unroll
    for (int i = 1; i < 10; ++i) {
        uint32_t hi0, lo0, hi1, lo1;
        mulwide(0xD2511F53u, c.x, hi0, lo0);
        mulwide(0xCD9E8D57u, c.z, hi1, lo1);
        c = make_uint4(hi1 ^ c.y ^ key.k0[i], lo1, hi0 ^ c.w ^ key.k1[i], lo0);
    }
    return c;
}

__device__ __forceinline__ double u01_f64(uint32_t x) {
    return ((double)x + 0.5) * 0x1p-32;
}

// v = (b >> 9) * 2^-22 - 1, exact in both precisions
__device__ __forceinline__ float vpm1_f32(uint32_t b) {
    return __uint_as_float(0x40000000u | (b >> 9)) - 3.0f;
}
__device__ __forceinline__ double vpm1_f64(uint32_t b) {
    return (double)(b >> 9) * 0x1p-22 - 1.0;
}

__device__ __forceinline__ float approx_lg2(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float approx_sqrt(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float approx_sin(float x) {
    float y;
    asm("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float approx_cos(float x) {
    float y;
    asm("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ln u for u = (a + 0.5) 2^-32 = (2a + 1) 2^-33, within a few ulp.  Tang's
// table-driven method (ACM TOMS 15(2), 1989): 2a + 1 = 2^e m with
// m in [0.75, 1.5) built from the integer's bits, m = c_j (1 + r) with
// c_j = 0.75 + j/128 the nearest table point, |r| <= 1/192, and
// ln u = (e - 33) ln 2 + ln c_j + log1p(r), log1p by its Taylor series to
// r^7 (the first omitted term is below 2^-56 of log1p(r)).  Near u = 1
// the result is log1p(r) alone, so it keeps full relative accuracy there.
__device__ __forceinline__ double ln_u01_f64(uint32_t a) {
    const unsigned long long v = 2ull * a + 1ull;              // odd, in [1, 2^33)
    const int lz = __clzll((long long)v);
    const int e = 63 - lz;                                      // 2^e <= v < 2^(e+1)
    const unsigned long long frac = ((v << lz) << 1) >> 12;     // the 52 bits below the leading one
    const uint32_t fhi = (uint32_t)(frac >> 32);                // top 20 of them
    const bool upper = fhi >= 0x80000u;                         // 1.f >= 1.5: use m = 1.f / 2
    const int j = upper ? (int)((fhi + 0x2000u) >> 14) - 32 : (int)((fhi + 0x1000u) >> 13) + 32;
    const int k = e - 33 + (upper ? 1 : 0);                     // in [-33, 0]
    const double m = __longlong_as_double((long long)(((upper ? 1022ull : 1023ull) << 52) | frac));
    const double d = m - __ldg(&F64_LOG_C[j]);                  // exact
    const double r = d * __ldg(&F64_LOG_INVC[j]);
    const double r2 = r * r;
    double q = 1.0 / 7.0;
    q = fma(q, r, -1.0 / 6.0);
    q = fma(q, r, 1.0 / 5.0);
    q = fma(q, r, -0.25);
    q = fma(q, r, 1.0 / 3.0);
    q = fma(q, r, -0.5);
    const double p = fma(q, r2, r);                             // log1p(r)
    return (__ldg(&F64_KLN2_HI[k + 35]) + __ldg(&F64_LOG_LNC[j])) + (__ldg(&F64_KLN2_LO[k + 35]) + p);
}

// sin(pi v), cos(pi v) for v = (b >> 9) 2^-22 - 1 in [-1, 1), within a few
// ulp: v = n/64 + f with |f| <= 1/128 exact, x = pi f, Taylor series of
// sin x to x^7 and cos x to x^6 (|x| <= pi/128: the first omitted terms
// are below 2^-58), and the angle-addition formulas with the tabulated
// sin(pi n/64), cos(pi n/64).  Where the result is near zero (n = 0, +-32,
// +-64) the table's other factor is exactly zero, so no cancellation.
__device__ __forceinline__ void sincospi_f64(uint32_t b, double &s, double &c) {
    const int q = (int)(b >> 9);                     // v = q 2^-22 - 1
    const int nn = (q + 0x8000) >> 16;               // n + 64, in [0, 128]
    const int qd = q - (nn << 16);                   // f = qd 2^-22, |qd| <= 2^15
    const double x = (double)qd * (0x1p-22 * F64_PI_HI);
    const double x2 = x * x;
    double ps = -1.0 / 5040.0;
    ps = fma(ps, x2, 1.0 / 120.0);
    ps = fma(ps, x2, -1.0 / 6.0);
    const double sx = fma(x * x2, ps, x);            // sin x
    double pc = -1.0 / 720.0;
    pc = fma(pc, x2, 1.0 / 24.0);
    pc = fma(pc, x2, -0.5);
    const double cx = fma(x2, pc, 1.0);              // cos x
    const double S = __ldg(&F64_SINPI_N[nn]), C = __ldg(&F64_COSPI_N[nn]);
    s = fma(S, cx, C * sx);
    c = fma(C, cx, -(S * sx));
}

template <typename R> struct Rng;

template <> struct Rng<double> {
    static __device__ __forceinline__ void normal2(uint32_t a, uint32_t b,
                                                   double &z0, double &z1) {
        const double r = sqrt(-2.0 * ln_u01_f64(a));
        double s, c;
        sincospi_f64(b, s, c);
        z0 = r * c;
        z1 = r * s;
    }
    // -log(u), the unit exponential
    static __device__ __forceinline__ double expo(uint32_t a) {
        return -ln_u01_f64(a);
    }
    static __device__ __forceinline__ double unif(uint32_t a) { return u01_f64(a); }
    static __device__ __forceinline__ void normal2_s(uint32_t a, uint32_t b,
                                                     double &z0, double &z1) {
        normal2(a, b, z0, z1);
        z0 *= 0.84932180028801907;  // 1 / sqrt(2 ln 2)
        z1 *= 0.84932180028801907;
    }
};

template <> struct Rng<float> {
    static __device__ __forceinline__ void normal2(uint32_t a, uint32_t b,
                                                   float &z0, float &z1) {
        const float u = fmaf((float)a, 0x1p-32f, 0x1p-33f);
        // -2 ln u = -2 ln2 * log2 u
        const float r = approx_sqrt(-1.38629436f * approx_lg2(u));
        const float th = angle(b);
        z0 = r * approx_cos(th);
        z1 = r * approx_sin(th);
    }
    // pi v = pi (s - 3) with s = 3 + v in [2, 4) built from the word's bits,
    // as one fused multiply-add
    static __device__ __forceinline__ float angle(uint32_t b) {
        return fmaf(__uint_as_float(0x40000000u | (b >> 9)), 3.14159265f, -9.42477796f);
    }
    // the same pair divided by sqrt(2 ln 2): r = sqrt(-log2 u), one multiply
    // less per pair for callers that fold the factor into their coefficients
    static __device__ __forceinline__ void normal2_s(uint32_t a, uint32_t b,
                                                     float &z0, float &z1) {
        const float u = fmaf((float)a, 0x1p-32f, 0x1p-33f);
        const float r = approx_sqrt(-approx_lg2(u));
        const float th = angle(b);
        z0 = r * approx_cos(th);
        z1 = r * approx_sin(th);
    }
    static __device__ __forceinline__ float expo(uint32_t a) {
        const float u = fmaf((float)a, 0x1p-32f, 0x1p-33f);
        return -0.69314718f * approx_lg2(u);
    }
    static __device__ __forceinline__ float unif(uint32_t a) {
        return fmaf((float)a, 0x1p-32f, 0x1p-33f);
    }
};

}  // namespace sdegpu
