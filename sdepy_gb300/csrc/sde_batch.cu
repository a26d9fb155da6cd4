// Batched integration of many heterogeneous SDE instances in one persistent
// launch: each warp takes work items -- (instance, slab of paths) -- from an
// atomic counter, integrates the slab's paths on the instance's uniform grid
// (FP32 states, Philox noise with the same counter layout as the single
// instance kernels), and writes one FP64 partial per item: count, mean and
// M2 of the terminal value X of the instance's first state variable, and
// the sums of its pathwise derivatives (tangent mode: every parameter's
// derivative is carried forward along the path).  A second kernel merges
// each instance's partials in a fixed order.  A plan owns the device arrays
// and, optionally, a CUDA graph of [reset counter, batch kernel, merge].
//
// Work items are sorted longest-first (steps x slab), so the long ones start
// early and the short ones fill the tail.  There are no waits on other
// warps: a warp that finds the counter past the last item exits.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "sde_kernels.cuh"

using namespace sdegpu;

namespace sdegpu {
int set_last_error(int code, const char *msg);
}

namespace {

int bfail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return set_last_error(code, buf);
}

#define CUB(call)                                                                           \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return bfail(SDE_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));     \
    } while (0)

constexpr int NB_GRAD = 8;
constexpr int NB_PART = 3 + NB_GRAD;  // n, mean, M2, grad sums

// device copy of one instance: everything the kernel needs, in FP32
struct DevInst {
    int32_t model, jump_law, nvars, n_steps;
    int64_t paths;
    float dt, sq;
    float x0[4];
    float d[4], b[4], c[4];       // x' = x + (b - d x) + c w  (LINEAR d = 0)
    float p0[4], p1[4], p2[4];    // raw coefficients (Heston, tangents)
    float ja, jb;                 // jump-size law (norm: a + b z)
    long long thr, thr1;          // Poisson count >= 1 / >= 2 thresholds of one step
    double p0d, lamdt;            // exp(-lam dt), lam dt
    float rho, rho_k;             // Heston rho and -rho/sqrt(1-rho^2)
    float chol10, chol11;         // Heston 2x2 Cholesky factor
    PhiloxKey key;
    uint32_t stream;
    int32_t out_exp;
};

struct Item {
    int32_t inst;
    int32_t nslab;   // paths in this item
    int64_t base;    // first path
};

__device__ __forceinline__ void kahan(float &s, float &c, float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

// integrate one path of instance I; returns X(T) and its derivatives
__device__ __forceinline__ float path_lin(const DevInst &I, const PhiloxKey &key, uint32_t p, float (&g)[NB_GRAD],
                                          int32_t *err) {
    float a = I.x0[0], sdw = 0.f, sja = 0.f, sjb = 0.f;
    const bool jumps = I.jump_law != SDE_JUMP_NONE;
    // one variable: one Philox call per two steps, as the forward kernel
    const PathPre<1> pre(key, p, 0u, I.stream);
    PairedSteps<float, 1> pair;
    // the step loop's coefficients in registers (the loop's global writes
    // would otherwise force a reload of every field each step)
    const float b0 = I.b[0], c0 = I.c[0], sq = I.sq;
    const long long thr = I.thr, thr1 = I.thr1;
    const int n_steps = I.n_steps;
#pragma unroll 1
    for (int k = 0; k < n_steps; ++k) {
        float z0;
        uint32_t pw;
        pair.get(key, pre, k, 0u, z0, pw);
        a = a + b0 + c0 * z0;
        sdw += sq * z0;
        if (jumps && (long long)pw > thr) {
            const int cnt = (long long)pw <= thr1 ? 1 : poisson_tail(pw, I.p0d, I.lamdt, err);
            for (int j = 0; j < cnt; ++j) {
                const uint4 q = philox4x32_10(make_uint4(p, (uint32_t)k, 0x80000000u | (uint32_t)j, I.stream), key);
                float y0, y1;
                Rng<float>::normal2(q.x, q.y, y0, y1);
                a += I.ja + I.jb * y0;
                sja += 1.f;
                sjb += y0;
            }
        }
    }
    const float X = I.out_exp ? __expf(a) : a;
    const float xb = I.out_exp ? X : 1.f;
    g[0] = xb;                          // d/d x0 (integration variable)
    g[1] = xb * (I.dt * I.n_steps);     // d/d c_dt
    g[2] = xb * sdw;                    // d/d c_dw
    g[3] = 0.f;
    g[4] = xb * sja;                    // d/d jump a
    g[5] = xb * sjb;                    // d/d jump b
    g[6] = g[7] = 0.f;
    return X;
}

// WM: the states the step loop carries (the instance's W <= WM; 1, 2 or 4)
template <int WM>
__device__ __forceinline__ float path_ou(const DevInst &I, const PhiloxKey &key, uint32_t p, float (&g)[NB_GRAD]) {
    float x[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) x[m] = I.x0[m];
    // tangents of x[0] w.r.t. x0, k, theta, sigma
    float tx, tth, tk = 0.f, tsg = 0.f;
    const float rho0 = 1.f - I.d[0];
    const int W = I.nvars;
    const PathPre<1> pre(key, p, 0u, I.stream);
    // one or two variables: one Philox call per two steps
    PairedSteps<float, 1> pair1;
    PairedSteps<float, 2> pair2;
    // the step loop's coefficients in registers
    float cd[4], cb[4], cc[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        cd[m] = I.d[m];
        cb[m] = I.b[m];
        cc[m] = I.c[m];
    }
    const float th0 = I.p1[0], dt = I.dt, sq = I.sq;
    const int n_steps = I.n_steps;
#pragma unroll 1
    for (int k = 0; k < n_steps; ++k) {
        float z[4];
        if (WM == 1) {
            uint32_t pw;
            pair1.get(key, pre, k, 0u, z[0], pw);
            z[1] = z[2] = z[3] = 0.f;
        } else if (WM == 2) {
            pair2.get(key, pre, k, 0u, z[0], z[1]);
            z[2] = z[3] = 0.f;
        } else {
            const uint4 r = philox_from_round0(pre.r0[0], (uint32_t)k, key);
            Rng<float>::normal2(r.x, r.y, z[0], z[1]);
            if (W > 2) Rng<float>::normal2(r.z, r.w, z[2], z[3]);
            else z[2] = z[3] = 0.f;
        }
        const float dth = th0 - x[0];
        tk = fmaf(rho0, tk, dth * dt);
        tsg = fmaf(rho0, tsg, sq * z[0]);
#pragma unroll
        for (int m = 0; m < WM; ++m)
            if (m < W) x[m] = x[m] + fmaf(-cd[m], x[m], cb[m]) + cc[m] * z[m];
    }
    // the path-independent tangents: d x / d x0 = (1 - k dt)^n and
    // d x / d theta = 1 - (1 - k dt)^n (the recursions t' = (1 - k dt) t
    // and t' = (1 - k dt) t + k dt in closed form)
    tx = powf(rho0, (float)n_steps);
    tth = 1.f - tx;
    g[0] = tx;
    g[1] = tk;
    g[2] = tth;
    g[3] = tsg;
    g[4] = g[5] = g[6] = g[7] = 0.f;
    return x[0];
}

__device__ __forceinline__ float path_heston(const DevInst &I, const PhiloxKey &key, uint32_t p,
                                             float (&g)[NB_GRAD]) {
    float a = I.x0[0], y = I.x0[1];
    // tangents (d a, d y) w.r.t. [x0, mu, sigma, y0, k, theta, xi, rho]: y
    // does not depend on x0, mu, sigma, and a depends on them additively
    // (d a / d x0 = 1), so only the last five carry a (d a, d y) pair
    constexpr int NT = 5;                 // y0, k, theta, xi, rho
    float ta1 = 0.f, ta2 = 0.f, ta[NT], ty[NT];
#pragma unroll
    for (int j = 0; j < NT; ++j) ta[j] = ty[j] = 0.f;
    ty[0] = 1.f;
    const float mu = I.p0[0], sg = I.p1[0], kk = I.p0[1], th = I.p1[1], xi = I.p2[1];
    const float dt = I.dt, sq = I.sq;
    const float chol10 = I.chol10, chol11 = I.chol11, rho_k = I.rho_k;
    const int n_steps = I.n_steps;
    const PathPre<1> pre(key, p, 0u, I.stream);
    PairedSteps<float, 2> pair;   // one Philox call per two steps
    // the tangent recursion's constants (dt is the instance's)
    const float hsdt = -0.5f * sg * sg * dt, kdt1 = 1.f - kk * dt, kdt = kk * dt, sgdt = sg * dt;
    const float xrsq = xi * sq, xrksq = xi * rho_k * sq;
#pragma unroll 1
    for (int k = 0; k < n_steps; ++k) {
        float z0, z1;
        pair.get(key, pre, k, 0u, z0, z1);
        const float dW1 = z0 * sq;
        const float dW2 = (chol10 * z0 + chol11 * z1) * sq;
        const float yp = fmaxf(y, 0.f);
        const float s = approx_sqrt(yp);
        float Ay = 0.f, By = 1.f;
        if (y > 0.f && s > 0.f) {
            const float inv = __fdividef(0.5f, s);   // (approximate: a derivative term)
            Ay = fmaf(sg * dW1, inv, hsdt);
            By = fmaf(xi * dW2, inv, kdt1);
        }
        ta2 = fmaf(s, dW1, fmaf(-sgdt, yp, ta2));
        const float ey[NT] = {0.f, (th - yp) * dt, kdt, s * dW2, s * fmaf(xrksq, z1, xrsq * z0)};
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const float nta = ta[j] + Ay * ty[j];
            ty[j] = By * ty[j] + ey[j];
            ta[j] = nta;
        }
        const float na = a + (mu - sg * sg * yp * 0.5f) * dt + sg * s * dW1;
        y = y + kk * (th - yp) * dt + xi * s * dW2;
        a = na;
    }
    ta1 = (float)n_steps * dt;   // the sum of the steps
    const float X = __expf(a);
    g[0] = X;
    g[1] = X * ta1;
    g[2] = X * ta2;
#pragma unroll
    for (int j = 0; j < NT; ++j) g[3 + j] = X * ta[j];
    return X;
}

// CLS 0: the linear and OU instances, CLS 1: Heston.  Each class is its own
// persistent launch over its own items, so that the light class is not held
// to the register count of the Heston tangents.  Resident blocks per SM,
// measured on the 4096-instance workload (slab 1024): light 3 / Heston 2
// 247 ms, 4 / 2 256 ms, 4 / 3 265 ms, 2 / 2 269 ms (one kernel for both at
// 2 blocks: 290 ms).
#ifndef SDE_BATCH_LIGHT_MIN_BLOCKS
#define SDE_BATCH_LIGHT_MIN_BLOCKS 3
#endif
#ifndef SDE_BATCH_HEAVY_MIN_BLOCKS
#define SDE_BATCH_HEAVY_MIN_BLOCKS 2
#endif
template <int CLS>
__global__ void __launch_bounds__(BLOCK, CLS == 0 ? SDE_BATCH_LIGHT_MIN_BLOCKS : SDE_BATCH_HEAVY_MIN_BLOCKS)
batch_kernel(const DevInst *insts, const Item *items, int n_items, unsigned int *counter, double *part,
             int32_t *err) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        int it = 0;
        if (lane == 0) it = (int)atomicAdd(counter, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= n_items) return;
        const Item item = items[it];   // items of this class; `part` is indexed by it as well
        const DevInst &I = insts[item.inst];
        const PhiloxKey key = I.key;  // in registers for the whole item
        // per lane: Welford of X, Kahan sums of the derivatives
        float n = 0.f, mean = 0.f, m2 = 0.f;
        float gs[NB_GRAD], gc[NB_GRAD];
#pragma unroll
        for (int j = 0; j < NB_GRAD; ++j) gs[j] = gc[j] = 0.f;
        for (int q = lane; q < item.nslab; q += 32) {
            const uint32_t p = (uint32_t)(item.base + q);
            float g[NB_GRAD];
            float X;
            if (CLS == 1) X = path_heston(I, key, p, g);
            else if (I.model == SDE_MODEL_LINEAR) X = path_lin(I, key, p, g, err);
            else if (I.nvars == 1) X = path_ou<1>(I, key, p, g);
            else if (I.nvars == 2) X = path_ou<2>(I, key, p, g);
            else X = path_ou<4>(I, key, p, g);
            n += 1.f;
            const float dd = X - mean;
            mean += dd / n;
            m2 = fmaf(dd, X - mean, m2);
#pragma unroll
            for (int j = 0; j < NB_GRAD; ++j) kahan(gs[j], gc[j], g[j]);
        }
        // warp merge: Chan for (n, mean, M2) in FP64, sums of the derivatives
        double dn = n, dmean = mean, dm2 = m2;
        double dg[NB_GRAD];
#pragma unroll
        for (int j = 0; j < NB_GRAD; ++j) dg[j] = (double)gs[j] - (double)gc[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double on = __shfl_xor_sync(0xffffffffu, dn, o);
            const double om = __shfl_xor_sync(0xffffffffu, dmean, o);
            const double o2 = __shfl_xor_sync(0xffffffffu, dm2, o);
            const double tn = dn + on;
            if (tn > 0.0) {
                const double delta = om - dmean;
                dmean = dmean + delta * (on / tn);
                dm2 = dm2 + o2 + delta * delta * (dn * on / tn);
            }
            dn = tn;
#pragma unroll
            for (int j = 0; j < NB_GRAD; ++j) dg[j] += __shfl_xor_sync(0xffffffffu, dg[j], o);
        }
        if (lane == 0) {
            double *w = part + (int64_t)it * NB_PART;
            w[0] = dn;
            w[1] = dmean;
            w[2] = dm2;
            for (int j = 0; j < NB_GRAD; ++j) w[3 + j] = dg[j];
        }
    }
}

// merge the partials of every instance in a fixed order: res[i] = (n, mean, std, grad[8]/n)
__global__ void batch_merge_kernel(const double *part, const int *item_start, const int *item_list, int n_inst,
                                   double *res) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_inst) return;
    double n = 0, mean = 0, m2 = 0, g[NB_GRAD] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int t = item_start[i]; t < item_start[i + 1]; ++t) {
        const double *w = part + (int64_t)item_list[t] * NB_PART;
        const double tn = n + w[0];
        if (tn > 0) {
            const double delta = w[1] - mean;
            mean = mean + delta * (w[0] / tn);
            m2 = m2 + w[2] + delta * delta * (n * w[0] / tn);
        }
        n = tn;
        for (int j = 0; j < NB_GRAD; ++j) g[j] += w[3 + j];
    }
    double *r = res + (int64_t)i * (3 + NB_GRAD);
    r[0] = n;
    r[1] = mean;
    r[2] = n > 0 ? sqrt(m2 / n) : 0.0;
    for (int j = 0; j < NB_GRAD; ++j) r[3 + j] = n > 0 ? g[j] / n : 0.0;
}

struct Plan {
    int dev = -1;
    int n_inst = 0, n_items = 0, slab = 0, blocks = 0;
    int n_light = 0;        // items [0, n_light) are linear / OU, the rest Heston
    int blocks_heavy = 0;   // persistent grid of the Heston launch
    DevInst *d_inst = nullptr;
    Item *d_items = nullptr;
    int *d_start = nullptr, *d_list = nullptr;
    unsigned int *d_counter = nullptr;
    double *d_part = nullptr, *d_res = nullptr;
    int32_t *d_err = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double last_ms = 0;
};

std::mutex g_bmu;
std::vector<Plan *> g_plans;

void plan_free(Plan *P) {
    if (!P) return;
    if (P->exec) cudaGraphExecDestroy(P->exec);
    if (P->graph) cudaGraphDestroy(P->graph);
    cudaFree(P->d_inst);
    cudaFree(P->d_items);
    cudaFree(P->d_start);
    cudaFree(P->d_list);
    cudaFree(P->d_counter);
    cudaFree(P->d_part);
    cudaFree(P->d_res);
    cudaFree(P->d_err);
    if (P->e0) cudaEventDestroy(P->e0);
    if (P->e1) cudaEventDestroy(P->e1);
    if (P->stream) cudaStreamDestroy(P->stream);
    delete P;
}

int enqueue(Plan *P) {
    CUB(cudaMemsetAsync(P->d_counter, 0, 2 * sizeof(unsigned int), P->stream));
    // Heston first (the longest items), then the light class
    const int nh = P->n_items - P->n_light;
    if (nh > 0)
        batch_kernel<1><<<P->blocks_heavy, BLOCK, 0, P->stream>>>(P->d_inst, P->d_items + P->n_light, nh,
                                                                   P->d_counter + 1, P->d_part + (size_t)P->n_light * NB_PART,
                                                                   P->d_err);
    if (P->n_light > 0)
        batch_kernel<0><<<P->blocks, BLOCK, 0, P->stream>>>(P->d_inst, P->d_items, P->n_light, P->d_counter,
                                                             P->d_part, P->d_err);
    CUB(cudaGetLastError());
    batch_merge_kernel<<<(P->n_inst + 127) / 128, 128, 0, P->stream>>>(P->d_part, P->d_start, P->d_list,
                                                                     P->n_inst, P->d_res);
    CUB(cudaGetLastError());
    return SDE_OK;
}

}  // namespace

extern "C" int32_t sde_batch_create(const SdeBatchInstance *inst, int32_t n, int32_t slab, int32_t *handle) {
    if (!inst || n < 1 || !handle) return bfail(SDE_ERR_INVALID, "bad batch arguments");
    if (slab < 32 || slab % 32 != 0 || slab > (1 << 20)) return bfail(SDE_ERR_INVALID, "slab must be a multiple of 32");
    std::vector<DevInst> hi(n);
    std::vector<Item> items;
    for (int i = 0; i < n; ++i) {
        const SdeBatchInstance &s = inst[i];
        DevInst &d = hi[i];
        memset(&d, 0, sizeof d);
        if (s.model != SDE_MODEL_LINEAR && s.model != SDE_MODEL_OU && s.model != SDE_MODEL_HESTON)
            return bfail(SDE_ERR_UNSUPPORTED, "instance %d: unknown model", i);
        if (s.paths < 1 || s.paths > 0x7fffffffLL || s.n_steps < 1 || !(s.T > 0))
            return bfail(SDE_ERR_INVALID, "instance %d: bad paths / steps / horizon", i);
        if (s.model == SDE_MODEL_HESTON && s.nvars != 2) return bfail(SDE_ERR_INVALID, "instance %d: Heston has 2 states", i);
        if (s.model == SDE_MODEL_LINEAR && s.nvars != 1) return bfail(SDE_ERR_UNSUPPORTED, "instance %d: 1 state", i);
        if (s.nvars < 1 || s.nvars > 4) return bfail(SDE_ERR_UNSUPPORTED, "instance %d: 1..4 states", i);
        if (s.jump_law != SDE_JUMP_NONE && (s.model != SDE_MODEL_LINEAR || s.jump_law != SDE_JUMP_NORM))
            return bfail(SDE_ERR_UNSUPPORTED, "instance %d: normal jumps on the linear model only", i);
        d.model = s.model;
        d.jump_law = s.jump_law;
        d.nvars = s.nvars;
        d.n_steps = s.n_steps;
        d.paths = s.paths;
        const double dt = s.T / s.n_steps, sq = sqrt(dt);
        d.dt = (float)dt;
        d.sq = (float)sq;
        for (int m = 0; m < s.nvars; ++m) {
            d.x0[m] = (float)s.x0[m];
            d.p0[m] = (float)s.params[0][m];
            d.p1[m] = (float)s.params[1][m];
            d.p2[m] = (float)s.params[2][m];
            if (s.model == SDE_MODEL_OU) {
                d.d[m] = (float)(s.params[0][m] * dt);
                d.b[m] = (float)(s.params[0][m] * s.params[1][m] * dt);
                d.c[m] = (float)(s.params[2][m] * sq);
            } else if (s.model == SDE_MODEL_LINEAR) {
                d.b[m] = (float)(s.params[0][m] * dt);
                d.c[m] = (float)(s.params[1][m] * sq);
            }
        }
        if (s.jump_law == SDE_JUMP_NORM) {
            const double L = s.params[2][0] * dt;
            if (!(L >= 0) || L > 700) return bfail(SDE_ERR_INVALID, "instance %d: bad intensity", i);
            d.p0d = exp(-L);
            d.lamdt = L;
            poisson_thresholds(d.p0d, d.lamdt, d.thr, d.thr1);
            d.ja = (float)s.params[3][0];
            d.jb = (float)s.params[4][0];
        }
        if (s.model == SDE_MODEL_HESTON) {
            if (!(fabs(s.rho) < 1)) return bfail(SDE_ERR_INVALID, "instance %d: |rho| must be < 1", i);
            d.rho = (float)s.rho;
            d.chol10 = (float)s.rho;
            d.chol11 = (float)sqrt(1 - s.rho * s.rho);
            d.rho_k = (float)(-s.rho / sqrt(1 - s.rho * s.rho));
        }
        d.key = philox_schedule(s.seed);
        d.stream = s.stream;
        d.out_exp = s.out_exp;
        for (int64_t b = 0; b < s.paths; b += slab) {
            Item it;
            it.inst = i;
            it.base = b;
            it.nslab = (int)std::min<int64_t>(slab, s.paths - b);
            items.push_back(it);
        }
    }
    // the light class first, then Heston; longest first within each
    std::stable_sort(items.begin(), items.end(), [&](const Item &x, const Item &y) {
        const int cx = hi[x.inst].model == SDE_MODEL_HESTON, cy = hi[y.inst].model == SDE_MODEL_HESTON;
        if (cx != cy) return cx < cy;
        return (int64_t)hi[x.inst].n_steps * x.nslab > (int64_t)hi[y.inst].n_steps * y.nslab;
    });
    int n_light = 0;
    for (const Item &it : items) n_light += hi[it.inst].model != SDE_MODEL_HESTON;
    // per-instance item lists (ascending item index: a fixed merge order)
    std::vector<int> start(n + 1, 0), list(items.size());
    for (const Item &it : items) start[it.inst + 1]++;
    for (int i = 0; i < n; ++i) start[i + 1] += start[i];
    {
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int t = 0; t < (int)items.size(); ++t) list[fill[items[t].inst]++] = t;
    }
    Plan *P = new Plan();
    cudaGetDevice(&P->dev);
    P->n_inst = n;
    P->n_items = (int)items.size();
    P->slab = slab;
    P->n_light = n_light;
    int sms = 0, bps = 0, bph = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, P->dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, batch_kernel<0>, BLOCK, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bph, batch_kernel<1>, BLOCK, 0);
    P->blocks = sms * (bps > 0 ? bps : 1);
    P->blocks_heavy = sms * (bph > 0 ? bph : 1);
    int rc = SDE_OK;
#define CUP(call)                                                                                        \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            rc = bfail(SDE_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));                    \
            plan_free(P);                                                                                \
            return rc;                                                                                   \
        }                                                                                                \
    } while (0)
    CUP(cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking));
    CUP(cudaEventCreate(&P->e0));
    CUP(cudaEventCreate(&P->e1));
    CUP(cudaMalloc(&P->d_inst, sizeof(DevInst) * n));
    CUP(cudaMalloc(&P->d_items, sizeof(Item) * items.size()));
    CUP(cudaMalloc(&P->d_start, sizeof(int) * (n + 1)));
    CUP(cudaMalloc(&P->d_list, sizeof(int) * items.size()));
    CUP(cudaMalloc(&P->d_counter, 2 * sizeof(unsigned int)));
    CUP(cudaMalloc(&P->d_part, sizeof(double) * NB_PART * items.size()));
    CUP(cudaMalloc(&P->d_res, sizeof(double) * (3 + NB_GRAD) * n));
    CUP(cudaMalloc(&P->d_err, 16));
    CUP(cudaMemcpy(P->d_inst, hi.data(), sizeof(DevInst) * n, cudaMemcpyHostToDevice));
    CUP(cudaMemcpy(P->d_items, items.data(), sizeof(Item) * items.size(), cudaMemcpyHostToDevice));
    CUP(cudaMemcpy(P->d_start, start.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
    CUP(cudaMemcpy(P->d_list, list.data(), sizeof(int) * items.size(), cudaMemcpyHostToDevice));
    CUP(cudaMemset(P->d_err, 0, 16));
#undef CUP
    std::lock_guard<std::mutex> lk(g_bmu);
    g_plans.push_back(P);
    *handle = (int32_t)g_plans.size() - 1;
    return SDE_OK;
}

static Plan *get_plan(int32_t h) {
    std::lock_guard<std::mutex> lk(g_bmu);
    if (h < 0 || h >= (int32_t)g_plans.size()) return nullptr;
    return g_plans[h];
}

extern "C" int32_t sde_batch_run(int32_t handle, int32_t use_graph, double *results, double *ms) {
    Plan *P = get_plan(handle);
    if (!P) return bfail(SDE_ERR_INVALID, "unknown batch handle %d", handle);
    int rc;
    CUB(cudaEventRecord(P->e0, P->stream));
    if (use_graph) {
        if (!P->exec) {
            CUB(cudaStreamBeginCapture(P->stream, cudaStreamCaptureModeThreadLocal));
            rc = enqueue(P);
            cudaGraph_t g = nullptr;
            cudaError_t ce = cudaStreamEndCapture(P->stream, &g);
            if (rc) return rc;
            if (ce != cudaSuccess) return bfail(SDE_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
            P->graph = g;
            CUB(cudaGraphInstantiate(&P->exec, P->graph, 0));
        }
        CUB(cudaGraphLaunch(P->exec, P->stream));
    } else {
        if ((rc = enqueue(P))) return rc;
    }
    CUB(cudaEventRecord(P->e1, P->stream));
    if (results)
        CUB(cudaMemcpyAsync(results, P->d_res, sizeof(double) * (3 + NB_GRAD) * P->n_inst, cudaMemcpyDeviceToHost,
                            P->stream));
    int32_t herr = 0;
    CUB(cudaMemcpyAsync(&herr, P->d_err, sizeof herr, cudaMemcpyDeviceToHost, P->stream));
    CUB(cudaStreamSynchronize(P->stream));
    float t = 0.f;
    CUB(cudaEventElapsedTime(&t, P->e0, P->e1));
    P->last_ms = t;
    if (ms) *ms = t;
    if (herr) return bfail(SDE_ERR_DEVICE, "batch kernel error flag %d", herr);
    return SDE_OK;
}

extern "C" int32_t sde_batch_destroy(int32_t handle) {
    std::lock_guard<std::mutex> lk(g_bmu);
    if (handle < 0 || handle >= (int32_t)g_plans.size() || !g_plans[handle])
        return bfail(SDE_ERR_INVALID, "unknown batch handle %d", handle);
    plan_free(g_plans[handle]);
    g_plans[handle] = nullptr;
    return SDE_OK;
}

extern "C" int32_t sde_batch_info(int32_t handle, int32_t *info) {
    Plan *P = get_plan(handle);
    if (!P || !info) return bfail(SDE_ERR_INVALID, "unknown batch handle %d", handle);
    info[0] = P->n_inst;
    info[1] = P->n_items;
    info[2] = P->slab;
    info[3] = P->blocks;
    return SDE_OK;
}
