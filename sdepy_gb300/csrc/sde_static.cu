// sde_run_stats_static: the fused montecarlo summary of sde_run_stats for
// callers that cannot allocate device memory.
//
// Who needs it: hosts that must not call cudaMalloc once they are running --
// a serving or real-time loop where an allocation's implicit device
// synchronisation and latency are not acceptable, a plugin living inside a
// framework that owns all device memory through its own pool and forbids
// outside allocations, or a process whose memory budget is fixed at start-up.
// sde_run_stats allocates (and caches) device scratch for its tables, block
// partials and histogram; this variant uses instead one file-scope
// __device__ array of STATIC_SCRATCH_BYTES (16 MiB) that every GPU loading
// the library holds until the process exits.
//
// Limits and behaviour:
//   * device-RNG paths, no jumps, no path output (the summary only), the
//     summarised row given by req->row;
//   * everything the call needs (grid, coefficients, tables, block partials,
//     results, histogram and, when bins > 0 or for the FP32 LINEAR / OU
//     kernels, the summarised values) must fit in the 16 MiB array; larger
//     requests fail with SDE_ERR_INVALID;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) -- make that first
//     call before any stream capture.  The address is kept for the life of
//     the process: do not call this entry again on a device after
//     cudaDeviceReset (the reset unloads the module, and a reloaded array
//     may sit elsewhere);
//   * calls share the array, which keeps the last call's contents: the
//     counters are cleared at the start of every call, and calls that
//     overlap on the GPU would race (calls from different host threads are
//     serialised here; each call synchronises its stream before returning).
// No cudaMalloc, cudaFree or other allocating routine is called.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "sde_kernels.cuh"
#include "sde_stats.cuh"

using namespace sdegpu;

namespace sdegpu {
int set_last_error(int code, const char *msg);  // defined with the other entry points
}

namespace {

constexpr size_t STATIC_SCRATCH_BYTES = (size_t)16 << 20;

static __device__ __align__(256) unsigned char g_static_scratch[STATIC_SCRATCH_BYTES];

std::mutex g_static_mu;
void *g_static_ptr[64] = {};
int g_static_sms[64] = {};

int fail_static(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return set_last_error(code, buf);
}

#define CUS(call)                                                                               \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return fail_static(SDE_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));   \
    } while (0)

// per-step and per-variable tables in the run's precision, from the raw
// double inputs copied into the array
template <typename R>
__global__ void static_tables_kernel(const double *tt, int n_pts, const double *x0, const double *prm, int W,
                                     R *dt, R *sqdt, R *x0r, R *prmr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_pts - 1) {
        const double d = tt[i + 1] - tt[i];
        dt[i] = (R)d;
        sqdt[i] = (R)sqrt(fabs(d));
    }
    if (i < W) x0r[i] = (R)x0[i];
    if (i < SDE_MAX_PARAMS * W) prmr[i] = (R)prm[i];
}

// one run per step: (k, k + 1, row stored after step k, coefficient row k)
__global__ void static_runs_kernel(const int32_t *out_row, int n_steps, int4 *runs) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n_steps) runs[k] = make_int4(k, k + 1, out_row[k + 1], k);
}

// results [n_out][RES_STRIDE] -> moments [n_out][8] and payoff [n_out][n_strikes]
__global__ void static_pack_kernel(const double *res, int64_t n_out, int n_strikes, double *mom, double *pay) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n_out) return;
    for (int i = 0; i < 7; ++i) mom[o * 8 + i] = res[o * RES_STRIDE + i];
    mom[o * 8 + 7] = 0.0;
    for (int s = 0; s < n_strikes; ++s) pay[o * n_strikes + s] = res[o * RES_STRIDE + 9 + s];
}

struct Layout {
    size_t tt, row, x0, prm, dt, sq, x0r, prmr, coef, tshift, runs, part, res, edges, edges64, counts, vals, mom, pay, err, end;
};

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

template <typename R>
int run_static(const SdeSpec *s, const SdeGrid *gr, const SdeStatsReq *req, SdeStatsOut *so, cudaStream_t st) {
    // ---- validation (no allocation anywhere below) ---------------------------------
    if (!s || !gr || !req || !so || !so->moments) return fail_static(SDE_ERR_INVALID, "NULL argument");
    if (s->abi_version != SDE_ABI_VERSION) return fail_static(SDE_ERR_INVALID, "spec abi_version mismatch");
    if (s->model < SDE_MODEL_LINEAR || s->model > SDE_MODEL_CIR)
        return fail_static(SDE_ERR_UNSUPPORTED, "unknown model %d", s->model);
    if (s->jump_law != SDE_JUMP_NONE)
        return fail_static(SDE_ERR_UNSUPPORTED, "sde_run_stats_static does not integrate jump models");
    if (s->paths < 1 || s->paths > 0x7fffffffLL) return fail_static(SDE_ERR_INVALID, "paths out of range");
    if ((uint64_t)s->path_offset + (uint64_t)s->paths > 0x100000000ull)
        return fail_static(SDE_ERR_INVALID, "path_offset + paths must be <= 2^32");
    if (s->groups < 1 || s->groups > 65535) return fail_static(SDE_ERR_INVALID, "groups out of range");
    const int M = s->group_size;
    if (M < 1 || M > SDE_MAX_GROUP) return fail_static(SDE_ERR_UNSUPPORTED, "group size %d outside 1..%d", M, SDE_MAX_GROUP);
    if (s->model == SDE_MODEL_HESTON && M != 2 && M != 4 && M != 8 && M != 16)
        return fail_static(SDE_ERR_UNSUPPORTED, "Heston group size must be 2, 4, 8 or 16");
    if (!s->x0 || !s->params) return fail_static(SDE_ERR_INVALID, "x0 and params are required");
    int opg;
    switch (s->out_mode) {
    case SDE_OUT_STATE:
    case SDE_OUT_EXP: opg = M; break;
    case SDE_OUT_SUM: opg = 1; break;
    case SDE_OUT_HESTON_X: opg = M / 2; break;
    case SDE_OUT_HESTON_XY: opg = M; break;
    default: return fail_static(SDE_ERR_INVALID, "unknown out_mode %d", s->out_mode);
    }
    if ((s->out_mode == SDE_OUT_HESTON_X || s->out_mode == SDE_OUT_HESTON_XY) && s->model != SDE_MODEL_HESTON)
        return fail_static(SDE_ERR_INVALID, "Heston outputs need the Heston model");
    if (!gr->tt || !gr->out_row || gr->n_pts < 1) return fail_static(SDE_ERR_INVALID, "grid arrays are required");
    // a negative row would match the grid's unstored points (out_row -1)
    // and summarise nothing
    if (req->row < 0) return fail_static(SDE_ERR_INVALID, "stats row must be >= 0");
    bool row_seen = false;
    for (int k = 0; k < gr->n_pts; ++k) {
        if (!std::isfinite(gr->tt[k])) return fail_static(SDE_ERR_INVALID, "grid point %d is not finite", k);
        if (gr->out_row[k] < -1) return fail_static(SDE_ERR_INVALID, "grid out_row[%d] < -1", k);
        if (gr->out_row[k] == req->row) row_seen = true;
    }
    if (!row_seen) return fail_static(SDE_ERR_INVALID, "stats row %d is not on the grid", req->row);
    double sgn = 0.0;
    for (int k = 0; k + 1 < gr->n_pts; ++k) {
        const double d = gr->tt[k + 1] - gr->tt[k];
        const double sd = d < 0 ? -1.0 : 1.0;
        if (d == 0.0 || (sgn != 0.0 && sd != sgn))
            return fail_static(SDE_ERR_INVALID, "grid points must be strictly monotonic (step %d)", k);
        sgn = sd;
    }
    const int bins = req->bins;
    if (bins < 0) return fail_static(SDE_ERR_INVALID, "bins must be >= 0");
    if (bins > 0 && (!so->counts || !so->edges)) return fail_static(SDE_ERR_INVALID, "histogram arrays are required");
    if (req->n_strikes < 0 || req->n_strikes > SDE_MAX_STRIKES) return fail_static(SDE_ERR_INVALID, "bad n_strikes");
    if (req->n_strikes > 0 && !so->payoff) return fail_static(SDE_ERR_INVALID, "payoff array is required");
    if (req->has_range && !(std::isfinite(req->range_lo) && std::isfinite(req->range_hi) && req->range_lo <= req->range_hi))
        return fail_static(SDE_ERR_INVALID, "histogram range must be finite with min <= max");
    // the correlation factor, before anything is queued on the stream: a
    // failure below the first enqueue would leave work writing the shared
    // array after this call (and its lock) had returned
    double Lc[SDE_MAX_GROUP * SDE_MAX_GROUP];
    if (s->corr) {
        const int rc = sde_cholesky(s->corr, M, Lc);
        if (rc) return rc;
    }

    // ---- device and the array's address ------------------------------------------------
    int dev = 0;
    CUS(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail_static(SDE_ERR_NO_DEVICE, "device id out of range");
    if (!g_static_ptr[dev]) {
        void *p = nullptr;
        CUS(cudaGetSymbolAddress(&p, g_static_scratch));
        int sms = 0;
        CUS(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        g_static_sms[dev] = sms;
        g_static_ptr[dev] = p;
    }
    unsigned char *base = (unsigned char *)g_static_ptr[dev];

    const int W = s->groups * M, n_pts = gr->n_pts, n_steps = n_pts - 1;
    const int64_t paths = s->paths, n_out = (int64_t)s->groups * opg;
    int bps = 0;
    FwdLauncher<R> L = nullptr;
    const int maxm = M <= 1 ? 1 : M <= 2 ? 2 : M <= 4 ? 4 : M <= 8 ? 8 : 16;
    if constexpr (sizeof(R) == 4) {
        L = s->model == SDE_MODEL_CIR ? find_fwd_f32_cir(maxm, false, false, false, &bps)
                                      : find_fwd_f32_linear(s->model, maxm, false, false, &bps);
        if (!L) L = find_fwd_f32_ou_heston(s->model, maxm, false, false, &bps);
    } else {
        L = s->model == SDE_MODEL_CIR ? find_fwd_f64_cir(maxm, false, false, &bps)
                                      : find_fwd_f64_linear(s->model, maxm, false, false, &bps);
        if (!L) L = find_fwd_f64_ou_heston(s->model, maxm, false, false, &bps);
    }
    if (!L) return fail_static(SDE_ERR_UNSUPPORTED, "no kernel for model %d group size %d", s->model, M);
    // blocks along paths: the same rule as sde_run_stats
    if (bps < 1) bps = 1;
    int64_t want = (paths + BLOCK - 1) / BLOCK;
    int64_t per_group = ((int64_t)g_static_sms[dev] * bps + s->groups - 1) / s->groups;
    if (per_group < 1) per_group = 1;
    const int nbx = (int)(want < per_group ? want : per_group);

    // ---- layout of the array ------------------------------------------------------------------
    Layout lo;
    size_t o = 0;
    lo.tt = o; o = al256(o + sizeof(double) * n_pts);
    lo.row = o; o = al256(o + sizeof(int32_t) * n_pts);
    lo.x0 = o; o = al256(o + sizeof(double) * W);
    lo.prm = o; o = al256(o + sizeof(double) * SDE_MAX_PARAMS * W);
    lo.dt = o; o = al256(o + sizeof(R) * (n_steps + 1));
    lo.sq = o; o = al256(o + sizeof(R) * (n_steps + 1));
    lo.x0r = o; o = al256(o + sizeof(R) * W);
    lo.prmr = o; o = al256(o + sizeof(R) * SDE_MAX_PARAMS * W);
    const bool tab = sizeof(R) == 4 && (s->model == SDE_MODEL_LINEAR || s->model == SDE_MODEL_OU);
    lo.coef = o; o = al256(o + (tab ? sizeof(float) * 2 * (size_t)n_steps * s->groups * maxm : 0));
    lo.tshift = o; o = al256(o + (tab ? sizeof(float) * 2 * (size_t)s->groups * maxm : 0));
    lo.runs = o; o = al256(o + (tab ? sizeof(int4) * (size_t)n_steps : 0));
    lo.part = o; o = al256(o + sizeof(double) * NPART * (size_t)s->groups * nbx * opg);
    lo.res = o; o = al256(o + sizeof(double) * RES_STRIDE * n_out);
    lo.edges = o; o = al256(o + sizeof(R) * (size_t)(bins + 1) * n_out);
    lo.edges64 = o; o = al256(o + sizeof(double) * (size_t)(bins + 1) * n_out);
    lo.counts = o; o = al256(o + sizeof(int64_t) * (size_t)bins * n_out);
    // the summarised values: for the histogram, and for the kernels that
    // reduce the stored row in a second launch
    const bool need_vals = bins > 0 || fwd_summary_from_row(sizeof(R) == 4, s->model, false, false, false, false, false);
    lo.vals = o; o = al256(o + (need_vals ? sizeof(R) * (size_t)n_out * paths : 0));
    lo.mom = o; o = al256(o + sizeof(double) * 8 * n_out);
    lo.pay = o; o = al256(o + sizeof(double) * (size_t)req->n_strikes * n_out);
    lo.err = o; o = al256(o + 16);
    lo.end = o;
    if (lo.end > STATIC_SCRATCH_BYTES)
        return fail_static(SDE_ERR_INVALID,
                           "request needs %zu bytes of scratch; sde_run_stats_static holds %zu (use bins=0 "
                           "or fewer paths, or sde_run_stats)", lo.end, STATIC_SCRATCH_BYTES);

    // ---- inputs into the array, tables, cleared counters ------------------------------------------
    CUS(cudaMemcpyAsync(base + lo.tt, gr->tt, sizeof(double) * n_pts, cudaMemcpyHostToDevice, st));
    CUS(cudaMemcpyAsync(base + lo.row, gr->out_row, sizeof(int32_t) * n_pts, cudaMemcpyHostToDevice, st));
    CUS(cudaMemcpyAsync(base + lo.x0, s->x0, sizeof(double) * W, cudaMemcpyHostToDevice, st));
    CUS(cudaMemcpyAsync(base + lo.prm, s->params, sizeof(double) * SDE_MAX_PARAMS * W, cudaMemcpyHostToDevice, st));
    const int nt = n_pts > SDE_MAX_PARAMS * W ? n_pts : SDE_MAX_PARAMS * W;
    static_tables_kernel<R><<<(nt + 255) / 256, 256, 0, st>>>(
        (const double *)(base + lo.tt), n_pts, (const double *)(base + lo.x0), (const double *)(base + lo.prm), W,
        (R *)(base + lo.dt), (R *)(base + lo.sq), (R *)(base + lo.x0r), (R *)(base + lo.prmr));
    CUS(cudaGetLastError());
    CUS(cudaMemsetAsync(base + lo.err, 0, 16, st));
    if (bins > 0) CUS(cudaMemsetAsync(base + lo.counts, 0, sizeof(int64_t) * (size_t)bins * n_out, st));

    FwdArgs<R> a;
    memset(&a, 0, sizeof a);
    if (s->corr) {
        for (int i = 0; i < M; ++i)
            for (int j = 0; j <= i; ++j) a.chol[i * (i + 1) / 2 + j] = (R)Lc[i * M + j];
        a.has_corr = 1;
    }
    a.paths = paths;
    a.groups = s->groups;
    a.M = M;
    a.W = W;
    a.n_pts = n_pts;
    a.step_offset = gr->step_offset;
    a.jump_law = SDE_JUMP_NONE;
    a.out_mode = s->out_mode;
    a.opg = opg;
    a.seed = s->seed;
    a.stream = s->stream;
    a.path_offset = s->path_offset;
    a.tab_row0 = gr->out_row[0];
    a.sgn = (R)(sgn < 0 ? -1.0 : 1.0);
    a.dt = (const R *)(base + lo.dt);
    a.sqdt = (const R *)(base + lo.sq);
    a.out_row = (const int32_t *)(base + lo.row);
    a.x0 = (const R *)(base + lo.x0r);
    a.prm = (const R *)(base + lo.prmr);
    a.key = philox_schedule(s->seed);
    a.coef = nullptr;
    if (tab && n_steps > 0) {
        // the FP32 LINEAR / OU kernels read their per-step coefficients
        const int64_t n = (int64_t)n_steps * s->groups * maxm;
        coef_table_kernel<<<(unsigned)((n + BLOCK - 1) / BLOCK), BLOCK, 0, st>>>(
            (const double *)(base + lo.tt), n_steps, (const double *)(base + lo.x0), (const double *)(base + lo.prm),
            s->groups, M, maxm, s->model, (float *)(base + lo.coef), (float *)(base + lo.tshift));
        CUS(cudaGetLastError());
        a.coef = (const float *)(base + lo.coef);
        a.tshift = s->model == SDE_MODEL_OU ? (const float *)(base + lo.tshift) : nullptr;
        static_runs_kernel<<<(n_steps + 255) / 256, 256, 0, st>>>((const int32_t *)(base + lo.row), n_steps,
                                                                 (int4 *)(base + lo.runs));
        CUS(cudaGetLastError());
        a.runs = (const int4 *)(base + lo.runs);
        a.n_runs = n_steps;
    }
    a.n_out_vars = n_out;
    a.stats_row = req->row;
    a.n_strikes = req->n_strikes;
    for (int i = 0; i < req->n_strikes; ++i) a.strikes[i] = (R)req->strikes[i];
    a.partials = (double *)(base + lo.part);
    a.stats_vals = need_vals ? (R *)(base + lo.vals) : nullptr;
    a.err = (int32_t *)(base + lo.err);
    L(a, dim3(nbx, s->groups), st);
    CUS(cudaGetLastError());

    stats_finalize_kernel<R><<<(unsigned)n_out, BLOCK, 0, st>>>(
        a.partials, nbx, opg, req->n_strikes, bins, req->has_range, req->range_lo, req->range_hi,
        (double *)(base + lo.res), (R *)(base + lo.edges), (double *)(base + lo.edges64), a.err);
    CUS(cudaGetLastError());
    if (bins > 0) {
        int hb = (int)((paths + BLOCK * 16 - 1) / (BLOCK * 16));
        if (hb > 4 * g_static_sms[dev]) hb = 4 * g_static_sms[dev];
        if (hb < 1) hb = 1;
        const size_t smem = bins <= HIST_SMEM_BINS ? sizeof(unsigned) * bins : 0;
        hist_kernel<R><<<dim3(hb, (unsigned)n_out), BLOCK, smem, st>>>(
            a.stats_vals, paths, paths, bins, (const R *)(base + lo.edges), (const double *)(base + lo.res),
            req->has_range, (unsigned long long *)(base + lo.counts));
        CUS(cudaGetLastError());
    }
    static_pack_kernel<<<(unsigned)((n_out + 255) / 256), 256, 0, st>>>(
        (const double *)(base + lo.res), n_out, req->n_strikes, (double *)(base + lo.mom), (double *)(base + lo.pay));
    CUS(cudaGetLastError());

    // ---- results straight into the caller's arrays -------------------------------------------
    CUS(cudaMemcpyAsync(so->moments, base + lo.mom, sizeof(double) * 8 * n_out, cudaMemcpyDeviceToHost, st));
    if (req->n_strikes > 0)
        CUS(cudaMemcpyAsync(so->payoff, base + lo.pay, sizeof(double) * req->n_strikes * n_out, cudaMemcpyDeviceToHost, st));
    if (bins > 0) {
        CUS(cudaMemcpyAsync(so->counts, base + lo.counts, sizeof(int64_t) * (size_t)bins * n_out, cudaMemcpyDeviceToHost, st));
        CUS(cudaMemcpyAsync(so->edges, base + lo.edges64, sizeof(double) * (size_t)(bins + 1) * n_out, cudaMemcpyDeviceToHost, st));
    }
    int32_t herr = 0;
    CUS(cudaMemcpyAsync(&herr, base + lo.err, sizeof herr, cudaMemcpyDeviceToHost, st));
    CUS(cudaStreamSynchronize(st));
    if (herr & ERRF_RANGE) return fail_static(SDE_ERR_INVALID, "autodetected range of the histogram is not finite");
    if (herr) return fail_static(SDE_ERR_DEVICE, "kernel error flag %d", herr);
    return SDE_OK;
}

}  // namespace

extern "C" int32_t sde_run_stats_static(const SdeSpec *spec, const SdeGrid *grid, const SdeStatsReq *req,
                                        SdeStatsOut *stats, void *stream) {
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!spec) return fail_static(SDE_ERR_INVALID, "spec is NULL");
    if (grid && (grid->params_t || grid->corr_t))
        return fail_static(SDE_ERR_UNSUPPORTED, "constant parameters and correlation only (grid params_t and "
                                                "corr_t must be NULL)");
    if (spec->flags) return fail_static(SDE_ERR_UNSUPPORTED, "no spec flags (antithetic paths)");
    if (spec->precision == SDE_FP32) return run_static<float>(spec, grid, req, stats, (cudaStream_t)stream);
    if (spec->precision == SDE_FP64) return run_static<double>(spec, grid, req, stats, (cudaStream_t)stream);
    return fail_static(SDE_ERR_UNSUPPORTED, "unknown precision %d", spec->precision);
}
