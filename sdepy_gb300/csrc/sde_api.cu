// C-ABI runtime of sdepy_gb300: argument validation, host-side tables,
// device scratch cache, kernel dispatch and copies (include/sdepy_gb300.h).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "sde_kernels.cuh"
#include "sde_stats.cuh"
#include "sde_adjoint.cuh"
#include "sde_runtime.h"
#include "sde_jit.h"

using namespace sdegpu;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string g_err;

static int fail(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

namespace sdegpu {
// error text of entry points defined in other translation units
int set_last_error(int code, const char *msg) {
    g_err = msg;
    return code;
}
}  // namespace sdegpu

#define CU(call)                                                                         \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return fail(SDE_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));   \
    } while (0)

// ---------------------------------------------------------------------------
// per-device state: one blocking stream (ordered with the legacy default
// stream that torch uses by default) and a grow-only scratch cache
// ---------------------------------------------------------------------------
enum Slot {
    S_TABLES, S_NOISE_DW, S_NOISE_DJ, S_NOISE_DN, S_XX, S_NEG, S_JCNT, S_ROWJ,
    S_PART, S_RES, S_EDGES, S_EDGES64, S_COUNTS, S_VALS, S_ERR, S_SAMPLE, S_COEF,
    S_AUX0, S_AUX1, S_AUX2, S_AUX3, N_SLOTS   // entry points of other translation units
};

struct Device {
    bool init = false;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t user_stream = nullptr;
    bool has_user_stream = false;
    void *ptr[N_SLOTS] = {};
    size_t cap[N_SLOTS] = {};
    std::vector<char> host_tables;
    // optional kernel timing: events around the forward kernel and the
    // statistics kernels of the last call, on the launching stream
    bool timing = false;
    cudaEvent_t ev[4] = {};
    double last_ms[4] = {};
};

static std::mutex g_mu;
static Device g_dev[64];

static int current_device(Device **out) {
    int d = 0;
    cudaError_t e = cudaGetDevice(&d);
    if (e != cudaSuccess) return fail(SDE_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    if (d < 0 || d >= 64) return fail(SDE_ERR_NO_DEVICE, "device id %d out of range", d);
    Device &D = g_dev[d];
    if (!D.init) {
        int n = 0;
        CU(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d));
        D.sms = n;
        CU(cudaStreamCreate(&D.stream));
        for (int i = 0; i < 4; ++i) CU(cudaEventCreate(&D.ev[i]));
        D.init = true;
    }
    *out = &D;
    return SDE_OK;
}

static cudaStream_t dev_stream(Device *D) { return D->has_user_stream ? D->user_stream : D->stream; }

static int scratch(Device *D, Slot s, size_t bytes, void **p) {
    if (bytes == 0) bytes = 16;
    if (D->cap[s] < bytes) {
        if (D->ptr[s]) {
            CU(cudaStreamSynchronize(dev_stream(D)));
            CU(cudaFree(D->ptr[s]));
            D->ptr[s] = nullptr;
            D->cap[s] = 0;
        }
        size_t want = bytes + bytes / 8;
        CU(cudaMalloc(&D->ptr[s], want));
        D->cap[s] = want;
    }
    *p = D->ptr[s];
    return SDE_OK;
}

// ---------------------------------------------------------------------------
// runtime services for entry points defined in other translation units: the
// caller holds rt_mutex() for the whole call
// ---------------------------------------------------------------------------
namespace sdegpu {
std::mutex &rt_mutex() { return g_mu; }

int rt_begin(RtCall *c) {
    Device *D;
    int rc = current_device(&D);
    if (rc) return rc;
    c->st = dev_stream(D);
    c->sms = D->sms;
    c->timing = D->timing;
    c->ev0 = D->ev[0];
    c->ev1 = D->ev[1];
    c->last_ms = D->last_ms;
    return SDE_OK;
}

int rt_scratch(int aux, size_t bytes, void **p) {
    if (aux < 0 || aux > S_AUX3 - S_AUX0) return fail(SDE_ERR_INVALID, "scratch slot %d", aux);
    Device *D;
    int rc = current_device(&D);
    if (rc) return rc;
    return scratch(D, (Slot)(S_AUX0 + aux), bytes, p);
}

int rt_fail(int code, const char *msg) { return fail(code, "%s", msg); }
}  // namespace sdegpu

// ---------------------------------------------------------------------------
// exported utilities
// ---------------------------------------------------------------------------
extern "C" int32_t sde_abi_version(void) { return SDE_ABI_VERSION; }

extern "C" int32_t sde_last_error(char *buf, int32_t len) {
    if (!buf || len <= 0) return SDE_ERR_INVALID;
    snprintf(buf, (size_t)len, "%s", g_err.c_str());
    return SDE_OK;
}

extern "C" int32_t sde_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

extern "C" int32_t sde_release(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= 64) return SDE_OK;
    Device &D = g_dev[d];
    if (!D.init) return SDE_OK;
    cudaStreamSynchronize(dev_stream(&D));
    for (int s = 0; s < N_SLOTS; ++s) {
        if (D.ptr[s]) cudaFree(D.ptr[s]);
        D.ptr[s] = nullptr;
        D.cap[s] = 0;
    }
    return SDE_OK;
}

extern "C" int32_t sde_timing(int32_t enable, double *last_ms) {
    std::lock_guard<std::mutex> lk(g_mu);
    Device *D;
    int rc = current_device(&D);
    if (rc) return rc;
    if (last_ms)
        for (int i = 0; i < 4; ++i) last_ms[i] = D->last_ms[i];
    if (enable >= 0) D->timing = enable != 0;
    return SDE_OK;
}

// ---------------------------------------------------------------------------
// the Box-Muller transform of given word pairs, as the kernels apply it
// ---------------------------------------------------------------------------
template <typename R>
static __global__ void normal_pairs_kernel(const uint32_t *words, int64_t n, double *out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    R z0, z1;
    Rng<R>::normal2(words[2 * i], words[2 * i + 1], z0, z1);
    out[2 * i] = (double)z0;
    out[2 * i + 1] = (double)z1;
}

extern "C" int32_t sde_normal_pairs(const uint32_t *words, int64_t n, int32_t precision, double *out) {
    if (!words || !out || n < 0 || n > (1ll << 30)) return fail(SDE_ERR_INVALID, "sde_normal_pairs: bad arguments");
    if (precision != SDE_FP64 && precision != SDE_FP32)
        return fail(SDE_ERR_UNSUPPORTED, "unknown precision %d", precision);
    if (n == 0) return SDE_OK;
    std::lock_guard<std::mutex> lock(g_mu);
    Device *D;
    int rc;
    if ((rc = current_device(&D))) return rc;
    cudaStream_t st = D->stream;
    void *dw, *dz;
    if ((rc = scratch(D, S_NOISE_DW, sizeof(uint32_t) * 2 * (size_t)n, &dw))) return rc;
    if ((rc = scratch(D, S_NOISE_DJ, sizeof(double) * 2 * (size_t)n, &dz))) return rc;
    CU(cudaMemcpyAsync(dw, words, sizeof(uint32_t) * 2 * (size_t)n, cudaMemcpyHostToDevice, st));
    const unsigned nb = (unsigned)((n + BLOCK - 1) / BLOCK);
    if (precision == SDE_FP64) normal_pairs_kernel<double><<<nb, BLOCK, 0, st>>>((const uint32_t *)dw, n, (double *)dz);
    else normal_pairs_kernel<float><<<nb, BLOCK, 0, st>>>((const uint32_t *)dw, n, (double *)dz);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(out, dz, sizeof(double) * 2 * (size_t)n, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return SDE_OK;
}

extern "C" int32_t sde_host_alloc(int64_t bytes, void **ptr) {
    if (!ptr || bytes < 1) return fail(SDE_ERR_INVALID, "sde_host_alloc: bad arguments");
    *ptr = nullptr;
    CU(cudaHostAlloc(ptr, (size_t)bytes, cudaHostAllocPortable));
    return SDE_OK;
}

extern "C" int32_t sde_host_free(void *ptr) {
    if (!ptr) return SDE_OK;
    CU(cudaFreeHost(ptr));
    return SDE_OK;
}

extern "C" int32_t sde_set_stream(void *stream) {
    std::lock_guard<std::mutex> lk(g_mu);
    Device *D;
    int rc = current_device(&D);
    if (rc) return rc;
    D->user_stream = (cudaStream_t)stream;
    D->has_user_stream = stream != nullptr;
    return SDE_OK;
}

// Cholesky-Banachiewicz, row by row: L[i][j] = (C[i][j] - sum_{k<j} L[i][k] L[j][k]) / L[j][j],
// L[i][i] = sqrt(C[i][i] - sum_{k<i} L[i][k]^2).  A pivot <= 1e-14 * C[i][i]
// (semi-definite input, e.g. |rho| = 1) gives a zero column.
extern "C" int32_t sde_cholesky(const double *C, int32_t M, double *L) {
    if (!C || !L || M < 1 || M > 1024) return fail(SDE_ERR_INVALID, "sde_cholesky: bad arguments");
    for (int i = 0; i < M * M; ++i) L[i] = 0.0;
    for (int i = 0; i < M; ++i) {
        for (int j = 0; j <= i; ++j) {
            double s = C[i * M + j];
            for (int k = 0; k < j; ++k) s -= L[i * M + k] * L[j * M + k];
            if (i == j) {
                const double tol = 1e-14 * fabs(C[i * M + i]);
                if (s < -1e-10 * fabs(C[i * M + i]) - 1e-300)
                    return fail(SDE_ERR_INVALID, "correlation matrix is not positive semi-definite");
                L[i * M + i] = s > tol ? sqrt(s) : 0.0;
            } else {
                L[i * M + j] = L[j * M + j] > 0.0 ? s / L[j * M + j] : 0.0;
            }
        }
    }
    return SDE_OK;
}

// ---------------------------------------------------------------------------
// validation
// ---------------------------------------------------------------------------
static int check_spec(const SdeSpec *s, int *opg) {
    if (!s) return fail(SDE_ERR_INVALID, "spec is NULL");
    if (s->abi_version != SDE_ABI_VERSION)
        return fail(SDE_ERR_INVALID, "spec abi_version %d != %d", s->abi_version, SDE_ABI_VERSION);
    if (s->model < SDE_MODEL_LINEAR || s->model > SDE_MODEL_USER)
        return fail(SDE_ERR_UNSUPPORTED, "unknown model %d", s->model);
    if (s->model == SDE_MODEL_USER) {
        // every register and constant index in range before a launch
        const SdeUserProgram *u = s->program;
        if (!u) return fail(SDE_ERR_INVALID, "a user SDE needs its program");
        if (u->n_ops < 0 || u->n_ops > SDE_USER_MAX_OPS) return fail(SDE_ERR_INVALID, "user program: n_ops");
        if (u->n_terms < 0 || u->n_terms > SDE_USER_MAX_TERMS) return fail(SDE_ERR_INVALID, "user program: n_terms");
        if (u->n_eq < 1 || u->n_eq > SDE_USER_MAX_EQ || s->group_size % u->n_eq)
            return fail(SDE_ERR_INVALID, "user program: %d equations in groups of %d", u->n_eq, s->group_size);
        if (u->n_eq > 1 && s->group_size < 2) return fail(SDE_ERR_INVALID, "user program: system groups");
        int seen = 0;   // each source at most once
        for (int i = 0; i < u->n_terms; ++i) {
            const int src = u->term_source[i];
            if (src < SDE_SRC_DT || src > SDE_SRC_DJ || (seen & (1 << src)))
                return fail(SDE_ERR_INVALID, "user program: term %d", i);
            seen |= 1 << src;
            for (int e = 0; e < u->n_eq; ++e)
                if (u->term_register[e][i] < 0 || u->term_register[e][i] >= SDE_USER_MAX_REGS)
                    return fail(SDE_ERR_INVALID, "user program: term %d of equation %d", i, e);
        }
        for (int i = 0; i < u->n_ops; ++i) {
            const uint32_t op = u->ops[i];
            const uint32_t code = op & 0xff, d = (op >> 8) & 0xff, ra = (op >> 16) & 0xff, rb = op >> 24;
            if (code >= SDE_UOP_COUNT || d >= SDE_USER_MAX_REGS)
                return fail(SDE_ERR_INVALID, "user program: instruction %d", i);
            if (code == SDE_UOP_CONST ? ra >= SDE_USER_MAX_CONSTS : (ra >= SDE_USER_MAX_REGS || rb >= SDE_USER_MAX_REGS))
                return fail(SDE_ERR_INVALID, "user program: operand of instruction %d", i);
        }
        const bool has_dj = (seen >> SDE_SRC_DJ) & 1, has_dn = (seen >> SDE_SRC_DN) & 1;
        if (has_dj != (s->jump_law != SDE_JUMP_NONE))
            return fail(SDE_ERR_INVALID, "user program: a jump-size law goes with a dj term, and only with one");
        if ((has_dj || has_dn) && !u->jump_params)
            return fail(SDE_ERR_INVALID, "user program: dn / dj terms need jump_params");
        if (s->out_mode != SDE_OUT_STATE && s->out_mode != SDE_OUT_EXP)
            return fail(SDE_ERR_INVALID, "user SDEs store the state or its exp");
        if (s->flags & SDE_FLAG_ANTITHETIC) return fail(SDE_ERR_UNSUPPORTED, "antithetic paths of user SDEs");
    }
    if (s->precision != SDE_FP64 && s->precision != SDE_FP32)
        return fail(SDE_ERR_UNSUPPORTED, "unknown precision %d", s->precision);
    if (s->paths < 1 || s->paths > 0x7fffffffLL)
        return fail(SDE_ERR_INVALID, "paths must be in [1, 2^31-1], not %lld", (long long)s->paths);
    if ((uint64_t)s->path_offset + (uint64_t)s->paths > 0x100000000ull)
        return fail(SDE_ERR_INVALID, "path_offset + paths must be <= 2^32 (the counter's path word)");
    if (s->groups < 1) return fail(SDE_ERR_INVALID, "groups must be >= 1");
    if (s->groups > 65535) return fail(SDE_ERR_UNSUPPORTED, "more than 65535 groups per path");
    if (s->group_size < 1 || s->group_size > SDE_MAX_GROUP)
        return fail(SDE_ERR_UNSUPPORTED, "group size %d outside 1..%d", s->group_size, SDE_MAX_GROUP);
    if ((int64_t)s->groups * s->group_size >= (1 << 19))
        return fail(SDE_ERR_UNSUPPORTED, "too many state variables per path");
    if (s->jump_law < SDE_JUMP_NONE || s->jump_law > SDE_JUMP_EXP)
        return fail(SDE_ERR_UNSUPPORTED, "unknown jump law %d", s->jump_law);
    if (s->jump_law != SDE_JUMP_NONE && s->model != SDE_MODEL_LINEAR && s->model != SDE_MODEL_USER)
        return fail(SDE_ERR_UNSUPPORTED, "jumps are supported for the LINEAR model and user SDEs only");
    if (s->model == SDE_MODEL_HESTON) {
        const int M = s->group_size;
        if (M != 2 && M != 4 && M != 8 && M != 16)
            return fail(SDE_ERR_UNSUPPORTED, "Heston group size must be 2, 4, 8 or 16, not %d", M);
    }
    if (!s->x0 || !s->params) return fail(SDE_ERR_INVALID, "x0 and params are required");
    const int M = s->group_size;
    switch (s->out_mode) {
    case SDE_OUT_STATE:
    case SDE_OUT_EXP: *opg = M; break;
    case SDE_OUT_SUM: *opg = 1; break;
    case SDE_OUT_HESTON_X:
        if (s->model != SDE_MODEL_HESTON) return fail(SDE_ERR_INVALID, "HESTON_X output needs the HESTON model");
        *opg = M / 2;
        break;
    case SDE_OUT_HESTON_XY:
        if (s->model != SDE_MODEL_HESTON) return fail(SDE_ERR_INVALID, "HESTON_XY output needs the HESTON model");
        *opg = M;
        break;
    default: return fail(SDE_ERR_INVALID, "unknown out_mode %d", s->out_mode);
    }
    return SDE_OK;
}

static int check_grid(const SdeGrid *g, int n_rows) {
    if (!g || !g->tt || !g->out_row) return fail(SDE_ERR_INVALID, "grid arrays are required");
    if (g->n_pts < 1) return fail(SDE_ERR_INVALID, "grid needs at least one point");
    for (int k = 0; k < g->n_pts; ++k) {
        if (!std::isfinite(g->tt[k])) return fail(SDE_ERR_INVALID, "grid point %d is not finite", k);
        if (g->out_row[k] < -1 || g->out_row[k] >= n_rows)
            return fail(SDE_ERR_INVALID, "grid out_row[%d] = %d outside [-1, %d)", k, g->out_row[k], n_rows);
    }
    return SDE_OK;
}

static int maxm_of(int M) {
    if (M <= 1) return 1;
    if (M <= 2) return 2;
    if (M <= 4) return 4;
    if (M <= 8) return 8;
    return 16;
}

template <typename R> struct Finder;
template <> struct Finder<double> {
    static FwdLauncher<double> find(int model, int maxm, bool inj, bool jmp, int *bps) {
        if (model == SDE_MODEL_USER || model == SDE_MODEL_USER_SYS)
            return find_fwd_f64_user(maxm, inj, model == SDE_MODEL_USER_SYS, jmp, bps);
        if (model == SDE_MODEL_CIR) return jmp ? nullptr : find_fwd_f64_cir(maxm, inj, false, bps);
        FwdLauncher<double> f = find_fwd_f64_linear(model, maxm, inj, jmp, bps);
        return f ? f : find_fwd_f64_ou_heston(model, maxm, inj, jmp, bps);
    }
    static FwdLauncher<double> find_tdep(int, int, int *) { return nullptr; }
    static FwdLauncher<double> find_anti(int model, int maxm, bool jmp, bool, int *bps) {
        if (model == SDE_MODEL_CIR) return jmp ? nullptr : find_fwd_f64_cir(maxm, false, true, bps);
        return find_fwd_f64_anti(model, maxm, jmp, bps);
    }
};
template <> struct Finder<float> {
    static FwdLauncher<float> find(int model, int maxm, bool inj, bool jmp, int *bps) {
        if (model == SDE_MODEL_USER || model == SDE_MODEL_USER_SYS)
            return find_fwd_f32_user(maxm, inj, model == SDE_MODEL_USER_SYS, jmp, bps);
        if (model == SDE_MODEL_CIR) return jmp ? nullptr : find_fwd_f32_cir(maxm, inj, false, false, bps);
        FwdLauncher<float> f = find_fwd_f32_linear(model, maxm, inj, jmp, bps);
        return f ? f : find_fwd_f32_ou_heston(model, maxm, inj, jmp, bps);
    }
    // time-dependent coefficients: OU run tables with a time-dependent
    // theta, Heston and CIR with per-step reloads
    static FwdLauncher<float> find_tdep(int model, int maxm, int *bps) {
        if (model == SDE_MODEL_CIR) return find_fwd_f32_cir(maxm, false, true, false, bps);
        return find_fwd_f32_tdep(model, maxm, bps);
    }
    // tdep: the instantiations with per-step coefficients and correlation
    // factors (and OU rows with the theta term)
    static FwdLauncher<float> find_anti(int model, int maxm, bool jmp, bool tdep, int *bps) {
        if (model == SDE_MODEL_CIR) return jmp ? nullptr : find_fwd_f32_cir(maxm, false, tdep, true, bps);
        return tdep ? find_fwd_f32_anti_tdep(model, maxm, jmp, bps) : find_fwd_f32_anti(model, maxm, jmp, bps);
    }
};

// number of blocks along paths: enough for every SM, capped by the paths
static int path_blocks(Device *D, int64_t paths, int groups, int bps) {
    if (bps < 1) bps = 1;
    int64_t want = (paths + BLOCK - 1) / BLOCK;
    int64_t resident = (int64_t)D->sms * bps;
    int64_t per_group = (resident + groups - 1) / groups;
    if (per_group < 1) per_group = 1;
    int64_t nb = want < per_group ? want : per_group;
    if (nb < 1) nb = 1;
    return (int)nb;
}

// ---------------------------------------------------------------------------
// the run
// ---------------------------------------------------------------------------
template <typename R>
static int run_impl(const SdeSpec *s, const SdeGrid *gr, const SdeNoise *noise, SdeOut *out,
                    const SdeStatsReq *req, SdeStatsOut *so) {
    int opg = 0, rc;
    if ((rc = check_spec(s, &opg))) return rc;
    if (!out) return fail(SDE_ERR_INVALID, "out is NULL");
    if (out->n_rows < 1) return fail(SDE_ERR_INVALID, "out->n_rows must be >= 1");
    if ((rc = check_grid(gr, out->n_rows))) return rc;
    // a user program's jump terms: bit 0 dj, bit 1 dn
    int ujs = 0;
    if (s->model == SDE_MODEL_USER)
        for (int i = 0; i < s->program->n_terms; ++i) {
            if (s->program->term_source[i] == SDE_SRC_DJ) ujs |= 1;
            if (s->program->term_source[i] == SDE_SRC_DN) ujs |= 2;
        }
    const bool jumps = s->model == SDE_MODEL_USER ? ujs != 0 : s->jump_law != SDE_JUMP_NONE;
    if (gr->lam_t && !(s->model == SDE_MODEL_USER && jumps))
        return fail(SDE_ERR_INVALID, "grid lam_t applies to user SDEs with dn / dj terms");
    const bool inject = noise != nullptr;
    const bool anti = (s->flags & SDE_FLAG_ANTITHETIC) != 0;
    if (s->flags & ~SDE_FLAG_ANTITHETIC) return fail(SDE_ERR_INVALID, "unknown spec flags %d", s->flags);
    if (anti) {
        if (inject) return fail(SDE_ERR_INVALID, "antithetic paths are drawn on the device, not injected");
        if (s->paths % 2)
            return fail(SDE_ERR_INVALID, "the number of paths for sources with antithetics should be even, not %lld",
                        (long long)s->paths);
        if (s->group_size > 8) return fail(SDE_ERR_UNSUPPORTED, "antithetic paths take groups of up to 8 states");
    }
    if (inject) {
        // (a user SDE without a dw term has no Wiener source)
        bool user_dw = false;
        if (s->model == SDE_MODEL_USER)
            for (int i = 0; i < s->program->n_terms; ++i) user_dw |= s->program->term_source[i] == SDE_SRC_DW;
        if (!noise->dw && (s->model != SDE_MODEL_USER || user_dw))
            return fail(SDE_ERR_INVALID, "injected noise needs dw");
        if (s->model == SDE_MODEL_USER) {
            if ((ujs & 1) && !noise->dj) return fail(SDE_ERR_INVALID, "injected noise of a dj term needs dj");
            if ((ujs & 2) && !noise->dn) return fail(SDE_ERR_INVALID, "injected noise of a dn term needs dn");
        } else if (jumps && !noise->dj) {
            return fail(SDE_ERR_INVALID, "injected noise of a jump model needs dj");
        }
    }
    const bool stats = req != nullptr;
    if (stats) {
        if (!so || !so->moments) return fail(SDE_ERR_INVALID, "stats output arrays are required");
        if (req->row < 0 || req->row >= out->n_rows) return fail(SDE_ERR_INVALID, "stats row %d out of range", req->row);
        if (req->bins < 0) return fail(SDE_ERR_INVALID, "bins must be >= 0");
        if (req->bins > 0 && (!so->counts || !so->edges)) return fail(SDE_ERR_INVALID, "histogram arrays are required");
        if (req->n_strikes < 0 || req->n_strikes > SDE_MAX_STRIKES)
            return fail(SDE_ERR_INVALID, "n_strikes must be in 0..%d", SDE_MAX_STRIKES);
        if (req->n_strikes > 0 && !so->payoff) return fail(SDE_ERR_INVALID, "payoff array is required");
        if (req->has_range && !(std::isfinite(req->range_lo) && std::isfinite(req->range_hi) && req->range_lo <= req->range_hi))
            return fail(SDE_ERR_INVALID, "histogram range must be finite with min <= max");
    }
    const int M = s->group_size, W = s->groups * M;
    const int64_t paths = s->paths;
    const int n_steps = gr->n_pts - 1;
    const int64_t n_out = (int64_t)s->groups * opg;

    std::lock_guard<std::mutex> lk(g_mu);
    Device *D;
    if ((rc = current_device(&D))) return rc;
    cudaStream_t st = dev_stream(D);

    // ---- host tables, packed in one staging buffer ---------------------------
    // layout: dt[R n_steps] sqdt[R n_steps] out_row[int n_pts] x0[R W] prm[R 6W]
    //         lamdt[f64 n_steps*W] p0[f64 n_steps*W] thr[i64 n_steps*W] thr1[i64 n_steps*W]
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t o_dt = 0;
    const size_t o_sq = o_dt + al(sizeof(R) * (n_steps + 1));
    const size_t o_row = o_sq + al(sizeof(R) * (n_steps + 1));
    const size_t o_x0 = o_row + al(sizeof(int32_t) * gr->n_pts);
    const size_t o_prm = o_x0 + al(sizeof(R) * W);
    const size_t o_lam = o_prm + al(sizeof(R) * SDE_MAX_PARAMS * W);
    const size_t njt = jumps ? (size_t)n_steps * W + 1 : 1;
    const size_t o_p0 = o_lam + al(sizeof(double) * njt);
    const size_t o_thr = o_p0 + al(sizeof(double) * njt);
    const bool tab = sizeof(R) == 4 && !inject && (s->model == SDE_MODEL_LINEAR || s->model == SDE_MODEL_OU);
    const int tmaxm = maxm_of(M);
    // parameters of step k: the time-dependent table's row, or the constants
    const double *ptab = gr->params_t;
    auto params_of = [&](int k) -> const double * {
        return ptab ? ptab + (size_t)k * SDE_MAX_PARAMS * W : s->params;
    };
    // OU with a time-dependent theta: the state is held as the deviation from
    // the first step's theta0, and each row adds b = k dt (theta_k - theta0)
    bool ou_b = false;
    if (tab && ptab && s->model == SDE_MODEL_OU)
        for (int k = 0; k < n_steps && !ou_b; ++k)
            for (int w = 0; w < W && !ou_b; ++w) ou_b = params_of(k)[W + w] != params_of(0)[W + w];
    // time-dependent correlation (device noise): per-step Cholesky factors,
    // read by the kernels compiled with per-step reloads -- for FP32 the
    // time-dependent instantiations, whose OU form carries the b column
    const bool corr_steps = gr->corr_t != nullptr && !inject && M > 1;
    if (corr_steps && sizeof(R) == 4 && jumps && !anti)
        return fail(SDE_ERR_UNSUPPORTED, "time-dependent correlations of FP32 jump models");
    if (corr_steps && tab && s->model == SDE_MODEL_OU) ou_b = true;
    const int nb = ou_b ? 3 : 2;   // coefficient vectors per row
    // FP32 LINEAR / OU: the grid as runs of steps with one coefficient row
    // each, and the compact table of those rows (see FwdArgs::coef / runs)
    std::vector<int4> runs;
    std::vector<float> ctab, tshift;
    if (tab && n_steps > 0) {
        const size_t rowlen = (size_t)s->groups * nb * tmaxm;
        std::vector<float> cur(rowlen), nxt(rowlen);
        const int ps = s->model == SDE_MODEL_OU ? 2 : 1;   // the sigma slot
        const double *th0 = params_of(0) + W;
        // the same FP64 operations as coef_table_kernel
        auto coef_row = [&](int k, float *t) {
            const double dt = gr->tt[k + 1] - gr->tt[k], sq = sqrt(fabs(dt));
            const double *P = params_of(k);
            for (int g = 0; g < s->groups; ++g) {
                float *r = t + (size_t)g * nb * tmaxm;
                for (int m = 0; m < tmaxm; ++m) {
                    if (m >= M) {
                        for (int v = 0; v < nb; ++v) r[v * tmaxm + m] = 0.0f;
                        continue;
                    }
                    const int w = g * M + m;
                    const double cs = P[ps * W + w] * sq;
                    const double d = P[w] * dt;
                    r[m] = (float)d;
                    r[tmaxm + m] = (float)(cs * SDE_SQRT_2LN2);
                    if (ou_b) {
                        const double dth = P[W + w] - th0[w];
                        r[2 * tmaxm + m] = (float)(d * dth);
                    }
                }
            }
        };
        if (s->model == SDE_MODEL_OU) {
            tshift.assign((size_t)s->groups * 2 * tmaxm, 0.0f);
            for (int g = 0; g < s->groups; ++g)
                for (int m = 0; m < M; ++m) {
                    const int w = g * M + m;
                    tshift[(size_t)g * 2 * tmaxm + m] = (float)th0[w];
                    tshift[(size_t)(g * 2 + 1) * tmaxm + m] = (float)(s->x0[w] - th0[w]);
                }
        }
        int k = 0;
        while (k < n_steps) {
            coef_row(k, cur.data());
            const size_t nrows = ctab.size() / rowlen;
            int ci;
            if (nrows > 0 && memcmp(ctab.data() + (nrows - 1) * rowlen, cur.data(), rowlen * sizeof(float)) == 0) {
                ci = (int)nrows - 1;
            } else {
                ctab.insert(ctab.end(), cur.begin(), cur.end());
                ci = (int)nrows;
            }
            const int k0 = k;
            int row = -1;
            for (;;) {
                ++k;
                if (gr->out_row[k] >= 0) { row = gr->out_row[k]; break; }
                if (k == n_steps) break;
                coef_row(k, nxt.data());
                if (memcmp(nxt.data(), cur.data(), rowlen * sizeof(float)) != 0) break;
            }
            runs.push_back(make_int4(k0, k, row, ci));
        }
    } else if (n_steps > 0) {
        // the other kernels: runs of steps with one dt (and sqrt|dt|),
        // ending where a row is stored, split where an adjoint checkpoint
        // falls (bit 0 of w: a checkpoint before the run's first step)
        const int cseg = (out->ckpt && out->ckpt_seg > 0) ? out->ckpt_seg : 0;
        auto dts = [&](int k, R *d, R *q) {
            const double dt = gr->tt[k + 1] - gr->tt[k];
            *d = (R)dt;
            *q = (R)sqrt(fabs(dt));
        };
        int k = 0;
        while (k < n_steps) {
            const int k0 = k;
            R d0, q0, d1, q1;
            dts(k, &d0, &q0);
            int row = -1;
            for (;;) {
                ++k;
                if (gr->out_row[k] >= 0) { row = gr->out_row[k]; break; }
                if (k == n_steps || (cseg && k % cseg == 0)) break;
                dts(k, &d1, &q1);
                if (memcmp(&d1, &d0, sizeof(R)) != 0 || memcmp(&q1, &q0, sizeof(R)) != 0) break;
            }
            runs.push_back(make_int4(k0, k, row, (cseg && k0 % cseg == 0) ? 1 : 0));
        }
    }
    const size_t o_thr1 = o_thr + al(sizeof(long long) * njt);
    const size_t o_runs = o_thr1 + al(sizeof(long long) * njt);
    const size_t o_ctab = o_runs + al(sizeof(int4) * (runs.size() + 1));
    const size_t o_tsh = o_ctab + al(sizeof(float) * (ctab.size() + 4));
    // the other kernels read time-dependent coefficients (slots 0..2) per step
    const bool user = s->model == SDE_MODEL_USER;
    const int npt = user ? SDE_MAX_PARAMS : 3;   // parameter slots per table row
    const size_t nprmt = (ptab && !tab) ? (size_t)n_steps * npt * W : 0;
    const size_t o_prmt = o_tsh + al(sizeof(float) * (tshift.size() + 4));
    const size_t nchol = corr_steps ? (size_t)n_steps * NCHOL : 0;
    const size_t o_cholt = o_prmt + al(sizeof(R) * (nprmt + 1));
    const size_t ntk = user ? (size_t)n_steps : 0;   // step starts, for user SDEs
    const size_t o_tk = o_cholt + al(sizeof(R) * (nchol + 1));
    const size_t njp = (user && jumps) ? (size_t)3 * W : 0;   // a user dj term's law: a, b, pa
    const size_t o_jp = o_tk + al(sizeof(R) * (ntk + 1));
    const size_t o_end = o_jp + al(sizeof(R) * (njp + 1));
    D->host_tables.resize(o_end);
    char *H = D->host_tables.data();
    R *h_dt = (R *)(H + o_dt), *h_sq = (R *)(H + o_sq), *h_x0 = (R *)(H + o_x0), *h_prm = (R *)(H + o_prm);
    int32_t *h_row = (int32_t *)(H + o_row);
    double *h_lam = (double *)(H + o_lam), *h_p0 = (double *)(H + o_p0);
    long long *h_thr = (long long *)(H + o_thr), *h_thr1 = (long long *)(H + o_thr1);
    double sgn = 1.0;
    for (int k = 0; k < n_steps; ++k) {
        const double dt = gr->tt[k + 1] - gr->tt[k];
        if (k == 0) sgn = dt < 0 ? -1.0 : 1.0;
        if ((dt < 0 ? -1.0 : 1.0) != sgn || dt == 0.0)
            return fail(SDE_ERR_INVALID, "grid points must be strictly monotonic (step %d)", k);
        h_dt[k] = (R)dt;
        h_sq[k] = (R)sqrt(fabs(dt));
    }
    memcpy(h_row, gr->out_row, sizeof(int32_t) * gr->n_pts);
    for (int w = 0; w < W; ++w) h_x0[w] = (R)s->x0[w];
    for (int i = 0; i < SDE_MAX_PARAMS * W; ++i) h_prm[i] = (R)s->params[i];
    if (jumps && !inject) {
        for (int k = 0; k < n_steps; ++k) {
            const double adt = fabs(gr->tt[k + 1] - gr->tt[k]);
            for (int w = 0; w < W; ++w) {
                // a user SDE's intensity: its table at the step's midpoint, or its constant
                const double lam = !user          ? params_of(k)[2 * W + w]
                                   : gr->lam_t ? gr->lam_t[(size_t)k * W + w]
                                               : s->program->jump_params[w];
                if (!(lam >= 0.0) || !std::isfinite(lam))
                    return fail(SDE_ERR_INVALID, "Poisson intensity must be finite and >= 0");
                const double L = adt * lam;
                if (L > 700.0) return fail(SDE_ERR_UNSUPPORTED, "lam*dt = %g too large for inversion sampling", L);
                const double p0 = exp(-L);
                const size_t i = (size_t)k * W + w;
                h_lam[i] = L;
                h_p0[i] = p0;
                poisson_thresholds(p0, L, h_thr[i], h_thr1[i]);
            }
        }
        // the jump-size law's a, b, pa: parameter slots 3..5, or a user
        // program's jump_params rows 1..3
        const double *law = user ? s->program->jump_params + W : s->params + 3 * W;
        if (s->jump_law == SDE_JUMP_DOUBLE_EXP)
            for (int w = 0; w < W; ++w) {
                const double a = law[w], b = law[W + w], pa = law[2 * W + w];
                if (!(a > 0) || !(b > 0) || !(pa >= 0 && pa <= 1))
                    return fail(SDE_ERR_INVALID, "domain error in arguments");
            }
    }
    if (njp) {
        R *h_jp = (R *)(H + o_jp);
        for (size_t i = 0; i < njp; ++i) h_jp[i] = (R)s->program->jump_params[W + i];
    }

    if (!runs.empty()) memcpy(H + o_runs, runs.data(), sizeof(int4) * runs.size());
    if (!ctab.empty()) memcpy(H + o_ctab, ctab.data(), sizeof(float) * ctab.size());
    if (!tshift.empty()) memcpy(H + o_tsh, tshift.data(), sizeof(float) * tshift.size());
    if (nprmt) {
        R *h_prmt = (R *)(H + o_prmt);
        for (int k = 0; k < n_steps; ++k)
            for (int v = 0; v < npt; ++v)
                for (int w = 0; w < W; ++w) h_prmt[((size_t)k * npt + v) * W + w] = (R)params_of(k)[v * W + w];
    }
    if (ntk) {
        R *h_tk = (R *)(H + o_tk);
        for (int k = 0; k < n_steps; ++k) h_tk[k] = (R)gr->tt[k];
    }
    if (nchol) {
        R *h_cholt = (R *)(H + o_cholt);
        std::vector<double> L(M * M);
        for (int k = 0; k < n_steps; ++k) {
            if ((rc = sde_cholesky(gr->corr_t + (size_t)k * M * M, M, L.data()))) {
                char m[256];
                snprintf(m, sizeof m, "correlation of step %d: %s", k, g_err.c_str());
                return fail(rc, "%s", m);
            }
            R *row = h_cholt + (size_t)k * NCHOL;
            for (int i = 0; i < NCHOL; ++i) row[i] = R(0);
            for (int i = 0; i < M; ++i)
                for (int j = 0; j <= i; ++j) row[i * (i + 1) / 2 + j] = (R)L[i * M + j];
        }
    }

    FwdArgs<R> a;
    memset(&a, 0, sizeof a);
    if (s->corr) {
        std::vector<double> L(M * M);
        if ((rc = sde_cholesky(s->corr, M, L.data()))) return rc;
        for (int i = 0; i < M; ++i)
            for (int j = 0; j <= i; ++j) a.chol[i * (i + 1) / 2 + j] = (R)L[i * M + j];
        a.has_corr = 1;
    }

    void *d_tab;
    if ((rc = scratch(D, S_TABLES, o_end, &d_tab))) return rc;
    CU(cudaMemcpyAsync(d_tab, H, o_end, cudaMemcpyHostToDevice, st));
    char *T = (char *)d_tab;

    a.paths = paths;
    a.groups = s->groups;
    a.M = M;
    a.W = W;
    a.n_pts = gr->n_pts;
    a.step_offset = gr->step_offset;
    a.jump_law = s->jump_law;
    a.out_mode = s->out_mode;
    a.opg = opg;
    a.seed = s->seed;
    a.stream = s->stream;
    a.path_offset = s->path_offset;
    a.tab_row0 = gr->out_row[0];
    a.sgn = (R)sgn;
    a.dt = (const R *)(T + o_dt);
    a.sqdt = (const R *)(T + o_sq);
    a.out_row = (const int32_t *)(T + o_row);
    a.lamdt = (const double *)(T + o_lam);
    a.p0 = (const double *)(T + o_p0);
    a.thr = (const long long *)(T + o_thr);
    a.thr1 = (const long long *)(T + o_thr1);
    a.x0 = (const R *)(T + o_x0);
    a.prm = (const R *)(T + o_prm);
    a.coef = nullptr;
    a.runs = nullptr;
    if (tab && n_steps > 0) {
        a.coef = (const float *)(T + o_ctab);
        a.runs = (const int4 *)(T + o_runs);
        a.n_runs = (int32_t)runs.size();
        a.tshift = tshift.empty() ? nullptr : (const float *)(T + o_tsh);
    } else if (!runs.empty()) {   // the other kernels' runs of one dt
        a.runs = (const int4 *)(T + o_runs);
        a.n_runs = (int32_t)runs.size();
    }
    a.prm_t = nprmt ? (const R *)(T + o_prmt) : nullptr;
    a.chol_t = nchol ? (const R *)(T + o_cholt) : nullptr;
    if (nchol) a.has_corr = 1;
    a.tk = ntk ? (const R *)(T + o_tk) : nullptr;
    if (user) a.uprog = *s->program;
    a.jprm = njp ? (const R *)(T + o_jp) : nullptr;
    a.user_jsrc = ujs;
    a.key = philox_schedule(s->seed);
    a.n_out_vars = n_out;

    // ---- injected noise ---------------------------------------------------------
    const size_t nz = (size_t)n_steps * W * paths;
    if (inject && n_steps > 0) {
        void *p;
        if (noise->dw) {
            if ((rc = scratch(D, S_NOISE_DW, nz * sizeof(double), &p))) return rc;
            CU(cudaMemcpyAsync(p, noise->dw, nz * sizeof(double), cudaMemcpyHostToDevice, st));
            a.dw = (const double *)p;
        }
        // (a user SDE's dj and dn are its two sources, each when its term is there)
        if (jumps && (!user || (ujs & 1))) {
            if ((rc = scratch(D, S_NOISE_DJ, nz * sizeof(double), &p))) return rc;
            CU(cudaMemcpyAsync(p, noise->dj, nz * sizeof(double), cudaMemcpyHostToDevice, st));
            a.dj = (const double *)p;
        }
        if (jumps && (!user || (ujs & 2))) {
            if (noise->dn) {
                if ((rc = scratch(D, S_NOISE_DN, nz * sizeof(int64_t), &p))) return rc;
                CU(cudaMemcpyAsync(p, noise->dn, nz * sizeof(int64_t), cudaMemcpyHostToDevice, st));
                a.dn = (const long long *)p;
            }
        }
    }

    // ---- outputs -------------------------------------------------------------------
    const bool dev = out->on_device != 0;
    const size_t xx_bytes = (size_t)out->n_rows * n_out * paths * sizeof(R);
    int rmin = out->n_rows, rmax = -1;
    for (int k = 0; k < gr->n_pts; ++k)
        if (gr->out_row[k] >= 0) {
            rmin = gr->out_row[k] < rmin ? gr->out_row[k] : rmin;
            rmax = gr->out_row[k] > rmax ? gr->out_row[k] : rmax;
        }
    // host output in pinned (page-locked) memory: the kernel stores its rows
    // straight into it, with no device buffer and no separate copy
    bool xx_mapped = false;
    if (out->xx) {
        if (dev) {
            a.xx = (R *)out->xx;
        } else {
            cudaPointerAttributes pa;
            if (cudaPointerGetAttributes(&pa, out->xx) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
                pa.devicePointer != nullptr) {
                a.xx = (R *)pa.devicePointer;
                xx_mapped = true;
            } else {
                cudaGetLastError();
                void *p;
                if ((rc = scratch(D, S_XX, xx_bytes, &p))) return rc;
                a.xx = (R *)p;
            }
        }
    }
    const int h = M / 2;
    const size_t neg_n = (size_t)s->groups * h * paths, jc_n = (size_t)W * paths;
    if (out->neg_count && s->model == SDE_MODEL_HESTON) {
        if (dev) a.neg_count = out->neg_count;
        else {
            void *p;
            if ((rc = scratch(D, S_NEG, neg_n * sizeof(int32_t), &p))) return rc;
            a.neg_count = (int32_t *)p;
        }
    }
    if (jumps && !user && out->jump_count) {
        if (dev) a.jump_count = out->jump_count;
        else {
            void *p;
            if ((rc = scratch(D, S_JCNT, jc_n * sizeof(int32_t), &p))) return rc;
            a.jump_count = (int32_t *)p;
        }
    }
    if (jumps && !user && out->row_jumps) {
        if (dev) a.row_jumps = (unsigned long long *)out->row_jumps;
        else {
            void *p;
            if ((rc = scratch(D, S_ROWJ, sizeof(int64_t) * out->n_rows, &p))) return rc;
            a.row_jumps = (unsigned long long *)p;
        }
        CU(cudaMemsetAsync(a.row_jumps, 0, sizeof(int64_t) * out->n_rows, st));
    }
    // adjoint checkpoints (device memory of the caller)
    if (out->ckpt && n_steps > 0) {
        if (out->ckpt_seg < 1) return fail(SDE_ERR_INVALID, "ckpt_seg must be >= 1");
        if (inject || anti)
            return fail(SDE_ERR_UNSUPPORTED, "checkpoints are written for device-RNG paths without antithetics");
        // (the FP32 OU run-table kernel writes them for the state output with
        // constant parameters and correlation)
        const bool tab_ck = s->model == SDE_MODEL_OU && s->out_mode == SDE_OUT_STATE && !gr->params_t &&
                            !gr->corr_t && M <= 8;
        if (tab && !tab_ck)
            return fail(SDE_ERR_UNSUPPORTED, "the FP32 LINEAR run-table kernels, and the OU one with a time-dependent "
                                             "coefficient or correlation or another output, write no checkpoints");
        a.ckpt = (R *)out->ckpt;
        a.ckpt_seg = out->ckpt_seg;
    }
    void *d_err;
    if ((rc = scratch(D, S_ERR, 16, &d_err))) return rc;
    CU(cudaMemsetAsync(d_err, 0, 16, st));
    a.err = (int32_t *)d_err;

    // ---- launch ----------------------------------------------------------------------
    int bps = 0;
    // the FP32 Heston and CIR kernels of device noise read per-step
    // coefficients only in their time-dependent instantiation
    const bool tdep_k = ou_b || (sizeof(R) == 4 && !inject &&
                                 ((nprmt && (s->model == SDE_MODEL_HESTON || s->model == SDE_MODEL_CIR)) ||
                                  corr_steps));
    // (user-SDE kernels reload per-step parameters and factors in every form)
    const int kmodel = user && s->program->n_eq > 1 ? SDE_MODEL_USER_SYS : s->model;
    // a user program compiled at run time, or an instantiated kernel
    cudaKernel_t jk = nullptr;
    FwdLauncher<R> L = nullptr;
    if (user && s->program->jit) {
        std::string err;
        if ((rc = jit_fwd_kernel(*s->program, sizeof(R) == 8, maxm_of(M), inject, jumps, &jk, &bps, &err)))
            return fail(rc, "%s", err.c_str());
    } else {
        L = user     ? Finder<R>::find(kmodel, maxm_of(M), inject, jumps, &bps)
            : anti   ? Finder<R>::find_anti(s->model, maxm_of(M), jumps, tdep_k, &bps)
            : tdep_k ? Finder<R>::find_tdep(s->model, maxm_of(M), &bps)
                     : Finder<R>::find(s->model, maxm_of(M), inject, jumps, &bps);
        if (!L) return fail(SDE_ERR_UNSUPPORTED, "no kernel for model %d group size %d", s->model, M);
    }
    // antithetic kernels integrate two paths per thread
    const int nbx = path_blocks(D, anti ? paths / 2 : paths, s->groups, bps);
    a.stats_row = -1;
    const int bins = stats ? req->bins : 0;
    if (stats) {
        a.stats_row = req->row;
        a.n_strikes = req->n_strikes;
        for (int i = 0; i < req->n_strikes; ++i) a.strikes[i] = (R)req->strikes[i];
        void *p;
        if ((rc = scratch(D, S_PART, sizeof(double) * NPART * (size_t)s->groups * nbx * opg, &p))) return rc;
        a.partials = (double *)p;
        // the histogram pass, and the summary of the kernels that reduce the
        // stored row in a second launch, read device memory: a private copy
        // of the row when the paths go only to host memory
        const bool row_pass = fwd_summary_from_row(sizeof(R) == 4, s->model, inject, jumps, anti, tdep_k, user);
        if ((bins > 0 || row_pass) && (!a.xx || xx_mapped)) {
            if ((rc = scratch(D, S_VALS, sizeof(R) * n_out * paths, &p))) return rc;
            a.stats_vals = (R *)p;
        }
    }
    if (D->timing) CU(cudaEventRecord(D->ev[0], st));
    if (jk) {
        void *args[] = {(void *)&a};
        CU(cudaLaunchKernel((const void *)jk, dim3(nbx, s->groups), dim3(BLOCK), args, 0, st));
    } else {
        L(a, dim3(nbx, s->groups), st);
    }
    CU(cudaGetLastError());
    if (D->timing) CU(cudaEventRecord(D->ev[1], st));

    // ---- fused statistics --------------------------------------------------------------
    if (stats) {
        void *res, *edges, *edges64, *counts;
        if ((rc = scratch(D, S_RES, sizeof(double) * RES_STRIDE * n_out, &res))) return rc;
        if ((rc = scratch(D, S_EDGES, sizeof(R) * (bins + 1) * n_out, &edges))) return rc;
        if ((rc = scratch(D, S_EDGES64, sizeof(double) * (bins + 1) * n_out, &edges64))) return rc;
        stats_finalize_kernel<R><<<(unsigned)n_out, BLOCK, 0, st>>>(
            a.partials, nbx, opg, req->n_strikes, bins, req->has_range, req->range_lo, req->range_hi,
            (double *)res, (R *)edges, (double *)edges64, a.err);
        CU(cudaGetLastError());
        if (bins > 0) {
            if ((rc = scratch(D, S_COUNTS, sizeof(int64_t) * bins * n_out, &counts))) return rc;
            CU(cudaMemsetAsync(counts, 0, sizeof(int64_t) * bins * n_out, st));
            const R *vals;
            int64_t vstride;
            if (a.xx && !xx_mapped) {
                vals = a.xx + (int64_t)req->row * n_out * paths;
                vstride = paths;
            } else {
                vals = a.stats_vals;
                vstride = paths;
            }
            int hb = (int)((paths + BLOCK * 16 - 1) / (BLOCK * 16));
            if (hb > 4 * D->sms) hb = 4 * D->sms;
            if (hb < 1) hb = 1;
            const size_t smem = bins <= HIST_SMEM_BINS ? sizeof(unsigned) * bins : 0;
            hist_kernel<R><<<dim3(hb, (unsigned)n_out), BLOCK, smem, st>>>(
                vals, vstride, paths, bins, (const R *)edges, (const double *)res, req->has_range,
                (unsigned long long *)counts);
            CU(cudaGetLastError());
        }
        if (D->timing) CU(cudaEventRecord(D->ev[2], st));
        std::vector<double> hres(RES_STRIDE * n_out);
        CU(cudaMemcpyAsync(hres.data(), res, sizeof(double) * RES_STRIDE * n_out, cudaMemcpyDeviceToHost, st));
        if (bins > 0) {
            CU(cudaMemcpyAsync(so->counts, counts, sizeof(int64_t) * bins * n_out, cudaMemcpyDeviceToHost, st));
            CU(cudaMemcpyAsync(so->edges, edges64, sizeof(double) * (bins + 1) * n_out, cudaMemcpyDeviceToHost, st));
        }
        CU(cudaStreamSynchronize(st));
        for (int64_t o = 0; o < n_out; ++o) {
            for (int i = 0; i < 7; ++i) so->moments[o * 8 + i] = hres[o * RES_STRIDE + i];
            so->moments[o * 8 + 7] = 0.0;
            for (int k = 0; k < req->n_strikes; ++k)
                so->payoff[o * req->n_strikes + k] = hres[o * RES_STRIDE + 9 + k];
        }
    }

    // ---- copies back ----------------------------------------------------------------------
    if (!dev) {
        if (out->xx && !xx_mapped && rmax >= rmin) {
            const size_t row_bytes = (size_t)n_out * paths * sizeof(R);
            CU(cudaMemcpyAsync((char *)out->xx + rmin * row_bytes, (char *)a.xx + rmin * row_bytes,
                               (size_t)(rmax - rmin + 1) * row_bytes, cudaMemcpyDeviceToHost, st));
        }
        if (a.neg_count) CU(cudaMemcpyAsync(out->neg_count, a.neg_count, neg_n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        if (a.jump_count) CU(cudaMemcpyAsync(out->jump_count, a.jump_count, jc_n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        if (a.row_jumps) CU(cudaMemcpyAsync(out->row_jumps, a.row_jumps, sizeof(int64_t) * out->n_rows, cudaMemcpyDeviceToHost, st));
    }
    int32_t herr = 0;
    CU(cudaMemcpyAsync(&herr, d_err, sizeof herr, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (D->timing) {
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, D->ev[0], D->ev[1]));
        D->last_ms[0] = ms;
        D->last_ms[1] = 0.0;
        if (stats) {
            CU(cudaEventElapsedTime(&ms, D->ev[1], D->ev[2]));
            D->last_ms[1] = ms;
        }
        D->last_ms[2] = (double)nbx;
        D->last_ms[3] = (double)(stats ? (bins > 0 ? 3 : 2) : 1);
    }
    if (herr & ERRF_JUMP_CAP) return fail(SDE_ERR_DEVICE, "more than %d jumps in one step", SDE_MAX_JUMPS_PER_STEP);
    if (herr & ERRF_RANGE) return fail(SDE_ERR_INVALID, "autodetected range of the histogram is not finite");
    if (herr & ERRF_ARGS) return fail(SDE_ERR_DEVICE, "kernel launched without its coefficient table");
    return SDE_OK;
}

extern "C" int32_t sde_run(const SdeSpec *spec, const SdeGrid *grid, const SdeNoise *noise, SdeOut *out) {
    if (!spec) return fail(SDE_ERR_INVALID, "spec is NULL");
    if (spec->precision == SDE_FP32) return run_impl<float>(spec, grid, noise, out, nullptr, nullptr);
    return run_impl<double>(spec, grid, noise, out, nullptr, nullptr);
}

extern "C" int32_t sde_run_stats(const SdeSpec *spec, const SdeGrid *grid, const SdeNoise *noise, SdeOut *out,
                                 const SdeStatsReq *req, SdeStatsOut *stats) {
    if (!spec) return fail(SDE_ERR_INVALID, "spec is NULL");
    if (!req) return fail(SDE_ERR_INVALID, "stats request is NULL");
    if (spec->precision == SDE_FP32) return run_impl<float>(spec, grid, noise, out, req, stats);
    return run_impl<double>(spec, grid, noise, out, req, stats);
}

// ---------------------------------------------------------------------------
// summaries of an existing sample
// ---------------------------------------------------------------------------
template <typename R>
static int sample_stats_impl(const void *sample, int on_device, int64_t n_vars, int64_t paths,
                             const SdeStatsReq *req, SdeStatsOut *so) {
    int rc;
    if (!sample || !req || !so || !so->moments) return fail(SDE_ERR_INVALID, "NULL argument");
    if (n_vars < 1 || paths < 1 || n_vars > 65535) return fail(SDE_ERR_INVALID, "bad sample shape");
    const int bins = req->bins;
    if (bins < 0) return fail(SDE_ERR_INVALID, "bins must be >= 0");
    if (bins > 0 && (!so->counts || !so->edges)) return fail(SDE_ERR_INVALID, "histogram arrays are required");
    std::lock_guard<std::mutex> lk(g_mu);
    Device *D;
    if ((rc = current_device(&D))) return rc;
    cudaStream_t st = dev_stream(D);
    const R *vals;
    if (on_device) {
        vals = (const R *)sample;
    } else {
        void *p;
        if ((rc = scratch(D, S_SAMPLE, sizeof(R) * n_vars * paths, &p))) return rc;
        CU(cudaMemcpyAsync(p, sample, sizeof(R) * n_vars * paths, cudaMemcpyHostToDevice, st));
        vals = (const R *)p;
    }
    int bps = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, sample_partials_kernel<R>, BLOCK, 0);
    const int nbx = path_blocks(D, paths, (int)n_vars, bps);
    void *part, *res, *edges, *edges64, *counts, *d_err;
    if ((rc = scratch(D, S_PART, sizeof(double) * NPART * n_vars * nbx, &part))) return rc;
    if ((rc = scratch(D, S_RES, sizeof(double) * RES_STRIDE * n_vars, &res))) return rc;
    if ((rc = scratch(D, S_EDGES, sizeof(R) * (bins + 1) * n_vars, &edges))) return rc;
    if ((rc = scratch(D, S_EDGES64, sizeof(double) * (bins + 1) * n_vars, &edges64))) return rc;
    if ((rc = scratch(D, S_ERR, 16, &d_err))) return rc;
    CU(cudaMemsetAsync(d_err, 0, 16, st));
    sample_partials_kernel<R><<<dim3(nbx, (unsigned)n_vars), BLOCK, 0, st>>>(vals, paths, (double *)part, nullptr);
    CU(cudaGetLastError());
    stats_finalize_kernel<R><<<(unsigned)n_vars, BLOCK, 0, st>>>(
        (const double *)part, nbx, 1, 0, bins, req->has_range, req->range_lo, req->range_hi,
        (double *)res, (R *)edges, (double *)edges64, (int32_t *)d_err);
    CU(cudaGetLastError());
    if (bins > 0) {
        if ((rc = scratch(D, S_COUNTS, sizeof(int64_t) * bins * n_vars, &counts))) return rc;
        CU(cudaMemsetAsync(counts, 0, sizeof(int64_t) * bins * n_vars, st));
        int hb = (int)((paths + BLOCK * 16 - 1) / (BLOCK * 16));
        if (hb > 4 * D->sms) hb = 4 * D->sms;
        if (hb < 1) hb = 1;
        const size_t smem = bins <= HIST_SMEM_BINS ? sizeof(unsigned) * bins : 0;
        hist_kernel<R><<<dim3(hb, (unsigned)n_vars), BLOCK, smem, st>>>(
            vals, paths, paths, bins, (const R *)edges, (const double *)res, req->has_range,
            (unsigned long long *)counts);
        CU(cudaGetLastError());
        CU(cudaMemcpyAsync(so->counts, counts, sizeof(int64_t) * bins * n_vars, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(so->edges, edges64, sizeof(double) * (bins + 1) * n_vars, cudaMemcpyDeviceToHost, st));
    }
    std::vector<double> hres(RES_STRIDE * n_vars);
    int32_t herr = 0;
    CU(cudaMemcpyAsync(hres.data(), res, sizeof(double) * RES_STRIDE * n_vars, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&herr, d_err, sizeof herr, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (herr & ERRF_RANGE) return fail(SDE_ERR_INVALID, "autodetected range of the histogram is not finite");
    for (int64_t o = 0; o < n_vars; ++o) {
        for (int i = 0; i < 7; ++i) so->moments[o * 8 + i] = hres[o * RES_STRIDE + i];
        so->moments[o * 8 + 7] = 0.0;
    }
    return SDE_OK;
}

extern "C" int32_t sde_sample_stats(const void *sample, int32_t is_fp32, int32_t on_device, int64_t n_vars,
                                    int64_t paths, const SdeStatsReq *req, SdeStatsOut *stats) {
    if (is_fp32) return sample_stats_impl<float>(sample, on_device, n_vars, paths, req, stats);
    return sample_stats_impl<double>(sample, on_device, n_vars, paths, req, stats);
}

template <typename R>
static int sample_hist_impl(const void *sample, int on_device, int64_t n_vars, int64_t paths, int bins,
                            const double *edges_in, int64_t *counts_out) {
    int rc;
    if (!sample || !edges_in || !counts_out || bins < 1 || n_vars < 1 || paths < 0 || n_vars > 65535)
        return fail(SDE_ERR_INVALID, "bad histogram arguments");
    for (int64_t o = 0; o < n_vars; ++o)
        for (int i = 0; i < bins; ++i)
            if (!(edges_in[o * (bins + 1) + i] <= edges_in[o * (bins + 1) + i + 1]))
                return fail(SDE_ERR_INVALID, "`bins` must increase monotonically, when an array");
    std::lock_guard<std::mutex> lk(g_mu);
    Device *D;
    if ((rc = current_device(&D))) return rc;
    cudaStream_t st = dev_stream(D);
    if (paths == 0) {
        memset(counts_out, 0, sizeof(int64_t) * bins * n_vars);
        return SDE_OK;
    }
    const R *vals;
    if (on_device) {
        vals = (const R *)sample;
    } else {
        void *p;
        if ((rc = scratch(D, S_SAMPLE, sizeof(R) * n_vars * paths, &p))) return rc;
        CU(cudaMemcpyAsync(p, sample, sizeof(R) * n_vars * paths, cudaMemcpyHostToDevice, st));
        vals = (const R *)p;
    }
    // explicit edges: general (non-uniform) bins by binary search, numpy's
    // searchsorted rule: right-closed last bin
    std::vector<R> he((bins + 1) * n_vars);
    std::vector<double> hres(RES_STRIDE * n_vars, 0.0);
    for (size_t i = 0; i < he.size(); ++i) he[i] = (R)edges_in[i];
    void *edges, *res, *counts;
    if ((rc = scratch(D, S_EDGES, sizeof(R) * he.size(), &edges))) return rc;
    if ((rc = scratch(D, S_RES, sizeof(double) * hres.size(), &res))) return rc;
    if ((rc = scratch(D, S_COUNTS, sizeof(int64_t) * bins * n_vars, &counts))) return rc;
    CU(cudaMemcpyAsync(edges, he.data(), sizeof(R) * he.size(), cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(res, 0, sizeof(double) * hres.size(), st));
    CU(cudaMemsetAsync(counts, 0, sizeof(int64_t) * bins * n_vars, st));
    int hb = (int)((paths + BLOCK * 16 - 1) / (BLOCK * 16));
    if (hb > 4 * D->sms) hb = 4 * D->sms;
    if (hb < 1) hb = 1;
    const size_t smem = bins <= HIST_SMEM_BINS ? sizeof(unsigned) * bins : 0;
    hist_edges_kernel<R><<<dim3(hb, (unsigned)n_vars), BLOCK, smem, st>>>(
        vals, paths, paths, bins, (const R *)edges, (unsigned long long *)counts);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(counts_out, counts, sizeof(int64_t) * bins * n_vars, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return SDE_OK;
}

extern "C" int32_t sde_sample_histogram(const void *sample, int32_t is_fp32, int32_t on_device, int64_t n_vars,
                                        int64_t paths, int32_t bins, const double *edges, int64_t *counts) {
    if (is_fp32) return sample_hist_impl<float>(sample, on_device, n_vars, paths, bins, edges, counts);
    return sample_hist_impl<double>(sample, on_device, n_vars, paths, bins, edges, counts);
}

// ---------------------------------------------------------------------------
// adjoint
// ---------------------------------------------------------------------------
// fixed-order FP64 tree over blocks: out[i] = sum_b part[b*stride + i]
__global__ void __launch_bounds__(BLOCK) reduce_partials_kernel(const double *part, int nb, int stride,
                                                                 double *out) {
    __shared__ double sh[BLOCK];
    const int i = blockIdx.x;
    double v = 0.0;
    for (int b = threadIdx.x; b < nb; b += BLOCK) v += part[(int64_t)b * stride + i];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = BLOCK / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[i] = sh[0];
}

template <typename R> struct AdjFinder;
template <> struct AdjFinder<float> {
    static AdjLauncher<float> find(int model, int maxm, bool jumps, int *bps) {
        if (model == SDE_MODEL_USER) return jumps ? nullptr : find_adj_user_f32(maxm, bps);
        return find_adj_f32(model, maxm, jumps, bps);
    }
    static AdjLauncher<float> find_td(int model, int maxm, int *bps) { return find_adj_td_f32(model, maxm, bps); }
    static AdjLauncher<float> find_heston(int seg, int *bps) { return find_adj_heston_f32(seg, bps); }
    static AdjLauncher<float> find_ou(int seg, int *bps) { return find_adj_ou_f32(seg, bps); }
};
template <> struct AdjFinder<double> {
    static AdjLauncher<double> find(int model, int maxm, bool jumps, int *bps) {
        if (model == SDE_MODEL_USER) return jumps ? nullptr : find_adj_user_f64(maxm, bps);
        return find_adj_f64(model, maxm, jumps, bps);
    }
    static AdjLauncher<double> find_td(int model, int maxm, int *bps) { return find_adj_td_f64(model, maxm, bps); }
    static AdjLauncher<double> find_heston(int, int *) { return nullptr; }
    static AdjLauncher<double> find_ou(int, int *) { return nullptr; }
};

// what the adjoint of a spec runs: a user program's terms (ujs bit 0 dj,
// bit 1 dn; nv the values per state and step the compiled kernel keeps:
// the state, dw, dn, dj); compiled programs, systems and jump terms take
// the reverse-mode kernel (sde_adj_user.cuh), the interpreter single
// equations driven by dt / dw (tangent mode)
struct AdjKind {
    bool user, ujit, jumps;
    int ujs, nv;
};

static AdjKind adjoint_kind(const SdeSpec *s) {
    AdjKind K;
    K.user = s->model == SDE_MODEL_USER;
    K.ujs = 0;
    K.nv = 1;
    if (K.user)
        for (int i = 0; i < s->program->n_terms; ++i) {
            const int src = s->program->term_source[i];
            if (src == SDE_SRC_DJ) K.ujs |= 1;
            if (src == SDE_SRC_DN) K.ujs |= 2;
            if (src != SDE_SRC_DT) ++K.nv;
        }
    K.ujit = K.user && (s->program->jit || s->program->n_eq > 1 || K.ujs);
    K.jumps = K.user ? K.ujs != 0 : s->jump_law != SDE_JUMP_NONE;
    return K;
}

// The adjoint's segments: level-1 checkpoints every `seg` steps (nseg of
// them), level 2 every `seg2` steps inside a level-1 segment (seg2 == seg:
// one level); the kernel's per-segment buffer holds at most `cap` steps.
// Without checkpoints from the forward, level 1 is ceil(sqrt(steps)) steps
// (capped), and runs needing more than ADJ_MAXSEG level-1 segments (the
// kernels' local checkpoint arrays) take level 1 every ceil(steps /
// ADJ_MAXSEG) steps and a second level inside, one more forward sweep.
// With checkpoints from the forward (read from device memory: any number),
// level 1 is their segment, split in two levels when longer than cap.
struct AdjPlan {
    bool heston_fast;   // the FP32 2-variable Heston kernel (sde_adj_heston.cuh)
    bool ou_fast;       // the scalar FP32 OU kernel (sde_adj_ou.cuh)
    int cap, seg, seg2, nseg;
    size_t ubytes;      // the compiled user-SDE kernel's shared-memory buffer
};

template <typename R>
static int adjoint_plan(const SdeSpec *s, int n_steps, bool jumps, bool td, bool corr_t, bool ujit, int nv,
                        int req_seg, bool fromck, AdjPlan *P) {
    const int M = s->group_size;
    const bool linear = s->model == SDE_MODEL_LINEAR;
    // the FP32 2-variable Heston adjoint keeps its segment in shared memory:
    // at most ADJ_HESTON_SEG steps, one checkpoint level; constant parameters
    // and correlation
    P->heston_fast = sizeof(R) == 4 && s->model == SDE_MODEL_HESTON && M == 2 && !jumps && !td && !corr_t &&
                     (fromck ? req_seg <= ADJ_HESTON_SEG
                             : (n_steps + ADJ_HESTON_SEG - 1) / ADJ_HESTON_SEG <= ADJ_MAXSEG);
    // and the scalar FP32 OU one: at most ADJ_OU_SEG steps, the state output
    P->ou_fast = sizeof(R) == 4 && s->model == SDE_MODEL_OU && M == 1 && !jumps && !td && !corr_t && !ujit &&
                 s->out_mode == SDE_OUT_STATE &&
                 (fromck ? req_seg <= ADJ_OU_SEG : (n_steps + ADJ_OU_SEG - 1) / ADJ_OU_SEG <= ADJ_MAXSEG);
    int cap = P->heston_fast ? ADJ_HESTON_SEG : P->ou_fast ? ADJ_OU_SEG : ADJ_MAXSEG;
    size_t per_step = 0;
    if (ujit) {   // nv * M values per thread and step in UADJ_SMEM bytes
        per_step = sizeof(R) * (size_t)nv * M * BLOCK;
        cap = (int)(UADJ_SMEM / per_step);
        if (cap > ADJ_MAXSEG) cap = ADJ_MAXSEG;
        if (cap < 1) return fail(SDE_ERR_UNSUPPORTED, "the adjoint's segment buffer does not fit groups of %d", M);
    }
    int seg, seg2;
    auto level2 = [&]() {   // level-2 length inside level-1 segments of seg steps
        int s2 = (int)ceil(sqrt((double)seg));
        if (s2 > cap) s2 = cap;
        if ((seg + s2 - 1) / s2 > ADJ_MAXSEG) s2 = (seg + ADJ_MAXSEG - 1) / ADJ_MAXSEG;
        return s2;
    };
    if (fromck) {
        seg = seg2 = req_seg;
        if (!linear && seg > cap) {
            seg2 = level2();
            if (seg2 > cap)
                return fail(SDE_ERR_UNSUPPORTED, "checkpoint segments of at most %d steps", ADJ_MAXSEG * cap);
        }
    } else {
        seg = req_seg > 0 ? req_seg : (int)ceil(sqrt((double)n_steps));
        if (seg > cap) seg = cap;
        if (seg < 1) seg = 1;
        seg2 = seg;
        if (!linear && (n_steps + seg - 1) / seg > ADJ_MAXSEG) {
            seg = (n_steps + ADJ_MAXSEG - 1) / ADJ_MAXSEG;
            seg2 = level2();
            if (seg2 > cap)
                return fail(SDE_ERR_UNSUPPORTED, "the adjoint supports up to %d steps for groups of %d",
                            ADJ_MAXSEG * ADJ_MAXSEG * cap, M);
        }
    }
    P->cap = cap;
    P->seg = seg;
    P->seg2 = seg2;
    P->nseg = (n_steps + seg - 1) / seg;
    P->ubytes = per_step * seg2;
    return SDE_OK;
}

template <typename R>
static int adjoint_impl(const SdeSpec *s, const SdeGrid *gr, const SdeAdjReq *req, double *grad, double *value) {
    int opg = 0, rc;
    if ((rc = check_spec(s, &opg))) return rc;
    if (!req || !grad) return fail(SDE_ERR_INVALID, "adjoint request and grad are required");
    if (!gr || !gr->tt || gr->n_pts < 2) return fail(SDE_ERR_INVALID, "the adjoint needs a grid of >= 2 points");
    const int n_steps = gr->n_pts - 1;
    for (int k = 0; k < n_steps; ++k)
        if (!(gr->tt[k + 1] > gr->tt[k])) return fail(SDE_ERR_UNSUPPORTED, "the adjoint integrates forward grids only");
    if (req->n_strikes < 0 || req->n_strikes > SDE_MAX_STRIKES) return fail(SDE_ERR_INVALID, "bad n_strikes");
    const int M = s->group_size, W = s->groups * M;
    const AdjKind K = adjoint_kind(s);
    const bool user = K.user, ujit = K.ujit;
    const int ujs = K.ujs, nv = K.nv;
    if (ujit && !jit_available())
        return fail(SDE_ERR_UNSUPPORTED, "the adjoint of user systems and jump terms compiles the program at run "
                                         "time: NVRTC is not available");
    const bool jumps = K.jumps;
    if (gr->lam_t && !(user && jumps))
        return fail(SDE_ERR_INVALID, "grid lam_t applies to user SDEs with dn / dj terms");
    if (user && jumps && !s->program->jump_params)
        return fail(SDE_ERR_INVALID, "a user program with dn / dj terms needs jump_params");
    int maxm = maxm_of(M);
    if (maxm > 8) return fail(SDE_ERR_UNSUPPORTED, "the adjoint supports groups of up to 8 state variables");
    // time-dependent parameter slots: per-step gradients into req->grad_t
    const bool td = gr->params_t != nullptr;
    const size_t td_smem = td ? sizeof(R) * (size_t)n_steps * 3 * maxm : 0;
    if (td) {
        if (user || jumps)
            return fail(SDE_ERR_UNSUPPORTED, "gradients with time-dependent parameters take the preset models "
                                             "without jumps");
        if (!req->grad_t) return fail(SDE_ERR_INVALID, "time-dependent parameters need the request's grad_t");
        if (td_smem > ADJ_TD_SMEM)
            return fail(SDE_ERR_UNSUPPORTED, "gradients with time-dependent parameters: at most %d steps for "
                                             "groups of %d", (int)(ADJ_TD_SMEM / (sizeof(R) * 3 * maxm)), M);
    }
    // checkpoints written by the forward run (the LINEAR adjoint takes none)
    const bool fromck = req->ckpt != nullptr && s->model != SDE_MODEL_LINEAR;
    if (fromck && req->checkpoint < 1)
        return fail(SDE_ERR_INVALID, "checkpoints from the forward need req->checkpoint, their segment length");
    AdjPlan plan;
    const bool corr_t = gr->corr_t != nullptr;
    if ((rc = adjoint_plan<R>(s, n_steps, jumps, td, corr_t, ujit, nv, req->checkpoint, fromck, &plan))) return rc;
    const bool heston_fast = plan.heston_fast;
    const int seg = plan.seg, seg2 = plan.seg2, nseg = plan.nseg;
    const size_t ubytes = plan.ubytes;

    std::lock_guard<std::mutex> lk(g_mu);
    Device *D;
    if ((rc = current_device(&D))) return rc;
    cudaStream_t st = dev_stream(D);

    AdjArgs<R> a;
    memset(&a, 0, sizeof a);
    // host tables: dt, sqdt, x0, prm, jump tables
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t njt = jumps ? (size_t)n_steps * W : 1;
    const size_t o_dt = 0, o_sq = o_dt + al(sizeof(R) * n_steps), o_x0 = o_sq + al(sizeof(R) * n_steps);
    const size_t o_prm = o_x0 + al(sizeof(R) * W), o_lam = o_prm + al(sizeof(R) * SDE_MAX_PARAMS * W);
    const size_t o_p0 = o_lam + al(sizeof(double) * njt), o_thr = o_p0 + al(sizeof(double) * njt);
    const size_t o_thr1 = o_thr + al(sizeof(long long) * njt);
    const size_t o_tk = o_thr1 + al(sizeof(long long) * njt);   // step starts, for user SDEs
    const size_t o_pt = o_tk + al(sizeof(R) * (user ? n_steps : 1));   // slots 0..2 per step
    const size_t o_jp = o_pt + al(sizeof(R) * (td ? (size_t)n_steps * 3 * W : 1));   // a user dj law's a, b, pa
    const size_t o_ct = o_jp + al(sizeof(R) * (user && jumps ? (size_t)3 * W : 1));   // per-step Cholesky rows
    const size_t o_sd = o_ct + al(sizeof(R) * (corr_t ? (size_t)n_steps * NCHOL : 1));   // per-segment dt
    const size_t o_end = o_sd + al(sizeof(R) * 2 * (size_t)nseg);
    D->host_tables.resize(o_end);
    char *H = D->host_tables.data();
    R *h_dt = (R *)(H + o_dt), *h_sq = (R *)(H + o_sq), *h_x0 = (R *)(H + o_x0), *h_prm = (R *)(H + o_prm);
    if (user)
        for (int k = 0; k < n_steps; ++k) ((R *)(H + o_tk))[k] = (R)gr->tt[k];
    double *h_lam = (double *)(H + o_lam), *h_p0 = (double *)(H + o_p0);
    long long *h_thr = (long long *)(H + o_thr), *h_thr1 = (long long *)(H + o_thr1);
    for (int k = 0; k < n_steps; ++k) {
        const double dt = gr->tt[k + 1] - gr->tt[k];
        h_dt[k] = (R)dt;
        h_sq[k] = (R)sqrt(dt);
    }
    for (int w = 0; w < W; ++w) h_x0[w] = (R)s->x0[w];
    for (int i = 0; i < SDE_MAX_PARAMS * W; ++i) h_prm[i] = (R)s->params[i];
    {   // each level-1 segment's dt and sqrt(dt), when its steps share them
        R *h_sd = (R *)(H + o_sd);
        for (int sg = 0; sg < nseg; ++sg) {
            const int k0 = sg * seg, k1 = k0 + seg < n_steps ? k0 + seg : n_steps;
            bool one = true;
            for (int k = k0 + 1; k < k1 && one; ++k)
                one = memcmp(&h_dt[k], &h_dt[k0], sizeof(R)) == 0 && memcmp(&h_sq[k], &h_sq[k0], sizeof(R)) == 0;
            h_sd[2 * sg] = one ? h_dt[k0] : (R)NAN;
            h_sd[2 * sg + 1] = one ? h_sq[k0] : (R)NAN;
        }
    }
    if (td) {   // slots 0..2 of each step of the grid's [steps][SDE_MAX_PARAMS][W] table
        R *h_pt = (R *)(H + o_pt);
        for (int k = 0; k < n_steps; ++k)
            for (int j = 0; j < 3; ++j)
                for (int w = 0; w < W; ++w)
                    h_pt[((size_t)k * 3 + j) * W + w] = (R)gr->params_t[((size_t)k * SDE_MAX_PARAMS + j) * W + w];
    }
    if (user && jumps)
        for (int i = 0; i < 3 * W; ++i) ((R *)(H + o_jp))[i] = (R)s->program->jump_params[W + i];
    if (jumps)
        for (int k = 0; k < n_steps; ++k)
            for (int w = 0; w < W; ++w) {
                // a user SDE's intensity: its table at the step's midpoint, or its constant
                const double lam = !user ? s->params[2 * W + w]
                                   : gr->lam_t ? gr->lam_t[(size_t)k * W + w] : s->program->jump_params[w];
                const double L = (gr->tt[k + 1] - gr->tt[k]) * lam;
                if (!(L >= 0.0) || L > 700.0) return fail(SDE_ERR_INVALID, "bad Poisson intensity");
                const double p0 = exp(-L);
                h_lam[(size_t)k * W + w] = L;
                h_p0[(size_t)k * W + w] = p0;
                poisson_thresholds(p0, L, h_thr[(size_t)k * W + w], h_thr1[(size_t)k * W + w]);
            }
    if (corr_t) {   // each step's factor, as the forward run factors them
        R *h_ct = (R *)(H + o_ct);
        std::vector<double> L(M * M);
        for (int k = 0; k < n_steps; ++k) {
            if ((rc = sde_cholesky(gr->corr_t + (size_t)k * M * M, M, L.data()))) {
                char m[256];
                snprintf(m, sizeof m, "correlation of step %d: %s", k, g_err.c_str());
                return fail(rc, "%s", m);
            }
            R *row = h_ct + (size_t)k * NCHOL;
            for (int i = 0; i < NCHOL; ++i) row[i] = R(0);
            for (int i = 0; i < M; ++i)
                for (int j = 0; j <= i; ++j) row[i * (i + 1) / 2 + j] = (R)L[i * M + j];
        }
        a.has_corr = 1;   // (no gradient of a time-dependent correlation)
    } else if (s->corr) {
        std::vector<double> L(M * M);
        if ((rc = sde_cholesky(s->corr, M, L.data()))) return rc;
        for (int i = 0; i < M; ++i)
            for (int j = 0; j <= i; ++j) a.chol[i * (i + 1) / 2 + j] = (R)L[i * M + j];
        a.has_corr = 1;
        if (M == 2 && s->model == SDE_MODEL_HESTON) {
            const double rho = s->corr[2];
            if (fabs(rho) < 1.0) {
                a.rho_grad = 1;
                a.rho_k = (R)(-rho / sqrt(1.0 - rho * rho));
            }
        }
    }
    void *d_tab;
    if ((rc = scratch(D, S_TABLES, o_end, &d_tab))) return rc;
    CU(cudaMemcpyAsync(d_tab, H, o_end, cudaMemcpyHostToDevice, st));
    char *T = (char *)d_tab;
    a.paths = s->paths;
    a.groups = s->groups;
    a.M = M;
    a.W = W;
    a.n_steps = n_steps;
    a.seg = seg;
    a.nseg = nseg;
    a.seg2 = seg2;
    a.ckpt = fromck ? (const R *)req->ckpt : nullptr;
    a.chol_t = corr_t ? (const R *)(T + o_ct) : nullptr;
    a.segdt = (const R *)(T + o_sd);
    a.step_offset = gr->step_offset;
    a.out_mode = s->out_mode;
    a.jump_law = s->jump_law;
    a.seed = s->seed;
    a.stream = s->stream;
    a.path_offset = s->path_offset;
    a.key = philox_schedule(s->seed);
    a.dt = (const R *)(T + o_dt);
    a.sqdt = (const R *)(T + o_sq);
    a.x0 = (const R *)(T + o_x0);
    a.prm = (const R *)(T + o_prm);
    a.lamdt = (const double *)(T + o_lam);
    a.p0 = (const double *)(T + o_p0);
    a.thr = (const long long *)(T + o_thr);
    a.thr1 = (const long long *)(T + o_thr1);
    if (user) {
        a.uprog = *s->program;
        a.tk = (const R *)(T + o_tk);
        a.user_jsrc = ujs;
        if (jumps) a.jprm = (const R *)(T + o_jp);
    }
    if (td) a.prm_t = (const R *)(T + o_pt);
    a.n_strikes = req->n_strikes;
    for (int i = 0; i < req->n_strikes; ++i) {
        a.strikes[i] = (R)req->strikes[i];
        a.weights[i] = (R)req->weights[i];
    }
    a.wmean = (R)req->mean_weight;
    void *d_err;
    if ((rc = scratch(D, S_ERR, 16, &d_err))) return rc;
    CU(cudaMemsetAsync(d_err, 0, 16, st));
    a.err = (int32_t *)d_err;

    int bps = 0;
    // a user program compiled at run time, or an instantiated kernel
    cudaKernel_t jk = nullptr;
    AdjLauncher<R> L = nullptr;
    if (ujit) {
        std::string err;
        if ((rc = jit_adj_kernel(*s->program, sizeof(R) == 8, M, &jk, &err))) return fail(rc, "%s", err.c_str());
        CU(cudaFuncSetAttribute((const void *)jk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ubytes));
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void *)jk, BLOCK, ubytes));
        if (bps < 1) bps = 1;
    } else if (heston_fast) {
        L = AdjFinder<R>::find_heston(seg, &bps);
    } else if (plan.ou_fast) {
        L = AdjFinder<R>::find_ou(seg, &bps);
    } else {
        L = td ? AdjFinder<R>::find_td(s->model, maxm, &bps) : AdjFinder<R>::find(s->model, maxm, jumps, &bps);
        if (!L) return fail(SDE_ERR_UNSUPPORTED, "no adjoint kernel for model %d group size %d%s", s->model, M,
                            td ? " with time-dependent parameters" : "");
    }
    if (td) {   // the per-step table lowers the resident blocks
        const int by_smem = (int)(ADJ_TD_SMEM_SM / (td_smem + 1024));
        if (by_smem < bps) bps = by_smem < 1 ? 1 : by_smem;
    }
    const int nbx = path_blocks(D, s->paths, s->groups, bps);
    const int npa = maxm * NGV + 2;
    void *part, *res;
    if ((rc = scratch(D, S_PART, sizeof(double) * (size_t)s->groups * nbx * npa, &part))) return rc;
    if ((rc = scratch(D, S_RES, sizeof(double) * (size_t)s->groups * npa, &res))) return rc;
    a.partials = (double *)part;
    const int ntd = td ? n_steps * 3 * maxm : 0;
    void *tdpart = nullptr, *tdres = nullptr;
    if (td) {
        if ((rc = scratch(D, S_VALS, sizeof(double) * (size_t)s->groups * nbx * ntd, &tdpart))) return rc;
        if ((rc = scratch(D, S_EDGES64, sizeof(double) * (size_t)s->groups * ntd, &tdres))) return rc;
        a.tdpart = (double *)tdpart;
    }
    if (D->timing) CU(cudaEventRecord(D->ev[0], st));
    if (jk) {
        void *args[] = {(void *)&a};
        CU(cudaLaunchKernel((const void *)jk, dim3(nbx, s->groups), dim3(BLOCK), args, ubytes, st));
    } else {
        L(a, dim3(nbx, s->groups), st);
    }
    CU(cudaGetLastError());
    if (D->timing) CU(cudaEventRecord(D->ev[1], st));
    for (int g = 0; g < s->groups; ++g) {
        reduce_partials_kernel<<<npa, BLOCK, 0, st>>>((const double *)part + (size_t)g * nbx * npa, nbx, npa,
                                                     (double *)res + (size_t)g * npa);
        if (td)
            reduce_partials_kernel<<<ntd, BLOCK, 0, st>>>((const double *)tdpart + (size_t)g * nbx * ntd, nbx, ntd,
                                                         (double *)tdres + (size_t)g * ntd);
    }
    CU(cudaGetLastError());
    std::vector<double> h((size_t)s->groups * npa), htd((size_t)s->groups * ntd);
    int32_t herr = 0;
    CU(cudaMemcpyAsync(h.data(), res, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
    if (td) CU(cudaMemcpyAsync(htd.data(), tdres, sizeof(double) * htd.size(), cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&herr, d_err, sizeof herr, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (D->timing) {
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, D->ev[0], D->ev[1]));
        D->last_ms[0] = ms;
        D->last_ms[1] = 0.0;
        D->last_ms[2] = nbx;
        D->last_ms[3] = 1 + s->groups;
    }
    if (herr & ERRF_JUMP_CAP) return fail(SDE_ERR_DEVICE, "more than %d jumps in one step", SDE_MAX_JUMPS_PER_STEP);
    const double inv = 1.0 / (double)s->paths;
    double v = 0.0;
    for (int g = 0; g < s->groups; ++g) {
        for (int m = 0; m < M; ++m)
            for (int j = 0; j < NGV; ++j) grad[((size_t)g * M + m) * NGV + j] = h[(size_t)g * npa + m * NGV + j] * inv;
        v += h[(size_t)g * npa + maxm * NGV];
    }
    if (value) *value = v * inv;
    if (td)   // grad_t[k][j][w], w = g * M + m
        for (int g = 0; g < s->groups; ++g)
            for (int k = 0; k < n_steps; ++k)
                for (int j = 0; j < 3; ++j)
                    for (int m = 0; m < M; ++m)
                        req->grad_t[((size_t)k * 3 + j) * W + (size_t)g * M + m] =
                            htd[(size_t)g * ntd + ((size_t)k * 3 + j) * maxm + m] * inv;
    return SDE_OK;
}

template <typename R>
static int adjoint_checkpoints_impl(const SdeSpec *s, const SdeGrid *gr, int32_t *seg, int64_t *bytes) {
    int opg = 0, rc;
    if ((rc = check_spec(s, &opg))) return rc;
    if (!gr || gr->n_pts < 2) return fail(SDE_ERR_INVALID, "the adjoint needs a grid of >= 2 points");
    *seg = 0;
    *bytes = 0;
    const int n_steps = gr->n_pts - 1;
    // none read (LINEAR), or none written: antithetic runs, and the FP32 OU
    // run-table forward but for the state output with constant parameters
    // and correlation
    const bool table_none = sizeof(R) == 4 && s->model == SDE_MODEL_OU &&
                            (s->out_mode != SDE_OUT_STATE || gr->params_t || gr->corr_t);
    if (s->model == SDE_MODEL_LINEAR || table_none || s->flags) return SDE_OK;
    const AdjKind K = adjoint_kind(s);
    AdjPlan P;
    if ((rc = adjoint_plan<R>(s, n_steps, K.jumps, gr->params_t != nullptr, gr->corr_t != nullptr, K.ujit, K.nv, 0,
                              false, &P)))
        return rc;
    *seg = P.seg;
    *bytes = (int64_t)P.nseg * s->groups * s->group_size * s->paths * (int64_t)sizeof(R);
    return SDE_OK;
}

extern "C" int32_t sde_adjoint_checkpoints(const SdeSpec *spec, const SdeGrid *grid, int32_t *seg, int64_t *bytes) {
    if (!spec || !seg || !bytes) return fail(SDE_ERR_INVALID, "spec, seg and bytes are required");
    if (spec->precision == SDE_FP32) return adjoint_checkpoints_impl<float>(spec, grid, seg, bytes);
    return adjoint_checkpoints_impl<double>(spec, grid, seg, bytes);
}

extern "C" int32_t sde_adjoint(const SdeSpec *spec, const SdeGrid *grid, const SdeAdjReq *req, double *grad,
                               double *value) {
    if (!spec) return fail(SDE_ERR_INVALID, "spec is NULL");
    if (spec->flags) return fail(SDE_ERR_UNSUPPORTED, "the adjoint takes no spec flags (antithetic paths)");
    if (spec->precision == SDE_FP32) return adjoint_impl<float>(spec, grid, req, grad, value);
    return adjoint_impl<double>(spec, grid, req, grad, value);
}
