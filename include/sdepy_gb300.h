/*
 * sdepy_gb300 C-ABI: Monte Carlo path integration of the sdepy preset SDEs
 * on one GB300 GPU (sm_103a).
 *
 * Plain C types only: the Python host binds it with ctypes, and any other
 * host (C, C++, Fortran, another FFI) can bind it the same way.
 *
 * Every entry point returns an int status (SDE_OK == 0, negative on error);
 * sde_last_error() returns the message of the last failure on the calling
 * thread.
 *
 * Vocabulary follows sdepy:
 *   paths   - independent realisations (last axis of every array);
 *   wshape  - working shape of the integrated state of one path, flattened
 *             here to groups * group_size state variables;
 *   group   - the state variables that share one correlated Wiener
 *             increment (sdepy correlates along the last wshape axis);
 *   steps   - points of the integration grid (sdepy's steps_tt);
 *   rows    - points of the output timeline (sdepy's tt / xx[i]).
 *
 * Array layouts (C order, paths innermost):
 *   xx  [n_rows][n_out_vars][paths]   precision of the run (f64 or f32)
 *   dw  [n_steps][groups*group_size][paths]  f64, injected increments
 */
#ifndef SDEPY_GB300_H
#define SDEPY_GB300_H

#ifndef __CUDACC_RTC__   /* runtime compilation (NVRTC) defines the integer types itself */
#include <stdint.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SDE_API __attribute__((visibility("default")))
#else
#define SDE_API
#endif

#define SDE_ABI_VERSION 6

#define SDE_MAX_GROUP   16   /* largest correlated group (state vars) */
#define SDE_MAX_PARAMS  6    /* coefficient arrays per state variable */
#define SDE_MAX_STRIKES 8    /* payoff strikes of one fused reduction  */
#define SDE_MAX_JUMPS_PER_STEP 4096

/* status codes */
#define SDE_OK                 0
#define SDE_ERR_INVALID       -1   /* bad argument (shape, pointer, value) */
#define SDE_ERR_UNSUPPORTED   -2   /* valid request outside the GPU path  */
#define SDE_ERR_CUDA          -3   /* CUDA runtime failure                */
#define SDE_ERR_DEVICE        -4   /* kernel reported an error flag       */
#define SDE_ERR_NO_DEVICE     -5   /* no CUDA device visible              */

/* model: the coefficient form integrated by the Euler step */
#define SDE_MODEL_LINEAR  0  /* dx = c_dt*dt + c_dw*dw [+ dj]: wiener, lognorm, jumpdiff */
#define SDE_MODEL_OU      1  /* dx = k*(theta - x)*dt + sigma*dw: OU, Hull-White factors */
#define SDE_MODEL_HESTON  2  /* (log x, y) with full truncation y+ = max(y, 0)           */
#define SDE_MODEL_CIR     3  /* dx = k*(theta - x+)*dt + xi*sqrt(x+)*dw, x+ = max(x, 0)  */
#define SDE_MODEL_USER    4  /* dx = sum of A_s(t, x, p)*ds, s in dt, dw, dn, dj; SdeUserProgram */

/* params[p][w] meaning, per model (w = state variable index):
 *   LINEAR : p0 = c_dt, p1 = c_dw, p2 = lam, p3 = a, p4 = b, p5 = pa
 *   OU     : p0 = k, p1 = theta, p2 = sigma
 *   HESTON : w in the first half of a group (log-price):  p0 = mu, p1 = sigma
 *            w in the second half of a group (variance):  p0 = k, p1 = theta, p2 = xi
 *   CIR    : p0 = k, p1 = theta, p2 = xi
 *   USER   : p0..p5 = the SDE function's parameters, in the program's order
 */

/* A user SDE (sdepy's integrate decorator, sdepy/integration.py:1843-1955):
 * the coefficients A_dt and A_dw of q equations (q = n_eq; 1 for a single
 * SDE), compiled from the SDE function into a straight-line program.  The
 * program runs per step and per component: on the component's state x of
 * a single equation, or on the states of that component in every equation
 * of a system (sdepy's SDEs: a group of the spec is one last-axis slice of
 * the working shape, holding group_size / q components of each equation,
 * equation e's component h at e * (group_size / q) + h).  Registers: r0 =
 * the state of equation 0, r1 = t (the step's start), r2..r7 = parameters
 * p0..p5, r8..r(6 + q) = the states of equations 1..q-1, the rest
 * temporaries; SDE_USER_MAX_REGS in all.  An instruction is code | dst << 8
 * | a << 16 | b << 24 (SDE_UOP_*: dst = f(ra, rb); SDE_UOP_CONST: dst =
 * consts[a]).  Equation e steps x + (A_1 dZ_1 + ... + A_n dZ_n), summed
 * left to right, its coefficients in registers term_register[e][0..n-1],
 * the sources term_source[] in the order of the SDE function's returned
 * dict (sdepy's euler_next, sdepy/integration.py:707-718).  dZ is dt, the
 * Wiener increment dw, the Poisson increment dn (sdepy's source_dn,
 * sdepy/integration.py:1346-1378) or the compound Poisson increment dj
 * (source_dj, :1380-1423).  With dn or dj terms, jump_params holds per
 * state the Poisson intensity lam (shared by dn and dj, as the reference
 * shares its 'lam' argument) and the jump-size law's a, b, pa (law
 * SdeSpec.jump_law, which is SDE_JUMP_NONE without a dj term); dn and dj
 * of one program are independent Poisson processes. */
#define SDE_USER_MAX_OPS    64
#define SDE_USER_MAX_CONSTS 16
#define SDE_USER_MAX_REGS   48
#define SDE_USER_MAX_EQ     8
#define SDE_USER_MAX_TERMS  4
#define SDE_SRC_DT 0
#define SDE_SRC_DW 1
#define SDE_SRC_DN 2
#define SDE_SRC_DJ 3
enum {
    SDE_UOP_CONST = 0, SDE_UOP_ADD, SDE_UOP_SUB, SDE_UOP_MUL, SDE_UOP_DIV, SDE_UOP_NEG,
    SDE_UOP_ABS, SDE_UOP_EXP, SDE_UOP_LOG, SDE_UOP_SQRT, SDE_UOP_MAX, SDE_UOP_MIN,
    SDE_UOP_SIN, SDE_UOP_COS, SDE_UOP_TAN, SDE_UOP_TANH, SDE_UOP_POW, SDE_UOP_EXPM1,
    SDE_UOP_LOG1P, SDE_UOP_ARCTAN, SDE_UOP_COPY, SDE_UOP_COUNT
};
typedef struct SdeUserProgram {
    int32_t n_ops;
    int32_t n_eq;                     /* equations q, 1..SDE_USER_MAX_EQ          */
    int32_t n_terms;                  /* terms of each equation's sum, 0..4      */
    int32_t term_source[SDE_USER_MAX_TERMS];     /* SDE_SRC_*, each at most once */
    int32_t term_register[SDE_USER_MAX_EQ][SDE_USER_MAX_TERMS];   /* coefficients */
    uint32_t ops[SDE_USER_MAX_OPS];
    double consts[SDE_USER_MAX_CONSTS];
    const double *jump_params;        /* [4][groups*M] lam, a, b, pa; NULL without dn / dj */
    int32_t jit;                      /* 1: compile the program to native code for the
                                       * forward kernel (NVRTC, cached per process;
                                       * sde_jit_available()), 0: interpret it */
    int32_t reserved;
} SdeUserProgram;

/* jump-size law of the compound Poisson source (LINEAR model, and user
 * SDEs with a dj term) */
#define SDE_JUMP_NONE        0
#define SDE_JUMP_NORM        1   /* y = a + b*z                    */
#define SDE_JUMP_DOUBLE_EXP  2   /* y = a*e w.p. pa, else -b*e     */
#define SDE_JUMP_UNIFORM     3   /* y = a + (b - a)*u              */
#define SDE_JUMP_EXP         4   /* y = a*e                        */

/* arithmetic of the path states */
#define SDE_FP64  0
#define SDE_FP32  1

/* how a group's state is stored into an output row */
#define SDE_OUT_STATE      0  /* all group_size states, as integrated          */
#define SDE_OUT_EXP        1  /* exp() of all states (sdepy log=True models)   */
#define SDE_OUT_SUM        2  /* one value: sum of the states (Hull-White)     */
#define SDE_OUT_HESTON_X   3  /* exp() of the first half (heston_process)      */
#define SDE_OUT_HESTON_XY  4  /* exp() of first half, second half as is        */

/* SdeSpec.flags: antithetic paths (device noise only): with paths = 2K,
 * path K + q takes the draws of path q with opposite Wiener increments and
 * the same Poisson counts and jump sizes, as sdepy's odd_wiener_source with
 * even_cpoisson_source (sdepy/infrastructure.py:2047-2150); groups of up to
 * 8 states, constant or time-dependent coefficients and correlations. */
#define SDE_FLAG_ANTITHETIC 1

typedef struct SdeSpec {
    int32_t abi_version;   /* SDE_ABI_VERSION */
    int32_t model;         /* SDE_MODEL_* */
    int32_t precision;     /* SDE_FP64 | SDE_FP32 */
    int32_t jump_law;      /* SDE_JUMP_* */
    int64_t paths;
    int32_t groups;        /* independent groups per path */
    int32_t group_size;    /* M: states per group, 1..SDE_MAX_GROUP */
    int32_t out_mode;      /* SDE_OUT_* */
    int32_t flags;         /* SDE_FLAG_* */
    const double *x0;      /* [groups*M] initial state (already log()-ed for log models) */
    const double *params;  /* [SDE_MAX_PARAMS][groups*M] */
    const double *corr;    /* [M*M] correlation matrix shared by all groups, or NULL */
    uint64_t seed;         /* Philox-4x32-10 key */
    uint32_t stream;       /* Philox counter word 3 (call / instance id) */
    /* Added to the local path index in Philox counter word 0: the call
     * integrates paths [path_offset, path_offset + paths) of a larger sample
     * (path_offset + paths <= 2^32), so that contiguous path ranges run on
     * different devices or calls reproduce one run of all the paths. */
    uint32_t path_offset;
    const SdeUserProgram *program;   /* SDE_MODEL_USER: the coefficients, else NULL */
} SdeSpec;

typedef struct SdeGrid {
    const double *tt;       /* [n_pts] integration points, in integration order      */
    const int32_t *out_row; /* [n_pts] output row stored at each point, or -1         */
    int32_t n_pts;          /* >= 1; n_steps = n_pts - 1                               */
    uint32_t step_offset;   /* added to the step index in the Philox counter          */
    /* Time-dependent parameters, or NULL (SdeSpec.params apply at every
     * step): [n_pts - 1][SDE_MAX_PARAMS][groups*M], row k the parameters of
     * step k from tt[k] to tt[k+1].  Slots 0..2 are the SDE's coefficients
     * evaluated at tt[k] (sdepy's SDE.A, sdepy/integration.py:1216-1225);
     * for jump models slot 2 is the Poisson intensity evaluated at the
     * step's midpoint tt[k] + dt/2 (sdepy/infrastructure.py:1629); slots
     * 3..5 (jump-size laws) are read from SdeSpec.params.  sde_run and
     * sde_run_stats accept it, and sde_adjoint (per-step gradients,
     * SdeAdjReq.grad_t); sde_run_stats_static returns SDE_ERR_UNSUPPORTED. */
    const double *params_t;
    /* Time-dependent correlation, or NULL (SdeSpec.corr applies at every
     * step): [n_pts - 1][M][M], row k the correlation matrix of the Wiener
     * increments of step k, evaluated at its midpoint tt[k] + dt/2 as
     * sdepy's wiener_source evaluates a callable corr
     * (sdepy/infrastructure.py:1540).  The library factors every step's
     * matrix (sde_cholesky).  Ignored with injected increments;
     * sde_adjoint draws with the same factors (the correlation is not
     * differentiated: no rho gradient); sde_run_stats_static returns
     * SDE_ERR_UNSUPPORTED. */
    const double *corr_t;
    /* User SDEs with dn / dj terms: time-dependent Poisson intensity, or
     * NULL (SdeUserProgram.jump_params row 0 applies at every step):
     * [n_pts - 1][groups*M], row k evaluated at step k's midpoint
     * tt[k] + dt/2 (sdepy/infrastructure.py:1629). */
    const double *lam_t;
} SdeGrid;

typedef struct SdeNoise {   /* host arrays of injected increments (f64) */
    const double *dw;       /* [n_steps][groups*M][paths], required        */
    const double *dj;       /* [n_steps][groups*M][paths] or NULL           */
    const int64_t *dn;      /* [n_steps][groups*M][paths] or NULL: the Poisson
                             * counts of dj (jump_count info), or, for a user
                             * SDE with a dn term, that source's increments */
} SdeNoise;

typedef struct SdeOut {
    void *xx;               /* [n_rows][n_out_vars][paths] or NULL (write nothing)  */
    int32_t n_rows;
    int32_t on_device;      /* 1: every pointer below and xx is device memory      */
    int32_t *neg_count;     /* HESTON: [groups*M/2][paths] steps with y < 0, or NULL */
    int32_t *jump_count;    /* jumps:  [groups*M][paths] Poisson events, or NULL     */
    int64_t *row_jumps;     /* jumps:  [n_rows] events per output interval, or NULL  */
    /* Adjoint checkpoints, or NULL: device memory the run fills with the
     * state before every ckpt_seg-th step (steps 0, ckpt_seg, 2 ckpt_seg,
     * ...), [ceil(n_steps / ckpt_seg)][groups*M][paths] in the spec's
     * precision, so that an sde_adjoint of the same spec and grid reads them
     * (SdeAdjReq.ckpt) instead of its own forward sweep;
     * sde_adjoint_checkpoints gives the segment and the bytes.  Device RNG
     * only, no antithetic paths; the FP32 LINEAR / OU run-table kernels
     * write none (SDE_ERR_UNSUPPORTED; the adjoint recomputes them). */
    void *ckpt;
    int32_t ckpt_seg;
} SdeOut;

typedef struct SdeStatsReq {
    int32_t row;            /* output row whose values are summarised              */
    int32_t bins;           /* histogram bins, 0 for none                          */
    int32_t has_range;      /* 1: use [range_lo, range_hi], else data min..max     */
    int32_t n_strikes;      /* payoff sums E[max(x - K, 0)], 0..SDE_MAX_STRIKES    */
    double range_lo, range_hi;
    double strikes[SDE_MAX_STRIKES];
} SdeStatsReq;

/* per output variable o (host arrays):
 *   moments[o*8 + 0..7] = n, mean, M2, M3, M4 (central sums), min, max, 0
 *   payoff [o*n_strikes + s] = mean of max(x - K_s, 0)
 *   counts [o*bins + b], edges [o*(bins+1) + e] as numpy.histogram returns them
 */
typedef struct SdeStatsOut {
    double *moments;
    double *payoff;
    int64_t *counts;
    double *edges;
} SdeStatsOut;

/* ---- version / device / errors --------------------------------------- */

SDE_API int32_t sde_abi_version(void);

/* message of the last failed call on this thread (NUL-terminated, truncated) */
SDE_API int32_t sde_last_error(char *buf, int32_t len);

/* number of visible CUDA devices (0 if none); never fails */
SDE_API int32_t sde_device_count(void);

/* 1 if user SDE programs can be compiled at run time (NVRTC found), else 0. */
SDE_API int32_t sde_jit_available(void);

/* Compile, without loading, the forward kernel of a user program for a
 * precision (SDE_FP64 / SDE_FP32), group size, noise mode (injected 0/1)
 * and jump terms (0/1): a check of the code generation that needs no
 * device.  Returns SDE_OK or an error with NVRTC's log in log[len]. */
SDE_API int32_t sde_jit_compile(const SdeUserProgram *program, int32_t precision, int32_t group_size,
                                int32_t injected, int32_t jumps, char *log, int32_t len);

/* The same for the adjoint kernel of a program (single equations and
 * systems, any terms) for groups of group_size states (1..8, whole
 * components of a system): the coefficients and the generated
 * reverse-mode step compiled in. */
SDE_API int32_t sde_jit_compile_adjoint(const SdeUserProgram *program, int32_t precision, int32_t group_size,
                                        char *log, int32_t len);

/* free the device scratch cached by the library on the current device */
SDE_API int32_t sde_release(void);

/* run later calls on the current device on this cudaStream_t (NULL: the
 * library's own stream, which is ordered with the legacy default stream) */
SDE_API int32_t sde_set_stream(void *stream);

/* Kernel timing of later calls on the current device (enable = 1 / 0,
 * or -1 to leave it unchanged).  last_ms (4 doubles, may be NULL) receives,
 * for the last sde_run / sde_run_stats: [0] forward kernel ms, [1]
 * statistics kernels ms, [2] blocks of the forward grid, [3] kernels
 * launched -- measured with CUDA events on the launching stream. */
SDE_API int32_t sde_timing(int32_t enable, double *last_ms);

/* Peak-rate probe used as roofline denominator for the non-tensor,
 * non-HBM-bound kernels: which = 0 SFU (lg2/sqrt/sin/cos approx) ops/s,
 * 1 FP32 FMA ops/s, 2 32-bit integer multiply-high ops/s; result in ops/s
 * for the whole device, measured with CUDA events. */
SDE_API int32_t sde_peak_probe(int32_t which, double *ops_per_s);

/* The Box-Muller transform the kernels apply to a pair of Philox words
 * (a, b) -> (z0, z1), for n pairs in host memory (words[2i], words[2i+1]),
 * in FP64 or FP32 (returned as doubles).  No counterpart in sdepy: it lets
 * tests check the device transform against other implementations on
 * chosen words (extremes included). */
SDE_API int32_t sde_normal_pairs(const uint32_t *words, int64_t n, int32_t precision, double *out);

/* Page-locked host memory for results; stands where sdepy allocates the
 * result array with numpy (sdepy/integration.py:550, np.full of NaN in
 * paths_generator.__call__).  An output array (SdeOut.xx with
 * on_device == 0) that lives in such memory is written by the kernel
 * directly over the host link, with no device buffer and no separate copy;
 * other host memory goes through a device buffer and one copy. */
SDE_API int32_t sde_host_alloc(int64_t bytes, void **ptr);
SDE_API int32_t sde_host_free(void *ptr);

/* ---- host utilities (no GPU) ------------------------------------------ */

/* Lower-triangular L with L*L^T = corr (M x M, row-major); tolerant of
 * semi-definite input (zero pivots give zero columns).
 * Replaces the factorisation done inside numpy multivariate_normal
 * (sdepy/infrastructure.py:1532-1534). */
SDE_API int32_t sde_cholesky(const double *corr, int32_t M, double *L);

/* ---- path integration -------------------------------------------------- */

/* Euler-Maruyama integration of all paths along grid; stores the states at
 * the points flagged in grid->out_row into out->xx.
 * noise == NULL draws Philox normals / uniforms on the device; otherwise the
 * given increments are used (FP64 parity mode).
 * Replaces paths_generator.__call__ / _generate_paths with
 * integrator.euler_next (sdepy/integration.py:476-584, 392-474, 707-723),
 * SDE.A / SDEs.A (integration.py:1216-1225, 1711-1730) for the presets of
 * integration.py:2056-2747, and the sources wiener_source,
 * poisson_source, cpoisson_source (sdepy/infrastructure.py:1503-1560,
 * 1617-1633, 2017-2040). */
SDE_API int32_t sde_run(const SdeSpec *spec, const SdeGrid *grid,
                const SdeNoise *noise, SdeOut *out);

/* sde_run plus a fused montecarlo summary of one output row: moments,
 * payoff means and histogram, written to stats (host arrays).
 * out->xx may be NULL: the states are then reduced in-kernel and no path
 * array is written.
 * Replaces montecarlo(x[row], bins=..., range=...)
 * (sdepy/infrastructure.py:2826-2922, 2924-3021). */
SDE_API int32_t sde_run_stats(const SdeSpec *spec, const SdeGrid *grid,
                      const SdeNoise *noise, SdeOut *out,
                      const SdeStatsReq *req, SdeStatsOut *stats);

/* Pathwise gradients of  L = sum_o mean_paths f(X_o(T)),
 *   f(X) = mean_weight * X + sum_s weights[s] * max(X - strikes[s], 0),
 * X_o(T) the outputs at the last grid point, for the device-RNG paths of
 * (spec, grid) -- the same paths sde_run integrates.  grad is
 * [groups*M][8]: per state variable d L / d of x0 (integration variable),
 * params p0..p5, and in slot 7 of a group's first variable d L / d rho
 * (2-variable Heston group with corr = [[1, rho], [rho, 1]]).  value = L.
 * For a user SDE slot 1 + j is d L / d of the program's parameter p_j:
 * single equations driven by dt / dw with SdeUserProgram.jit = 0 run the
 * interpreted program in tangent mode; with jit = 1, and always for systems
 * and programs with dn / dj terms, the program is compiled at run time
 * with its generated reverse-mode step (NVRTC; SDE_ERR_UNSUPPORTED
 * without it).  For a system, f reads the first equation's states of each
 * group and slot 1 + j of state h holds the gradient of component h's
 * parameter; jump counts, intensities (SdeGrid.lam_t accepted) and
 * jump-size laws are not differentiated.
 * The adjoint of the Euler recursion is propagated backwards through
 * checkpointed segments recomputed from Philox counters (constant for the
 * LINEAR model); no path is stored.  No counterpart in the reference
 * (sdepy has no derivatives); it differentiates the recursion of
 * sdepy/integration.py:707-718. */
typedef struct SdeAdjReq {
    int32_t n_strikes;
    int32_t checkpoint;      /* steps per segment, 0: ceil(sqrt(steps)); runs
                              * needing more than 64 segments use two levels
                              * of checkpoints (up to 64^3 steps) */
    double strikes[SDE_MAX_STRIKES];
    double weights[SDE_MAX_STRIKES];
    double mean_weight;
    /* With SdeGrid.params_t (the preset models without jumps): out,
     * [n_steps][3][groups*M], d L / d of parameter slot j (0..2) of step k
     * of each state variable -- the per-step coefficients the table gives
     * (sdepy evaluates callable parameters per step, SDE.A at
     * sdepy/integration.py:1216-1225); grad's slots 1..3 are then unused.
     * NULL without params_t.  The per-step table is reduced in shared
     * memory: steps x 3 x group width x 4 (FP32) or 8 (FP64) bytes must not
     * exceed 160 KiB. */
    double *grad_t;
    /* Checkpoints written by the forward run of the same spec and grid
     * (SdeOut.ckpt with ckpt_seg == checkpoint), or NULL: the adjoint then
     * skips its checkpoint sweep and recomputes each segment from them, and
     * takes the terminal states from the last segment's recomputation.  The
     * gradient is the same: bit for bit in FP64 (the forward's and the
     * adjoint's paths are the same rounded operations), to FP32 rounding in
     * FP32 (the compiler may fuse a product into a sum differently in the
     * two kernels). */
    const void *ckpt;
} SdeAdjReq;

SDE_API int32_t sde_adjoint(const SdeSpec *spec, const SdeGrid *grid,
                            const SdeAdjReq *req, double *grad, double *value);

/* The checkpoints sde_adjoint can read for (spec, grid): *seg the steps per
 * segment to pass as SdeOut.ckpt_seg and SdeAdjReq.checkpoint, *bytes the
 * size of the SdeOut.ckpt array.  *seg = 0 (and *bytes = 0) where the
 * adjoint takes none: the LINEAR model (one sweep), the FP32 LINEAR / OU
 * run-table forward, time-dependent parameters. */
SDE_API int32_t sde_adjoint_checkpoints(const SdeSpec *spec, const SdeGrid *grid, int32_t *seg, int64_t *bytes);

/* sde_run_stats for callers that cannot allocate device memory: a serving
 * or real-time loop where cudaMalloc's implicit synchronisation is not
 * acceptable, a plugin inside a framework that owns all device memory, a
 * process with a memory budget fixed at start-up.  Same inputs and same
 * host outputs as sde_run_stats with out->xx == NULL (the fused summary of
 * device-RNG paths, nothing else written), computed with one library-owned
 * static device array of 16 MiB instead of allocated scratch; models with
 * jumps are not supported.  Requests that need more than the 16 MiB (grid,
 * tables, block partials, results and, when bins > 0, the summarised
 * values: 4 or 8 bytes x paths x outputs) fail with SDE_ERR_INVALID.
 * stream: a cudaStream_t, or NULL for the legacy default stream.  The first
 * call on a device looks up the array's device address; make it before any
 * stream capture.  Calls share the array and would race if they overlapped
 * on the GPU; each call finishes (synchronises its stream) before
 * returning.  Calls no cudaMalloc / cudaFree.  No counterpart in the
 * reference: an allocation-free variant of the fused summary above. */
SDE_API int32_t sde_run_stats_static(const SdeSpec *spec, const SdeGrid *grid,
                                     const SdeStatsReq *req, SdeStatsOut *stats,
                                     void *stream);

/* ---- batched instances ---------------------------------------------------- */

/* One SDE instance of a batch: `paths` paths on `n_steps` equal Euler steps
 * of [0, T] (device Philox noise with the counter layout of sde_run). */
typedef struct SdeBatchInstance {
    int32_t model;          /* SDE_MODEL_LINEAR | SDE_MODEL_OU | SDE_MODEL_HESTON      */
    int32_t jump_law;       /* SDE_JUMP_NONE, or SDE_JUMP_NORM with the LINEAR model   */
    int32_t nvars;          /* states: 1 (LINEAR), 1..4 (OU), 2 (HESTON)               */
    int32_t n_steps;
    int64_t paths;
    double T;
    double x0[4];           /* initial states, integration variable                    */
    double params[6][4];    /* as SdeSpec.params, per state                            */
    double rho;             /* HESTON: correlation of the two increments               */
    uint64_t seed;          /* Philox key                                              */
    uint32_t stream;        /* Philox counter word 3                                   */
    int32_t out_exp;        /* 1: X = exp(state) (log models)                          */
} SdeBatchInstance;

/* Build a batch plan: the instances split into work items of `slab` paths
 * (a multiple of 32), sorted longest first, and the device arrays of one
 * persistent launch.  *handle identifies the plan.  Replaces looping the
 * single-instance call over instances; no counterpart in the reference,
 * which integrates one process per call (sdepy/integration.py:476). */
SDE_API int32_t sde_batch_create(const SdeBatchInstance *inst, int32_t n,
                                 int32_t slab, int32_t *handle);

/* Run a plan: one persistent launch in which every warp takes work items
 * from an atomic queue, then a fixed-order merge per instance; with
 * use_graph the two launches are captured once into a CUDA graph and the
 * graph is relaunched.  results (host, may be NULL) is [n][11]: paths, mean
 * and std of X(T) of the first state, and 8 pathwise derivatives of the
 * mean of X(T) (tangent mode): LINEAR d/d(x0, c_dt, c_dw, -, jump a,
 * jump b), OU d/d(x0, k, theta, sigma), HESTON d/d(x0, mu, sigma, y0, k,
 * theta, xi, rho), x0 in the integration variable.  ms: device time.
 * Runs of the same plan must not overlap. */
SDE_API int32_t sde_batch_run(int32_t handle, int32_t use_graph,
                              double *results, double *ms);

/* info[4] = instances, work items, slab, persistent blocks */
SDE_API int32_t sde_batch_info(int32_t handle, int32_t *info);

SDE_API int32_t sde_batch_destroy(int32_t handle);

/* montecarlo summary of an existing sample [n_vars][paths] (f64 if
 * is_fp32 == 0, else f32; host or device per on_device).
 * Replaces montecarlo._update_moments / _update_histogram
 * (sdepy/infrastructure.py:2924-3021) for one update call. */
SDE_API int32_t sde_sample_stats(const void *sample, int32_t is_fp32, int32_t on_device,
                         int64_t n_vars, int64_t paths,
                         const SdeStatsReq *req, SdeStatsOut *stats);

/* Histogram of sample [n_vars][paths] against given edges [n_vars][bins+1]
 * with numpy.histogram's bin rule (used by montecarlo.update after the
 * first sample fixed the bins). */
SDE_API int32_t sde_sample_histogram(const void *sample, int32_t is_fp32, int32_t on_device,
                             int64_t n_vars, int64_t paths, int32_t bins,
                             const double *edges, int64_t *counts);

/* ---- process post-processing: summaries of written process values -------
 * x holds process values [n_rows][n_vars][paths] (f64, or f32 when
 * is_fp32), in device memory when on_device, else in host memory:
 * page-locked host memory (sde_host_alloc, cudaHostAlloc) is read in place
 * by the kernels, other host memory is copied to the device first. */

/* Summaries across paths of each of n_series = n_rows * n_vars series:
 * out[n_series][SDE_PMOM_STRIDE] = (sum, mean, M2, min, max, NaN count),
 * M2 = the sum of squared deviations from the mean (var = M2 / (paths -
 * ddof)), accumulated in FP64 whatever the data precision; min and max are
 * NaN when a value is.  Replaces process.pmin / pmax / psum / pmean / pvar /
 * pstd (sdepy/infrastructure.py:833-889). */
#define SDE_PMOM_STRIDE 6
SDE_API int32_t sde_process_moments(const void *x, int32_t is_fp32, int32_t on_device,
                                    int64_t n_series, int64_t paths, double *out);

/* The n_t time points at which sde_process_cdf / sde_process_chf read the
 * process: point i reads row lo[i] when hi[i] < 0, else the FP64 value
 * wh[i] * x[hi[i]] + wl[i] * x[lo[i]] rounded to the data precision --
 * scipy.interpolate.interp1d(kind='linear') with constant extrapolation,
 * as process.interp / process.__call__ evaluate it
 * (sdepy/infrastructure.py:544-633); the caller computes the rows and
 * weights. */
typedef struct {
    const int64_t *lo;
    const int64_t *hi;
    const double *wl;
    const double *wh;
    int64_t n_t;
} SdeTimes;

/* out[n_t][n_x][n_vars] = (number of paths whose value is <= xv[j]) /
 * paths, the comparison taken in FP64; NaN values count for no xv, a NaN
 * xv gives 0.  Replaces process.cdf (sdepy/infrastructure.py:1169-1212). */
SDE_API int32_t sde_process_cdf(const void *x, int32_t is_fp32, int32_t on_device,
                                int64_t n_rows, int64_t n_vars, int64_t paths,
                                const SdeTimes *at, const double *xv, int64_t n_x,
                                double *out);

/* out[n_t][n_u][n_vars][2] = the mean over paths of (cos(u_j v), sin(u_j
 * v)) with u_j v rounded to FP64: the real and imaginary parts of
 * exp(1j*u*v).mean(axis=-1).  Replaces process.chf
 * (sdepy/infrastructure.py:1125-1167). */
SDE_API int32_t sde_process_chf(const void *x, int32_t is_fp32, int32_t on_device,
                                int64_t n_rows, int64_t n_vars, int64_t paths,
                                const SdeTimes *at, const double *u, int64_t n_u,
                                double *out);

#ifdef __cplusplus
}
#endif
#endif /* SDEPY_GB300_H */
