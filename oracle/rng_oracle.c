/*
 * ORACLE -- test infrastructure only; the product never links this file.
 *
 * Plain-C restatement of the device-RNG integration of include/sdepy_gb300.h,
 * in FP64, path by path:
 *   - Philox-4x32-10 (Salmon et al., SC'11: multipliers 0xD2511F53,
 *     0xCD9E8D57; Weyl increments 0x9E3779B9, 0xBB67AE85; 10 rounds);
 *   - uniforms u = (x + 0.5) 2^-32, Box-Muller normals
 *     r = sqrt(-2 log u(a)), v = (b >> 9) 2^-22 - 1, (r cos pi v, r sin pi v),
 *     with the logarithm and sin / cos of pi v evaluated by the table-driven
 *     methods named at ln_u01 and sincospi_v (so the FP64 device transform,
 *     which uses the same methods, matches bit for bit);
 *   - Poisson counts by CDF inversion of one uniform word;
 *   - jump sizes of the norm / double_exp / uniform / exp laws;
 *   - the Euler step in sdepy's operation order
 *     (sdepy/integration.py:707-718 with the preset coefficients of
 *     sdepy/integration.py:2066-2747) and sdepy's output transforms.
 * The counter layout is (path, step + offset, group << 8 | call, stream) for
 * normals and Poisson uniforms and (path, step + offset,
 * 0x80000000 | var << 12 | jump, stream) for jump sizes; a user SDE with
 * both dj and dn terms draws dn's Poisson uniform from word x of (path,
 * step + offset, 0x40000000 | var, stream).  Groups of one
 * variable draw one call per two steps: the call of even step k gives its
 * Box-Muller pair's z0 to step k and z1 to step k + 1, and its words z and
 * w are the Poisson uniforms of steps k and k + 1.  Groups of two
 * variables without jumps also draw one call per two steps: words (x, y)
 * give the normals of step k, words (z, w) those of step k + 1.  With
 * SDE_FLAG_ANTITHETIC (paths = 2K) path K + q takes the counters of path q,
 * with opposite normals and the same jumps.
 *
 * Compiled with -ffp-contract=off so that every product and sum rounds as
 * written.  Pinned by the published Philox-4x32-10 known-answer vectors and by
 * scipy.stats.poisson.ppf (tests/test_oracle.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/sdepy_gb300.h"
#include "oracle_tables.h"

void oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int i = 0; i < 10; ++i) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static double u01(uint32_t x) { return ((double)x + 0.5) * 0x1p-32; }
static double vpm1(uint32_t b) { return (double)(b >> 9) * 0x1p-22 - 1.0; }

/*
 * ln u(a), u(a) = (a + 0.5) 2^-32 = (2a + 1) 2^-33, by Tang's table-driven
 * method (ACM TOMS 15(2), 1989): 2a + 1 = 2^e m with m in [0.75, 1.5) taken
 * from the integer's bits, m = c_j (1 + r) with c_j = 0.75 + j/128 the
 * nearest table point, ln u = (e - 33) ln 2 + ln c_j + log1p(r), log1p by
 * its Taylor series to r^7 evaluated with fused multiply-adds.  The tables
 * (oracle_tables.h) are 50-digit mpmath values rounded once.
 */
static double ln_u01(uint32_t a) {
    const uint64_t v = 2ull * a + 1ull;
    const int lz = __builtin_clzll(v);
    const int e = 63 - lz;
    const uint64_t frac = ((v << lz) << 1) >> 12;   /* the 52 bits below the leading one */
    const uint32_t fhi = (uint32_t)(frac >> 32);
    const int upper = fhi >= 0x80000u;              /* 1.f >= 1.5: m = 1.f / 2 */
    const int j = upper ? (int)((fhi + 0x2000u) >> 14) - 32 : (int)((fhi + 0x1000u) >> 13) + 32;
    const int k = e - 33 + upper;
    const uint64_t mbits = ((upper ? 1022ull : 1023ull) << 52) | frac;
    double m;
    memcpy(&m, &mbits, sizeof m);
    const double d = m - ORC_LOG_C[j];
    const double r = d * ORC_LOG_INVC[j];
    const double r2 = r * r;
    double q = 1.0 / 7.0;
    q = fma(q, r, -1.0 / 6.0);
    q = fma(q, r, 1.0 / 5.0);
    q = fma(q, r, -0.25);
    q = fma(q, r, 1.0 / 3.0);
    q = fma(q, r, -0.5);
    const double p = fma(q, r2, r);
    return (ORC_KLN2_HI[k + 35] + ORC_LOG_LNC[j]) + (ORC_KLN2_LO[k + 35] + p);
}

/*
 * sin(pi v), cos(pi v) for v = (b >> 9) 2^-22 - 1: v = n/64 + f, |f| <= 1/128,
 * x = pi f, Taylor series of sin x to x^7 and cos x to x^6, and the angle
 * addition formulas over the tabulated sin(pi n/64), cos(pi n/64).
 */
static void sincospi_v(uint32_t b, double *s, double *c) {
    const int q = (int)(b >> 9);
    const int nn = (q + 0x8000) >> 16;              /* n + 64 */
    const int qd = q - (nn << 16);                  /* f = qd 2^-22 */
    const double x = (double)qd * (0x1p-22 * ORC_PI_HI);
    const double x2 = x * x;
    double ps = -1.0 / 5040.0;
    ps = fma(ps, x2, 1.0 / 120.0);
    ps = fma(ps, x2, -1.0 / 6.0);
    const double sx = fma(x * x2, ps, x);
    double pc = -1.0 / 720.0;
    pc = fma(pc, x2, 1.0 / 24.0);
    pc = fma(pc, x2, -0.5);
    const double cx = fma(x2, pc, 1.0);
    const double S = ORC_SINPI_N[nn], C = ORC_COSPI_N[nn];
    *s = fma(S, cx, C * sx);
    *c = fma(C, cx, -(S * sx));
}

/* Box-Muller pair: r = sqrt(-2 ln u(a)), (r cos pi v, r sin pi v) */
void oracle_normal2(uint32_t a, uint32_t b, double *z0, double *z1) {
    const double r = sqrt(-2.0 * ln_u01(a));
    double s, c;
    sincospi_v(b, &s, &c);
    *z0 = r * c;
    *z1 = r * s;
}

/* the same pair by libm (log, cos, sin of the rounded angle pi v), kept to
 * check the table-driven pair against */
void oracle_normal2_libm(uint32_t a, uint32_t b, double *z0, double *z1) {
    const double r = sqrt(-2.0 * log(u01(a)));
    const double th = M_PI * vpm1(b);
    *z0 = r * cos(th);
    *z1 = r * sin(th);
}

/* the unit exponential -ln u(a) */
double oracle_expo(uint32_t a) { return -ln_u01(a); }

/* smallest k with u(word) <= F(k), F the Poisson(lam) CDF, p0 = exp(-lam) */
int oracle_poisson(uint32_t word, double p0, double lam) {
    const double u = u01(word);
    int k = 0;
    double pk = p0, F = p0;
    while (u > F) {
        ++k;
        pk = (pk * lam) / (double)k;
        F = F + pk;
        if (k >= SDE_MAX_JUMPS_PER_STEP) return -1;
    }
    return k;
}

/* Cholesky-Banachiewicz, zero column on a vanishing pivot */
int oracle_cholesky(const double *C, int M, double *L) {
    for (int i = 0; i < M * M; ++i) L[i] = 0.0;
    for (int i = 0; i < M; ++i)
        for (int j = 0; j <= i; ++j) {
            double s = C[i * M + j];
            for (int k = 0; k < j; ++k) s -= L[i * M + k] * L[j * M + k];
            if (i == j) {
                if (s < -1e-10 * fabs(C[i * M + i]) - 1e-300) return -1;
                L[i * M + i] = s > 1e-14 * fabs(C[i * M + i]) ? sqrt(s) : 0.0;
            } else {
                L[i * M + j] = L[j * M + j] > 0.0 ? s / L[j * M + j] : 0.0;
            }
        }
    return 0;
}

/* A user SDE's coefficients (SdeUserProgram): the program evaluated in FP64
 * with C's operators and libm, numpy's maximum / minimum (NaN-propagating). */
static double np_maxd(double a, double b) { return (a != a) ? a : (b != b) ? b : (a >= b ? a : b); }
static double np_mind(double a, double b) { return (a != a) ? a : (b != b) ? b : (a <= b ? a : b); }

static void user_coefs(const SdeUserProgram *u, const double *xs, double t, const double *p,
                       double out[][SDE_USER_MAX_TERMS]) {
    double r[SDE_USER_MAX_REGS] = {0};
    r[0] = xs[0];
    r[1] = t;
    for (int i = 0; i < 6; ++i) r[2 + i] = p[i];
    for (int e = 1; e < u->n_eq; ++e) r[7 + e] = xs[e];
    for (int i = 0; i < u->n_ops; ++i) {
        const uint32_t op = u->ops[i];
        const int c = op & 0xff, d = (op >> 8) & 0xff, ia = (op >> 16) & 0xff, ib = op >> 24;
        if (c == SDE_UOP_CONST) {
            r[d] = u->consts[ia];
            continue;
        }
        const double va = r[ia], vb = r[ib];
        double v;
        switch (c) {
        case SDE_UOP_ADD: v = va + vb; break;
        case SDE_UOP_SUB: v = va - vb; break;
        case SDE_UOP_MUL: v = va * vb; break;
        case SDE_UOP_DIV: v = va / vb; break;
        case SDE_UOP_NEG: v = -va; break;
        case SDE_UOP_ABS: v = fabs(va); break;
        case SDE_UOP_EXP: v = exp(va); break;
        case SDE_UOP_LOG: v = log(va); break;
        case SDE_UOP_SQRT: v = sqrt(va); break;
        case SDE_UOP_MAX: v = np_maxd(va, vb); break;
        case SDE_UOP_MIN: v = np_mind(va, vb); break;
        case SDE_UOP_SIN: v = sin(va); break;
        case SDE_UOP_COS: v = cos(va); break;
        case SDE_UOP_TAN: v = tan(va); break;
        case SDE_UOP_TANH: v = tanh(va); break;
        case SDE_UOP_POW: v = pow(va, vb); break;
        case SDE_UOP_EXPM1: v = expm1(va); break;
        case SDE_UOP_LOG1P: v = log1p(va); break;
        case SDE_UOP_ARCTAN: v = atan(va); break;
        default: v = va;
        }
        r[d] = v;
    }
    for (int e = 0; e < u->n_eq; ++e)
        for (int j = 0; j < SDE_USER_MAX_TERMS; ++j) out[e][j] = j < u->n_terms ? r[u->term_register[e][j]] : 0.0;
}

static double jump_size(int law, const uint32_t r[4], double a, double b, double pa) {
    double z0, z1;
    switch (law) {
    case SDE_JUMP_NORM:
        oracle_normal2(r[0], r[1], &z0, &z1);
        return a + b * z0;
    case SDE_JUMP_DOUBLE_EXP: {
        const double e = oracle_expo(r[0]);
        const double us = u01(r[2]);
        return (us <= pa) ? a * e : -(b * e);
    }
    case SDE_JUMP_UNIFORM:
        return a + (b - a) * u01(r[2]);
    case SDE_JUMP_EXP:
        return a * oracle_expo(r[0]);
    }
    return 0.0;
}

/*
 * Integrate every path of spec along grid (device-RNG mode) in FP64.
 * xx: [n_rows][n_out_vars][paths] doubles (rows not on the grid untouched);
 * neg / jcnt / rowj as in SdeOut (may be NULL).  Returns 0, or -1 on a bad
 * argument / jump cap.
 */
int oracle_run(const SdeSpec *s, const SdeGrid *g, double *xx, int32_t n_rows,
               int32_t *neg, int32_t *jcnt, int64_t *rowj) {
    const int M = s->group_size, G = s->groups, W = G * M;
    const int64_t paths = s->paths;
    const int n_steps = g->n_pts - 1;
    /* a user program's jump terms: bit 0 dj, bit 1 dn */
    int ujs = 0;
    if (s->model == SDE_MODEL_USER)
        for (int i = 0; i < s->program->n_terms; ++i) {
            if (s->program->term_source[i] == SDE_SRC_DJ) ujs |= 1;
            if (s->program->term_source[i] == SDE_SRC_DN) ujs |= 2;
        }
    const int user = s->model == SDE_MODEL_USER;
    const int jumps = user ? ujs != 0 : s->jump_law != SDE_JUMP_NONE;
    int opg;
    switch (s->out_mode) {
    case SDE_OUT_SUM: opg = 1; break;
    case SDE_OUT_HESTON_X: opg = M / 2; break;
    default: opg = M;
    }
    const int64_t n_out = (int64_t)G * opg;
    double L[SDE_MAX_GROUP * SDE_MAX_GROUP];
    if (s->corr && oracle_cholesky(s->corr, M, L)) return -1;
    /* time-dependent correlation: each step's factor (the grid's corr_t,
     * the step's matrix at its midpoint) */
    double *Lt = NULL;
    if (g->corr_t && n_steps > 0) {
        Lt = malloc(sizeof(double) * (size_t)n_steps * M * M);
        for (int k = 0; k < n_steps; ++k)
            if (oracle_cholesky(g->corr_t + (size_t)k * M * M, M, Lt + (size_t)k * M * M)) {
                free(Lt);
                return -1;
            }
    }
    const int has_corr = s->corr != NULL || Lt != NULL;
    const uint32_t key[2] = {(uint32_t)s->seed, (uint32_t)(s->seed >> 32)};
    double sgn = 1.0;
    if (n_steps > 0 && g->tt[1] < g->tt[0]) sgn = -1.0;
    double *dtv = malloc(sizeof(double) * (n_steps + 1));
    double *sqv = malloc(sizeof(double) * (n_steps + 1));
    for (int k = 0; k < n_steps; ++k) {
        dtv[k] = g->tt[k + 1] - g->tt[k];
        sqv[k] = sqrt(fabs(dtv[k]));
    }
    if (rowj) memset(rowj, 0, sizeof(int64_t) * n_rows);
    const double *prm = s->params;
    int rc = 0;
    const int anti = (s->flags & SDE_FLAG_ANTITHETIC) != 0;
    for (int64_t p = 0; p < paths && !rc; ++p) {
        /* the counters' path word, and the sign of the normals */
        const int64_t pc = ((anti && p >= paths / 2) ? p - paths / 2 : p) + s->path_offset;
        const double zsign = (anti && p >= paths / 2) ? -1.0 : 1.0;
        for (int gi = 0; gi < G && !rc; ++gi) {
            double st[SDE_MAX_GROUP], z[SDE_MAX_GROUP + 1], dW[SDE_MAX_GROUP], dJ[SDE_MAX_GROUP], dN[SDE_MAX_GROUP];
            int negc[SDE_MAX_GROUP] = {0}, jc[SDE_MAX_GROUP] = {0};
            int64_t row_jc = 0;
            double pz0 = 0.0, pz1 = 0.0;   /* one-variable groups: the even step's pair */
            uint32_t pw0 = 0, pw1 = 0;
            double pz[4] = {0.0, 0.0, 0.0, 0.0};   /* two-variable groups without jumps */
            for (int m = 0; m < M; ++m) st[m] = s->x0[gi * M + m];
            for (int k = -1; k < n_steps; ++k) {
                if (k >= 0) {
                    const double dt = dtv[k], sq = sqv[k];
                    /* coefficients of this step (slots 0..2; the Poisson
                     * intensity of jump models is slot 2) */
                    const double *pp = g->params_t ? g->params_t + (size_t)k * SDE_MAX_PARAMS * W : prm;
                    const uint32_t c1 = (uint32_t)k + g->step_offset;
                    const int P = (M + 1) / 2;
                    const int U = 2 * P + (jumps ? M : 0);
                    const int NC = (U + 3) / 4;
                    uint32_t u[4 * ((2 * SDE_MAX_GROUP + 2 + 3) / 4) + 4];
                    if (M == 1) {
                        if ((k & 1) == 0) {
                            const uint32_t ctr[4] = {(uint32_t)pc, c1, (uint32_t)gi << 8, s->stream};
                            uint32_t r[4];
                            oracle_philox(ctr, key, r);
                            oracle_normal2(r[0], r[1], &pz0, &pz1);
                            pw0 = r[2];
                            pw1 = r[3];
                        }
                        z[0] = (k & 1) ? pz1 : pz0;
                        u[2] = (k & 1) ? pw1 : pw0;   /* the Poisson word, index 2P + m */
                    } else if (M == 2 && !jumps) {
                        if ((k & 1) == 0) {
                            const uint32_t ctr[4] = {(uint32_t)pc, c1, (uint32_t)gi << 8, s->stream};
                            uint32_t r[4];
                            oracle_philox(ctr, key, r);
                            oracle_normal2(r[0], r[1], &pz[0], &pz[1]);
                            oracle_normal2(r[2], r[3], &pz[2], &pz[3]);
                        }
                        z[0] = (k & 1) ? pz[2] : pz[0];
                        z[1] = (k & 1) ? pz[3] : pz[1];
                    } else {
                        for (int c = 0; c < NC; ++c) {
                            const uint32_t ctr[4] = {(uint32_t)pc, c1, ((uint32_t)gi << 8) | (uint32_t)c, s->stream};
                            oracle_philox(ctr, key, &u[4 * c]);
                        }
                        for (int q = 0; q < P; ++q)
                            oracle_normal2(u[2 * q], u[2 * q + 1], &z[2 * q], &z[2 * q + 1]);
                    }
                    if (zsign < 0)   /* the antithetic path */
                        for (int m = 0; m < M; ++m) z[m] = -z[m];
                    const double *Lk = Lt ? Lt + (size_t)k * M * M : L;
                    for (int m = 0; m < M; ++m) {
                        if (has_corr) {
                            double acc = Lk[m * M + 0] * z[0];
                            for (int j = 1; j <= m; ++j) acc = acc + Lk[m * M + j] * z[j];
                            dW[m] = acc * sq;
                        } else {
                            dW[m] = z[m] * sq;
                        }
                        dJ[m] = 0.0;
                        dN[m] = 0.0;
                    }
                    if (jumps && user) {
                        /* a user SDE: dj from the Poisson word and as many jump
                         * sizes; dn from the same count, or with a dj term too,
                         * from its own word */
                        const double *jp = s->program->jump_params;
                        for (int m = 0; m < M; ++m) {
                            const int w = gi * M + m;
                            const double lamr = g->lam_t ? g->lam_t[(size_t)k * W + w] : jp[w];
                            const double lam = fabs(dt) * lamr;
                            const double p0 = exp(-lam);
                            uint32_t word = u[2 * P + m];
                            int cnt = u01(word) > p0 ? oracle_poisson(word, p0, lam) : 0;
                            if (cnt < 0) { rc = -1; break; }
                            if (ujs & 1) {
                                double S = 0.0;
                                for (int j = 0; j < cnt; ++j) {
                                    const uint32_t ctr[4] = {(uint32_t)pc, c1,
                                                             0x80000000u | ((uint32_t)w << 12) | (uint32_t)j, s->stream};
                                    uint32_t r[4];
                                    oracle_philox(ctr, key, r);
                                    const double y = jump_size(s->jump_law, r, jp[W + w], jp[2 * W + w], jp[3 * W + w]);
                                    S = (j == 0) ? y : S + y;
                                }
                                if (cnt) dJ[m] = sgn * S;
                                if (ujs & 2) {
                                    const uint32_t ctr[4] = {(uint32_t)pc, c1, 0x40000000u | (uint32_t)w, s->stream};
                                    uint32_t r[4];
                                    oracle_philox(ctr, key, r);
                                    word = r[0];
                                    cnt = u01(word) > p0 ? oracle_poisson(word, p0, lam) : 0;
                                    if (cnt < 0) { rc = -1; break; }
                                }
                            }
                            if ((ujs & 2) && cnt) dN[m] = sgn * (double)cnt;
                        }
                    } else if (jumps) {
                        for (int m = 0; m < M; ++m) {
                            const int w = gi * M + m;
                            const double lam = fabs(dt) * pp[2 * W + w];
                            const double p0 = exp(-lam);
                            const uint32_t word = u[2 * P + m];
                            if (u01(word) > p0) {
                                const int cnt = oracle_poisson(word, p0, lam);
                                if (cnt < 0) { rc = -1; break; }
                                double S = 0.0;
                                for (int j = 0; j < cnt; ++j) {
                                    const uint32_t ctr[4] = {(uint32_t)pc, c1,
                                                             0x80000000u | ((uint32_t)w << 12) | (uint32_t)j, s->stream};
                                    uint32_t r[4];
                                    oracle_philox(ctr, key, r);
                                    const double y = jump_size(s->jump_law, r, prm[3 * W + w], prm[4 * W + w], prm[5 * W + w]);
                                    S = (j == 0) ? y : S + y;
                                }
                                dJ[m] = sgn * S;
                                jc[m] += sgn < 0 ? -cnt : cnt;
                                row_jc += cnt;
                            }
                        }
                    }
                    if (s->model == SDE_MODEL_LINEAR) {
                        for (int m = 0; m < M; ++m) {
                            const int w = gi * M + m;
                            double inc = pp[0 * W + w] * dt + pp[1 * W + w] * dW[m];
                            if (jumps) inc = inc + dJ[m];
                            st[m] = st[m] + inc;
                        }
                    } else if (s->model == SDE_MODEL_OU) {
                        for (int m = 0; m < M; ++m) {
                            const int w = gi * M + m;
                            const double drift = pp[0 * W + w] * (pp[1 * W + w] - st[m]);
                            st[m] = st[m] + (drift * dt + pp[2 * W + w] * dW[m]);
                        }
                    } else if (s->model == SDE_MODEL_USER) {   /* sdepy/integration.py:707-718, 1711-1783 */
                        /* per component h: the states of the q equations
                         * (equation e's component h at e * nc + h) */
                        const int q = s->program->n_eq, nc = M / q;
                        double nx[SDE_MAX_GROUP];
                        for (int h = 0; h < nc; ++h) {
                            double pv[6], xs[SDE_USER_MAX_EQ], A[SDE_USER_MAX_EQ][SDE_USER_MAX_TERMS];
                            for (int i = 0; i < 6; ++i) pv[i] = pp[i * W + gi * M + h];
                            for (int e = 0; e < q; ++e) xs[e] = st[e * nc + h];
                            user_coefs(s->program, xs, g->tt[k], pv, A);
                            for (int e = 0; e < q; ++e) {
                                const int m = e * nc + h;
                                double sum = 0.0;
                                for (int i = 0; i < s->program->n_terms; ++i) {
                                    const int src = s->program->term_source[i];
                                    const double dz = src == SDE_SRC_DT   ? dt
                                                      : src == SDE_SRC_DW ? dW[m]
                                                      : src == SDE_SRC_DJ ? dJ[m]
                                                                          : dN[m];
                                    const double term = A[e][i] * dz;
                                    sum = i == 0 ? term : sum + term;
                                }
                                nx[m] = st[m] + sum;
                            }
                        }
                        for (int m = 0; m < M; ++m) st[m] = nx[m];
                    } else if (s->model == SDE_MODEL_CIR) {   /* sdepy/integration.py:2350-2354 */
                        for (int m = 0; m < M; ++m) {
                            const int w = gi * M + m;
                            const double xp = st[m] > 0.0 ? st[m] : 0.0;
                            const double drift = pp[0 * W + w] * (pp[1 * W + w] - xp);
                            const double vol = pp[2 * W + w] * sqrt(xp);
                            st[m] = st[m] + (drift * dt + vol * dW[m]);
                        }
                    } else {
                        const int h = M / 2;
                        double nx[SDE_MAX_GROUP];
                        for (int i = 0; i < h; ++i) {
                            const int wx = gi * M + i, wy = gi * M + h + i;
                            const double y = st[h + i];
                            if (y < 0.0) negc[i] += 1;
                            const double yp = y > 0.0 ? y : 0.0;
                            const double sqy = sqrt(yp);
                            const double mu = pp[0 * W + wx], sg = pp[1 * W + wx];
                            const double adt = mu - ((sg * sg) * yp) * 0.5;
                            const double adw = sg * sqy;
                            nx[i] = st[i] + (adt * dt + adw * dW[i]);
                            const double kk = pp[0 * W + wy], th = pp[1 * W + wy], xi = pp[2 * W + wy];
                            const double bdt = kk * (th - yp);
                            const double bdw = xi * sqy;
                            nx[h + i] = y + (bdt * dt + bdw * dW[h + i]);
                        }
                        for (int m = 0; m < M; ++m) st[m] = nx[m];
                    }
                }
                const int row = g->out_row[k + 1];
                if (row < 0) continue;
                double ov[SDE_MAX_GROUP];
                int no = M;
                switch (s->out_mode) {
                case SDE_OUT_EXP:
                    for (int m = 0; m < M; ++m) ov[m] = exp(st[m]);
                    break;
                case SDE_OUT_SUM: {
                    double a = st[0];
                    for (int m = 1; m < M; ++m) a = a + st[m];
                    ov[0] = a;
                    no = 1;
                    break;
                }
                case SDE_OUT_HESTON_X:
                    for (int m = 0; m < M / 2; ++m) ov[m] = exp(st[m]);
                    no = M / 2;
                    break;
                case SDE_OUT_HESTON_XY:
                    for (int m = 0; m < M; ++m) ov[m] = m < M / 2 ? exp(st[m]) : st[m];
                    break;
                default:
                    for (int m = 0; m < M; ++m) ov[m] = st[m];
                }
                for (int m = 0; m < no; ++m)
                    xx[((int64_t)row * n_out + (int64_t)gi * opg + m) * paths + p] = ov[m];
                if (rowj) rowj[row] += row_jc;
                row_jc = 0;
            }
            if (neg && s->model == SDE_MODEL_HESTON)
                for (int i = 0; i < M / 2; ++i) neg[((int64_t)gi * (M / 2) + i) * paths + p] = negc[i];
            if (jcnt && jumps)
                for (int m = 0; m < M; ++m) jcnt[((int64_t)gi * M + m) * paths + p] = jc[m];
        }
    }
    free(dtv);
    free(sqv);
    free(Lt);
    return rc;
}

/*
 * Adjoint of a user SDE (single equation, dt / dw terms; sde_adjoint of
 * include/sdepy_gb300.h): the gradient of
 *   L = mean_paths sum_states f(X(T)),  f(X) = w0 X + sum_s w_s max(X - K_s, 0),
 * X the stored output (the state, or its exp for SDE_OUT_EXP), with respect
 * to x0 (slot 0 of each state) and the program's parameters p_j (slot
 * 1 + j); grad is [groups*M][8], value = L.  Each path's states and Wiener
 * increments are recomputed from the same counters as oracle_run, then
 * x_bar is carried backwards: x_bar <- x_bar (1 + sum_i dA_i/dx dZ_i),
 * g_j += x_bar sum_i dA_i/dp_j dZ_i.  The tangents of the program follow
 * the chain rule per instruction: maximum / minimum / abs take the selected
 * branch, sqrt has derivative 0 at 0, a ** b adds v log a only where a > 0.
 * Returns 0, or -1 for another model or a bad argument.
 */
#define UTAN 7
static void user_tan(const SdeUserProgram *u, double x, double t, const double *p, double A[SDE_USER_MAX_TERMS],
                     double dA[SDE_USER_MAX_TERMS][UTAN]) {
    double r[SDE_USER_MAX_REGS] = {0}, d[SDE_USER_MAX_REGS][UTAN];
    memset(d, 0, sizeof d);
    r[0] = x;
    r[1] = t;
    d[0][0] = 1.0;
    for (int i = 0; i < 6; ++i) {
        r[2 + i] = p[i];
        d[2 + i][1 + i] = 1.0;
    }
    for (int i = 0; i < u->n_ops; ++i) {
        const uint32_t op = u->ops[i];
        const int c = op & 0xff, dst = (op >> 8) & 0xff, ia = (op >> 16) & 0xff, ib = op >> 24;
        if (c == SDE_UOP_CONST) {
            r[dst] = u->consts[ia];
            for (int j = 0; j < UTAN; ++j) d[dst][j] = 0.0;
            continue;
        }
        const double va = r[ia], vb = r[ib];
        double v, da = 0.0, db = 0.0;
        switch (c) {
        case SDE_UOP_ADD: v = va + vb; da = 1.0; db = 1.0; break;
        case SDE_UOP_SUB: v = va - vb; da = 1.0; db = -1.0; break;
        case SDE_UOP_MUL: v = va * vb; da = vb; db = va; break;
        case SDE_UOP_DIV: v = va / vb; da = 1.0 / vb; db = -v / vb; break;
        case SDE_UOP_NEG: v = -va; da = -1.0; break;
        case SDE_UOP_ABS: v = fabs(va); da = va < 0.0 ? -1.0 : 1.0; break;
        case SDE_UOP_EXP: v = exp(va); da = v; break;
        case SDE_UOP_LOG: v = log(va); da = 1.0 / va; break;
        case SDE_UOP_SQRT: v = sqrt(va); da = v > 0.0 ? 0.5 / v : 0.0; break;
        case SDE_UOP_MAX: v = np_maxd(va, vb); if (va >= vb) da = 1.0; else db = 1.0; break;
        case SDE_UOP_MIN: v = np_mind(va, vb); if (va <= vb) da = 1.0; else db = 1.0; break;
        case SDE_UOP_SIN: v = sin(va); da = cos(va); break;
        case SDE_UOP_COS: v = cos(va); da = -sin(va); break;
        case SDE_UOP_TAN: v = tan(va); da = 1.0 + v * v; break;
        case SDE_UOP_TANH: v = tanh(va); da = 1.0 - v * v; break;
        case SDE_UOP_POW:
            v = pow(va, vb);
            da = vb * pow(va, vb - 1.0);
            db = va > 0.0 ? v * log(va) : 0.0;
            break;
        case SDE_UOP_EXPM1: v = expm1(va); da = v + 1.0; break;
        case SDE_UOP_LOG1P: v = log1p(va); da = 1.0 / (1.0 + va); break;
        case SDE_UOP_ARCTAN: v = atan(va); da = 1.0 / (1.0 + va * va); break;
        default: v = va; da = 1.0;
        }
        double nd[UTAN];
        for (int j = 0; j < UTAN; ++j) {
            const double ta = d[ia][j], tb = d[ib][j];
            double sj = ta != 0.0 ? da * ta : 0.0;
            if (tb != 0.0 && db != 0.0) sj = sj + db * tb;
            nd[j] = sj;
        }
        r[dst] = v;
        for (int j = 0; j < UTAN; ++j) d[dst][j] = nd[j];
    }
    for (int i = 0; i < SDE_USER_MAX_TERMS; ++i) {
        const int reg = i < u->n_terms ? u->term_register[0][i] : 0;
        A[i] = i < u->n_terms ? r[reg] : 0.0;
        for (int j = 0; j < UTAN; ++j) dA[i][j] = i < u->n_terms ? d[reg][j] : 0.0;
    }
}

int oracle_adjoint_user(const SdeSpec *s, const SdeGrid *g, double mean_weight, int n_strikes,
                        const double *strikes, const double *weights, double *grad, double *value) {
    if (!s || !g || s->model != SDE_MODEL_USER || !s->program || s->program->n_eq != 1 || g->n_pts < 2 ||
        n_strikes < 0 || n_strikes > SDE_MAX_STRIKES)
        return -1;
    const SdeUserProgram *u = s->program;
    for (int i = 0; i < u->n_terms; ++i)
        if (u->term_source[i] != SDE_SRC_DT && u->term_source[i] != SDE_SRC_DW) return -1;
    const int M = s->group_size, G = s->groups, W = G * M;
    const int64_t paths = s->paths;
    const int n_steps = g->n_pts - 1;
    double L[SDE_MAX_GROUP * SDE_MAX_GROUP];
    if (s->corr && oracle_cholesky(s->corr, M, L)) return -1;
    const uint32_t key[2] = {(uint32_t)s->seed, (uint32_t)(s->seed >> 32)};
    double *xk = malloc(sizeof(double) * (size_t)(n_steps + 1) * M);
    double *wk = malloc(sizeof(double) * (size_t)n_steps * M);
    memset(grad, 0, sizeof(double) * (size_t)W * 8);
    double val = 0.0;
    const int P = (M + 1) / 2, NC = (2 * P + 3) / 4;
    for (int64_t p = 0; p < paths; ++p) {
        for (int gi = 0; gi < G; ++gi) {
            double st[SDE_MAX_GROUP], z[SDE_MAX_GROUP + 1], pz0 = 0.0, pz1 = 0.0, pz[4] = {0.0, 0.0, 0.0, 0.0};
            for (int m = 0; m < M; ++m) st[m] = s->x0[gi * M + m];
            /* forward: the states at each step's start and the increments,
             * drawn as oracle_run draws them */
            for (int k = 0; k < n_steps; ++k) {
                const double dt = g->tt[k + 1] - g->tt[k], sq = sqrt(fabs(dt));
                const uint32_t c1 = (uint32_t)k + g->step_offset;
                uint32_t uw[4 * ((2 * SDE_MAX_GROUP + 3) / 4) + 4];
                if (M == 1) {
                    if ((k & 1) == 0) {
                        const uint32_t ctr[4] = {(uint32_t)p + s->path_offset, c1, (uint32_t)gi << 8, s->stream};
                        uint32_t r[4];
                        oracle_philox(ctr, key, r);
                        oracle_normal2(r[0], r[1], &pz0, &pz1);
                    }
                    z[0] = (k & 1) ? pz1 : pz0;
                } else if (M == 2) {
                    if ((k & 1) == 0) {
                        const uint32_t ctr[4] = {(uint32_t)p + s->path_offset, c1, (uint32_t)gi << 8, s->stream};
                        uint32_t r[4];
                        oracle_philox(ctr, key, r);
                        oracle_normal2(r[0], r[1], &pz[0], &pz[1]);
                        oracle_normal2(r[2], r[3], &pz[2], &pz[3]);
                    }
                    z[0] = (k & 1) ? pz[2] : pz[0];
                    z[1] = (k & 1) ? pz[3] : pz[1];
                } else {
                    for (int c = 0; c < NC; ++c) {
                        const uint32_t ctr[4] = {(uint32_t)p + s->path_offset, c1, ((uint32_t)gi << 8) | (uint32_t)c, s->stream};
                        oracle_philox(ctr, key, &uw[4 * c]);
                    }
                    for (int q = 0; q < P; ++q) oracle_normal2(uw[2 * q], uw[2 * q + 1], &z[2 * q], &z[2 * q + 1]);
                }
                for (int m = 0; m < M; ++m) {
                    double dWm;
                    if (s->corr) {
                        double acc = L[m * M + 0] * z[0];
                        for (int j = 1; j <= m; ++j) acc = acc + L[m * M + j] * z[j];
                        dWm = acc * sq;
                    } else {
                        dWm = z[m] * sq;
                    }
                    const int w = gi * M + m;
                    double pv[6], A[SDE_USER_MAX_TERMS][SDE_USER_MAX_TERMS];
                    for (int i = 0; i < 6; ++i) pv[i] = s->params[i * W + w];
                    xk[(size_t)k * M + m] = st[m];
                    wk[(size_t)k * M + m] = dWm;
                    user_coefs(u, &st[m], g->tt[k], pv, A);
                    double sum = 0.0;
                    for (int i = 0; i < u->n_terms; ++i) {
                        const double term = A[0][i] * (u->term_source[i] == SDE_SRC_DT ? dt : dWm);
                        sum = i == 0 ? term : sum + term;
                    }
                    st[m] = st[m] + sum;
                }
            }
            /* the functional and its derivative in the final states */
            for (int m = 0; m < M; ++m) {
                const int w = gi * M + m;
                const double X = s->out_mode == SDE_OUT_EXP ? exp(st[m]) : st[m];
                double f = mean_weight * X, fp = mean_weight;
                for (int i = 0; i < n_strikes; ++i) {
                    f += weights[i] * (X > strikes[i] ? X - strikes[i] : 0.0);
                    if (X > strikes[i]) fp += weights[i];
                }
                val += f;
                double xb = fp * (s->out_mode == SDE_OUT_EXP ? X : 1.0);
                double pv[6];
                for (int i = 0; i < 6; ++i) pv[i] = s->params[i * W + w];
                for (int k = n_steps - 1; k >= 0; --k) {
                    const double dt = g->tt[k + 1] - g->tt[k];
                    double A[SDE_USER_MAX_TERMS], dA[SDE_USER_MAX_TERMS][UTAN], gx = 0.0, gp[6] = {0};
                    user_tan(u, xk[(size_t)k * M + m], g->tt[k], pv, A, dA);
                    for (int i = 0; i < u->n_terms; ++i) {
                        const double dz = u->term_source[i] == SDE_SRC_DT ? dt : wk[(size_t)k * M + m];
                        gx += dA[i][0] * dz;
                        for (int j = 0; j < 6; ++j) gp[j] += dA[i][1 + j] * dz;
                    }
                    for (int j = 0; j < 6; ++j) grad[(size_t)w * 8 + 1 + j] += xb * gp[j];
                    xb = xb * (1.0 + gx);
                }
                grad[(size_t)w * 8] += xb;
            }
        }
    }
    for (int i = 0; i < W * 8; ++i) grad[i] /= (double)paths;
    if (value) *value = val / (double)paths;
    free(xk);
    free(wk);
    return 0;
}
