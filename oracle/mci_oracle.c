/*
 * mci_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY) for the GB300 Monte
 * Carlo integrator.  Plain C restatement of the reference's hot path; every
 * function cites the reference file:line it follows.  Compile with
 * -ffp-contract=off so that no multiply-add is fused: the reference is built
 * for baseline x86-64 (no FMA) and the device FP64 path avoids contraction too.
 *
 * Third-party algorithms restated here (the reference uses them through
 * libstdc++ of GCC 13.3; they are not part of the reference sources):
 *   - std::mt19937_64: Matsumoto & Nishimura's 64-bit Mersenne Twister
 *     (ACM TOMACS 10(4) 2000), seeding by the C++11 [rand.eng.mers] recurrence.
 *   - std::generate_canonical<double,53>: one 64-bit word w -> (double)w * 2^-64,
 *     clamped below 1.
 *   - std::uniform_real_distribution(a,b): canonical*(b-a)+a.
 *   - std::normal_distribution: Marsaglia's polar method with one cached value
 *     held by the distribution object.
 *   - std::uniform_int_distribution on a 64-bit engine: Lemire's
 *     multiply-and-reject downscaling with a 128-bit product (arXiv:1805.10941).
 *   - Philox4x32-10: Salmon et al., SC'11 ("Parallel random numbers: as easy as
 *     1, 2, 3"), used only to check the device generator.
 */
#define _GNU_SOURCE
#include "mci_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* error reporting                                                     */
/* ------------------------------------------------------------------ */
static char g_err[512];
static int fail(int code, const char *msg)
{
    snprintf(g_err, sizeof(g_err), "%s", msg);
    return code;
}
const char *orc_last_error(void) { return g_err; }

/* ------------------------------------------------------------------ */
/* mt19937_64                                                          */
/* ------------------------------------------------------------------ */
#define MT_N 312
#define MT_M 156
typedef struct { uint64_t x[MT_N]; int p; } mt64;

static void mt_seed(mt64 *m, uint64_t s)
{
    m->x[0] = s;
    for (int i = 1; i < MT_N; ++i) {
        uint64_t v = m->x[i - 1];
        v ^= v >> 62;
        m->x[i] = 6364136223846793005ULL * v + (uint64_t)i;
    }
    m->p = MT_N;
}

static void mt_twist(mt64 *m)
{
    const uint64_t UP = 0xFFFFFFFF80000000ULL, LO = 0x7FFFFFFFULL, A = 0xB5026F5AA96619E9ULL;
    int k;
    for (k = 0; k < MT_N - MT_M; ++k) {
        uint64_t y = (m->x[k] & UP) | (m->x[k + 1] & LO);
        m->x[k] = m->x[k + MT_M] ^ (y >> 1) ^ ((y & 1ULL) ? A : 0ULL);
    }
    for (; k < MT_N - 1; ++k) {
        uint64_t y = (m->x[k] & UP) | (m->x[k + 1] & LO);
        m->x[k] = m->x[k + (MT_M - MT_N)] ^ (y >> 1) ^ ((y & 1ULL) ? A : 0ULL);
    }
    uint64_t y = (m->x[MT_N - 1] & UP) | (m->x[0] & LO);
    m->x[MT_N - 1] = m->x[MT_M - 1] ^ (y >> 1) ^ ((y & 1ULL) ? A : 0ULL);
    m->p = 0;
}

static uint64_t mt_next(mt64 *m)
{
    if (m->p >= MT_N) { mt_twist(m); }
    uint64_t z = m->x[m->p++];
    z ^= (z >> 29) & 0x5555555555555555ULL;
    z ^= (z << 17) & 0x71D67FFFEDA60000ULL;
    z ^= (z << 37) & 0xFFF7EEE000000000ULL;
    z ^= z >> 43;
    return z;
}

static double canonical(mt64 *m)
{
    double r = (double)mt_next(m) / 18446744073709551616.0; /* 2^64, exact scaling */
    if (r >= 1.0) { r = nextafter(1.0, 0.0); }
    return r;
}

typedef struct { int avail; double saved; } normstate;

static double polar_normal(mt64 *m, normstate *st)
{
    if (st->avail) {
        st->avail = 0;
        return st->saved;
    }
    double x, y, r2;
    do {
        x = 2.0 * canonical(m) - 1.0;
        y = 2.0 * canonical(m) - 1.0;
        r2 = x * x + y * y;
    } while (r2 > 1.0 || r2 == 0.0);
    const double mult = sqrt(-2.0 * log(r2) / r2);
    st->saved = x * mult;
    st->avail = 1;
    return y * mult;
}

static uint64_t lemire_int(mt64 *m, uint64_t range /* number of values */)
{
    unsigned __int128 prod = (unsigned __int128)mt_next(m) * range;
    uint64_t low = (uint64_t)prod;
    if (low < range) {
        const uint64_t thresh = (0ULL - range) % range;
        while (low < thresh) {
            prod = (unsigned __int128)mt_next(m) * range;
            low = (uint64_t)prod;
        }
    }
    return (uint64_t)(prod >> 64);
}

void orc_mt64_stream(uint64_t seed, int64_t n, uint64_t *out)
{
    mt64 m;
    mt_seed(&m, seed);
    for (int64_t i = 0; i < n; ++i) { out[i] = mt_next(&m); }
}

void orc_canonical_stream(uint64_t seed, int64_t n, double *out)
{
    mt64 m;
    mt_seed(&m, seed);
    for (int64_t i = 0; i < n; ++i) { out[i] = canonical(&m); }
}

void orc_normal_stream(uint64_t seed, int64_t n, double *out)
{
    mt64 m;
    normstate st = {0, 0.};
    mt_seed(&m, seed);
    for (int64_t i = 0; i < n; ++i) { out[i] = polar_normal(&m, &st); }
}

void orc_uniform_int_stream(uint64_t seed, int64_t n, int64_t nvals, int64_t *out)
{
    mt64 m;
    mt_seed(&m, seed);
    for (int64_t i = 0; i < n; ++i) { out[i] = (int64_t)lemire_int(&m, (uint64_t)nvals); }
}

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n1 = (uint32_t)p1;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        const uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* ------------------------------------------------------------------ */
/* draw source: the engine (optionally recording) or a replay tape     */
/* ------------------------------------------------------------------ */
typedef struct {
    mt64 mt;
    const double *tape;
    int64_t tape_len, tape_pos;
    int recording;
    double *rec;
    int64_t rec_len, rec_cap;
    int exhausted;
    /* Philox source (orc_set_philox): the draws of the device kernels' counter layout,
     * one step's draws generated at its first draw, in the order this oracle consumes them */
    int philox;              /* 0 off, ORC_PHILOX_FLOAT or ORC_PHILOX_DOUBLE */
    uint32_t pkey[2], pchain;
    uint64_t pctr;           /* step counter of the chain (the device's ctr) */
    int pmove, psrrd, pveclen, pndim;
    int pms_nsteps, pms_srrd, pms_veclen; /* MultiStepMove: sub-steps and their vector move */
    double *pbuf;            /* [(pms_nsteps + 1) * (pndim + 2)] */
    int pbuf_n, pbuf_pos;
} drawsrc;

/* one Philox4x32-10 block of the device kernels' counter layout:
 * (step lo, step hi, chain, substep << 16 | tag << 12 | block) */
static void philox_block(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, const uint32_t key[2], uint32_t out[4])
{
    const uint32_t ctr[4] = {c0, c1, c2, c3};
    orc_philox4x32_10(ctr, key, out);
}

#define ORC_TAG_MOVE 0u
#define ORC_TAG_ACCEPT 1u
#define ORC_TAG_INDEX 2u

/* Box-Muller of the float kernels' draw layout (mcig_common.cuh box_muller_f), in double:
 * u = ((w0 >> 8) + 1/2) 2^-24 in (0, 1), angle 2 pi ((w1 >> 8) 2^-24 - 1/2) */
static void orc_bm_float(uint32_t w0, uint32_t w1, double *z0, double *z1)
{
    const double u = ((double)(w0 >> 8) + 0.5) * 0x1p-24;
    const double r = sqrt(-2.0 * log(u));
    const double th = 6.283185307179586 * ((double)(w1 >> 8) * 0x1p-24 - 0.5);
    *z0 = r * cos(th);
    *z1 = r * sin(th);
}

static double orc_u01_d(uint32_t hi, uint32_t lo)
{
    return (double)((((uint64_t)hi) << 21) | (uint64_t)(lo >> 11)) * 0x1p-53;
}

/* the move draws of Philox block b of sub-step `sub` (float layout: 4 coordinates, double
 * layout: 2) with distribution srrd */
static void philox_move_block(const drawsrc *d, uint32_t sub, int srrd, uint32_t b, double *v)
{
    uint32_t q[4];
    philox_block((uint32_t)d->pctr, (uint32_t)(d->pctr >> 32), d->pchain, (sub << 16) | (ORC_TAG_MOVE << 12) | b, d->pkey, q);
    const int gauss = srrd == MCIG_SRRD_GAUSSIAN;
    if (d->philox == 1) {
        if (gauss) {
            orc_bm_float(q[0], q[1], &v[0], &v[1]);
            orc_bm_float(q[2], q[3], &v[2], &v[3]);
        } else {
            for (int k = 0; k < 4; ++k) { v[k] = (double)(q[k] >> 8) * 0x1p-24 * 2.0 - 1.0; }
        }
    } else if (gauss) { /* box_muller_d: u = 1 - u01(a, b) in (0, 1], angle 2 pi u01(c, d) */
        const double u = 1.0 - orc_u01_d(q[0], q[1]);
        const double r = sqrt(-2.0 * log(u));
        const double a = 6.283185307179586 * orc_u01_d(q[2], q[3]);
        v[0] = r * cos(a);
        v[1] = r * sin(a);
    } else {
        v[0] = orc_u01_d(q[0], q[1]) * 2.0 - 1.0;
        v[1] = orc_u01_d(q[2], q[3]) * 2.0 - 1.0;
    }
}

/* the acceptance uniform of sub-step `sub` (0: the step itself) */
static double philox_accept(const drawsrc *d, uint32_t sub)
{
    uint32_t q[4];
    philox_block((uint32_t)d->pctr, (uint32_t)(d->pctr >> 32), d->pchain, (sub << 16) | (ORC_TAG_ACCEPT << 12), d->pkey, q);
    return (d->philox == 1) ? (double)((q[0] >> 8) + 1u) * 0x1p-24 /* (0, 1] */ : orc_u01_d(q[0], q[1]);
}

/* the draws of one vector move of sub-step `sub` at position n of the buffer: the index
 * (32-bit multiply-shift of word a of the index block), the vector's draws; returns n */
static int philox_vec(drawsrc *d, uint32_t sub, int srrd, int veclen, int n)
{
    const int cpb = (d->philox == 1) ? 4 : 2;
    uint32_t q[4];
    const uint32_t nvecs = (uint32_t)(d->pndim / veclen);
    philox_block((uint32_t)d->pctr, (uint32_t)(d->pctr >> 32), d->pchain, (sub << 16) | (ORC_TAG_INDEX << 12), d->pkey, q);
    const int vidx = (int)(((uint64_t)q[0] * nvecs) >> 32);
    d->pbuf[n++] = (double)vidx;
    const int lo = vidx * veclen;
    double v[4];
    for (int i = lo; i < lo + veclen; ++i) {
        if (i == lo || i % cpb == 0) { philox_move_block(d, sub, srrd, (uint32_t)(i / cpb), v); }
        d->pbuf[n++] = v[i % cpb];
    }
    return n;
}

/* the draws of one step in this oracle's consumption order: all-coordinate move: the
 * coordinates' draws; vector move: index and the vector's draws; MultiStepMove: per
 * sub-step s the vector move of sub-step 1 + s and its acceptance uniform; then the step's
 * acceptance uniform */
static void philox_fill(drawsrc *d)
{
    const int cpb = (d->philox == 1) ? 4 : 2;
    int n = 0;
    if (d->pmove == MCIG_MOVE_VEC) {
        n = philox_vec(d, 0, d->psrrd, d->pveclen, n);
    } else if (d->pmove == MCIG_MOVE_MULTISTEP) {
        for (int s = 0; s < d->pms_nsteps; ++s) {
            n = philox_vec(d, (uint32_t)(1 + s), d->pms_srrd, d->pms_veclen, n);
            d->pbuf[n++] = philox_accept(d, (uint32_t)(1 + s));
        }
    } else {
        double v[4];
        for (int i = 0; i < d->pndim; ++i) {
            if (i % cpb == 0) { philox_move_block(d, 0, d->psrrd, (uint32_t)(i / cpb), v); }
            d->pbuf[n++] = v[i % cpb];
        }
    }
    d->pbuf[n++] = philox_accept(d, 0);
    d->pbuf_n = n;
    d->pbuf_pos = 0;
}

static double philox_next(drawsrc *d)
{
    if (d->pbuf_pos >= d->pbuf_n) { philox_fill(d); }
    const double v = d->pbuf[d->pbuf_pos++];
    if (d->pbuf_pos >= d->pbuf_n) { ++d->pctr; } /* the step's acceptance draw: next step */
    return v;
}

static void rec_push(drawsrc *d, double v)
{
    if (!d->recording) { return; }
    if (d->rec_len == d->rec_cap) {
        d->rec_cap = d->rec_cap ? 2 * d->rec_cap : 4096;
        d->rec = (double *)realloc(d->rec, (size_t)d->rec_cap * sizeof(double));
    }
    d->rec[d->rec_len++] = v;
}

static int tape_next(drawsrc *d, double *v)
{
    if (d->tape_pos >= d->tape_len) {
        d->exhausted = 1;
        *v = 0.5;
        return 0;
    }
    *v = d->tape[d->tape_pos++];
    return 1;
}

/* uniform_real_distribution<double>(0,1) (MCIntegrator.hpp:34, MultiStepMove.hpp:28) */
static double draw_u01(drawsrc *d)
{
    double v;
    if (d->philox) { return philox_next(d); }
    if (d->tape) { tape_next(d, &v); return v; }
    v = canonical(&d->mt);
    rec_push(d, v);
    return v;
}

/* createSymRRD<uniform_real_distribution>() = U(-1,1) (TrialMoveInterface.hpp:120-124) */
static double draw_upm1(drawsrc *d)
{
    double v;
    if (d->philox) { return philox_next(d); }
    if (d->tape) { tape_next(d, &v); return v; }
    v = canonical(&d->mt) * 2.0 + -1.0;
    rec_push(d, v);
    return v;
}

/* normal_distribution<double>() (TrialMoveInterface.hpp:127-131) */
static double draw_normal(drawsrc *d, normstate *st)
{
    double v;
    if (d->philox) { return philox_next(d); }
    if (d->tape) { tape_next(d, &v); return v; }
    v = polar_normal(&d->mt, st);
    rec_push(d, v);
    return v;
}

/* uniform_int_distribution<int>(0, n-1) (SRRDVecMove.hpp:31,66) */
static int draw_index(drawsrc *d, int n)
{
    double v;
    if (d->philox) { return (int)philox_next(d); }
    if (d->tape) {
        tape_next(d, &v);
        int i = (int)v;
        return (i < 0) ? 0 : (i >= n ? n - 1 : i);
    }
    int i = (int)lemire_int(&d->mt, (uint64_t)n);
    rec_push(d, (double)i);
    return i;
}

/* ---- the other distributions of createSymRRD (include/mci/TrialMoveInterface.hpp:82-200),
 * restated from libstdc++ (GCC 13.3, bits/random.tcc and bits/random.h) with their default
 * parameters.  A distribution object keeps state between draws: the normal_distribution inside
 * it caches its second value, so each move holds three normal states: [0] the distribution's own
 * normal_distribution, [1] and [2] those of its gamma_distribution members. */

/* gamma_distribution<double>(alpha, beta)::operator() (random.tcc, Marsaglia & Tsang, ACM TOMS
 * 26 (2000) 363-372), with param_type::_M_initialize's constants; nd: the object's normal */
static double gamma_draw(mt64 *m, normstate *nd, double alpha, double beta)
{
    const double malpha = alpha < 1.0 ? alpha + 1.0 : alpha;
    const double a2 = 1.0 / sqrt(9.0 * (malpha - 1.0 / 3.0));
    const double a1 = malpha - 1.0 / 3.0;
    double u, v, n;
    do {
        do {
            n = polar_normal(m, nd);
            v = 1.0 + a2 * n;
        } while (v <= 0.0);
        v = v * v * v;
        u = canonical(m);
    } while (u > 1.0 - 0.0331 * n * n * n * n && log(u) > (0.5 * n * n + a1 * (1.0 - v + log(v))));
    if (alpha == malpha) { return a1 * v * beta; }
    do {
        u = canonical(m);
    } while (u == 0.0);
    return pow(u, 1.0 / alpha) * a1 * v * beta;
}

/* bernoulli_distribution(0.5)::operator() of SymmetrizedPRRD (TrialMoveInterface.hpp:82-98):
 * the positive value first, then the sign */
static double symmetrized(mt64 *m, double val)
{
    return (canonical(m) - 0.0 < 0.5 * (1.0 - 0.0)) ? val : -val;
}

/* one draw of SRRDType srrd (Factories.hpp:115-128) from the engine */
static double srrd_engine(mt64 *m, int srrd, normstate *st)
{
    switch (srrd) {
    case MCIG_SRRD_UNIFORM: return canonical(m) * 2.0 + -1.0;
    case MCIG_SRRD_GAUSSIAN: return polar_normal(m, &st[0]);
    case MCIG_SRRD_STUDENT: { /* student_t_distribution(n = 1): _M_nd * sqrt(n / _M_gd), gamma(n/2, 2);
                               * GCC evaluates the normal first */
        const double z = polar_normal(m, &st[0]);
        return z * sqrt(1.0 / gamma_draw(m, &st[1], 1.0 / 2, 2.0));
    }
    case MCIG_SRRD_CAUCHY: { /* cauchy_distribution(0, 1) */
        double u;
        do {
            u = canonical(m);
        } while (u == 0.5);
        const double pi = 3.1415926535897932384626433832795029;
        return 0.0 + 1.0 * tan(pi * u);
    }
    case MCIG_SRRD_EXPONENTIAL: return symmetrized(m, -log(1.0 - canonical(m)) / 1.0);
    case MCIG_SRRD_GAMMA: return symmetrized(m, gamma_draw(m, &st[1], 1.0, 1.0));
    case MCIG_SRRD_WEIBULL: return symmetrized(m, 1.0 * pow(-log(1.0 - canonical(m)), 1.0 / 1.0));
    case MCIG_SRRD_LOGNORMAL: return symmetrized(m, exp(1.0 * polar_normal(m, &st[0]) + 0.0));
    case MCIG_SRRD_CHISQ: return symmetrized(m, 2 * gamma_draw(m, &st[1], 1.0 / 2, 1.0));
    default: { /* FISHER: fisher_f_distribution(m = 1, n = 1): (gamma_x(m/2) n) / (gamma_y(n/2) m) */
        const double gx = gamma_draw(m, &st[1], 1.0 / 2, 1.0) * 1.0;
        const double gy = gamma_draw(m, &st[2], 1.0 / 2, 1.0) * 1.0;
        return symmetrized(m, gx / gy);
    }
    }
}

/* n draws of SRRDType srrd from a fresh distribution object and std::mt19937_64(seed) */
void orc_srrd_stream(int srrd, uint64_t seed, int64_t n, double *out)
{
    mt64 m;
    mt_seed(&m, seed);
    normstate st[3] = {{0, 0.}, {0, 0.}, {0, 0.}};
    for (int64_t i = 0; i < n; ++i) { out[i] = srrd_engine(&m, srrd, st); }
}

/* the move draw of SRRDType srrd: tape, Philox (uniform and Gaussian) or the engine */
static double draw_srrd(drawsrc *d, int srrd, normstate *st)
{
    if (srrd == MCIG_SRRD_GAUSSIAN) { return draw_normal(d, &st[0]); }
    if (srrd == MCIG_SRRD_UNIFORM) { return draw_upm1(d); }
    double v;
    if (d->philox) { return philox_next(d); } /* not reached: orc_set_philox takes uniform and Gaussian only */
    if (d->tape) { tape_next(d, &v); return v; }
    v = srrd_engine(&d->mt, srrd, st);
    rec_push(d, v);
    return v;
}

/* ------------------------------------------------------------------ */
/* sampling functions (test/common/TestMCIFunctions.hpp + config pdfs)  */
/* ------------------------------------------------------------------ */
typedef struct {
    int kind;
    int ndim;
    int nproto;
    int nparams;
    double *params;
    /* derived constants (GAUSS_BLOCK: 1/(2w^2); GAUSS_MIX: per-component log-normalisation) */
    double *derived;
} pdfdef;

static int pdf_init(pdfdef *p, int kind, int ndim, const double *params, int nparams)
{
    memset(p, 0, sizeof(*p));
    p->kind = kind;
    p->ndim = ndim;
    p->nparams = nparams;
    if (nparams > 0) {
        p->params = (double *)malloc((size_t)nparams * sizeof(double));
        memcpy(p->params, params, (size_t)nparams * sizeof(double));
    }
    switch (kind) {
    case MCIG_PDF_GAUSS_SUM: p->nproto = 1; break;
    case MCIG_PDF_GAUSS:
    case MCIG_PDF_EXP: p->nproto = ndim; break;
    case MCIG_PDF_GAUSS_PREC:
        if (nparams != ndim * ndim) { return fail(MCIG_ERR_INVALID_ARGUMENT, "GAUSS_PREC needs ndim*ndim params"); }
        p->nproto = 1;
        break;
    case MCIG_PDF_GAUSS_BLOCK:
        if (nparams != 3) { return fail(MCIG_ERR_INVALID_ARGUMENT, "GAUSS_BLOCK needs [b0,b1,w]"); }
        if ((int)params[0] < 0 || (int)params[1] > ndim || (int)params[0] >= (int)params[1] || !(params[2] > 0.)) {
            return fail(MCIG_ERR_INVALID_ARGUMENT, "GAUSS_BLOCK bad block");
        }
        p->nproto = 1;
        p->derived = (double *)malloc(sizeof(double));
        p->derived[0] = 0.5 / (params[2] * params[2]);
        break;
    case MCIG_PDF_GAUSS_MIX: {
        if (nparams < 1) { return fail(MCIG_ERR_INVALID_ARGUMENT, "GAUSS_MIX needs params"); }
        const int nc = (int)params[0];
        if (nc < 1 || nparams != 1 + nc + 2 * nc * ndim) { return fail(MCIG_ERR_INVALID_ARGUMENT, "GAUSS_MIX bad param count"); }
        p->nproto = 1;
        p->derived = (double *)malloc((size_t)nc * sizeof(double));
        const double *w = params + 1, *s = params + 1 + nc + nc * ndim;
        for (int c = 0; c < nc; ++c) {
            double l = log(w[c]) - 0.5 * ndim * log(2.0 * M_PI);
            for (int i = 0; i < ndim; ++i) { l -= log(s[c * ndim + i]); }
            p->derived[c] = l;
        }
        break;
    }
    default:
        return fail(MCIG_ERR_INVALID_ARGUMENT, "unknown sampling function kind");
    }
    return MCIG_OK;
}

static void pdf_free(pdfdef *p)
{
    free(p->params);
    free(p->derived);
    memset(p, 0, sizeof(*p));
}

/* log of the mixture density (GAUSS_MIX) */
static double mix_logp(const pdfdef *p, const double *x)
{
    const int nd = p->ndim, nc = (int)p->params[0];
    const double *m = p->params + 1 + nc, *s = p->params + 1 + nc + nc * nd;
    double e[64];
    double mx = -INFINITY;
    for (int c = 0; c < nc && c < 64; ++c) {
        double a = p->derived[c];
        for (int i = 0; i < nd; ++i) {
            const double z = (x[i] - m[c * nd + i]) / s[c * nd + i];
            a += -0.5 * (z * z);
        }
        e[c] = a;
        if (a > mx) { mx = a; }
    }
    double sum = 0.;
    for (int c = 0; c < nc && c < 64; ++c) { sum += exp(e[c] - mx); }
    return mx + log(sum);
}

/* protoFunction */
static void pdf_proto(const pdfdef *p, const double *x, double *pv)
{
    const int nd = p->ndim;
    switch (p->kind) {
    case MCIG_PDF_GAUSS_SUM: { /* ThreeDimGaussianPDF::protoFunction (:134-137), generalised */
        double s = x[0] * x[0];
        for (int i = 1; i < nd; ++i) { s = s + x[i] * x[i]; }
        pv[0] = s;
        break;
    }
    case MCIG_PDF_GAUSS: /* Gauss::protoFunction (:162-167) */
        for (int i = 0; i < nd; ++i) { pv[i] = x[i] * x[i]; }
        break;
    case MCIG_PDF_EXP: /* ExpNDPDF::protoFunction (:229-232) */
        for (int i = 0; i < nd; ++i) { pv[i] = fabs(x[i]); }
        break;
    case MCIG_PDF_GAUSS_PREC: {
        const double *P = p->params;
        double q = 0.;
        for (int i = 0; i < nd; ++i) {
            double t = 0.;
            for (int j = 0; j < nd; ++j) { t = t + P[i * nd + j] * x[j]; }
            q = q + x[i] * t;
        }
        pv[0] = 0.5 * q;
        break;
    }
    case MCIG_PDF_GAUSS_BLOCK: {
        const int b0 = (int)p->params[0], b1 = (int)p->params[1];
        double s = 0.;
        for (int i = b0; i < b1; ++i) { s = s + x[i] * x[i]; }
        pv[0] = s * p->derived[0];
        break;
    }
    case MCIG_PDF_GAUSS_MIX:
        pv[0] = -mix_logp(p, x);
        break;
    default: break;
    }
}

static double fold_sum(const double *v, int n)
{
    double s = 0.; /* std::accumulate(v, v+n, 0.) */
    for (int i = 0; i < n; ++i) { s = s + v[i]; }
    return s;
}

/* samplingFunction */
static double pdf_value(const pdfdef *p, const double *pv)
{
    switch (p->kind) {
    case MCIG_PDF_GAUSS:
    case MCIG_PDF_EXP: return exp(-fold_sum(pv, p->nproto)); /* Gauss (:169-172), ExpNDPDF (:234-237) */
    default: return exp(-pv[0]);                              /* ThreeDimGaussianPDF (:139-142) */
    }
}

/* acceptanceFunction */
static double pdf_accept(const pdfdef *p, const double *po, const double *pn)
{
    switch (p->kind) {
    case MCIG_PDF_GAUSS:
    case MCIG_PDF_EXP: { /* Gauss (:174-179), ExpNDPDF (:239-244) */
        double e = fold_sum(po, p->nproto);
        e = e - fold_sum(pn, p->nproto);
        return exp(e);
    }
    default: /* ThreeDimGaussianPDF (:144-147): exp(-new + old) */
        return exp(-pn[0] + po[0]);
    }
}

/* SamplingFunctionInterface::computeAcceptance (SamplingFunctionInterface.hpp:49-57) */
static double pdf_compute_acceptance(const pdfdef *p, const double *xn, int nchanged, const int *cidx,
                                     const double *po, double *pn)
{
    if (nchanged < p->ndim && (p->kind == MCIG_PDF_GAUSS || p->kind == MCIG_PDF_EXP)) {
        /* Gauss::updatedAcceptance (:181-189), ExpNDPDF::updatedAcceptance (:246-255) */
        double e = 0.;
        for (int i = 0; i < nchanged; ++i) {
            const int c = cidx[i];
            pn[c] = (p->kind == MCIG_PDF_GAUSS) ? xn[c] * xn[c] : fabs(xn[c]);
            e = e + (pn[c] - po[c]);
        }
        return exp(-e);
    }
    /* default updatedAcceptance (:92-97) and the all-changed branch (:54-56) */
    pdf_proto(p, xn, pn);
    return pdf_accept(p, po, pn);
}

/* ------------------------------------------------------------------ */
/* observables                                                         */
/* ------------------------------------------------------------------ */
typedef struct {
    int kind;
    int ndim;
    int nobs;
    int nparams;
    double *params;
    const pdfdef *pdf; /* LOGPDF: the sampling functions of the MCI (NULL: none) */
    const int *npdf;
} obsdef;

static int obs_init(obsdef *o, int kind, int ndim, const double *params, int nparams)
{
    memset(o, 0, sizeof(*o));
    o->kind = kind;
    o->ndim = ndim;
    o->nparams = nparams;
    if (nparams > 0) {
        o->params = (double *)malloc((size_t)nparams * sizeof(double));
        memcpy(o->params, params, (size_t)nparams * sizeof(double));
    }
    switch (kind) {
    case MCIG_OBS_X2SUM:
    case MCIG_OBS_X2MEAN:
    case MCIG_OBS_POLYNOM:
    case MCIG_OBS_GAUSSX2:
    case MCIG_OBS_LOGPDF: o->nobs = 1; break;
    case MCIG_OBS_CONST:
        if (nparams < 1) { return fail(MCIG_ERR_INVALID_ARGUMENT, "CONST needs its value"); }
        o->nobs = 1;
        break;
    case MCIG_OBS_XND:
    case MCIG_OBS_X2: o->nobs = ndim; break;
    case MCIG_OBS_XI:
        if (nparams < 1 || (int)params[0] < 0 || (int)params[0] >= ndim) { return fail(MCIG_ERR_INVALID_ARGUMENT, "XI needs an index in [0, ndim)"); }
        o->nobs = 1;
        break;
    case MCIG_OBS_X2BLOCK: {
        if (nparams < 2) { return fail(MCIG_ERR_INVALID_ARGUMENT, "X2BLOCK needs [nb, b0..b_nb]"); }
        const int nb = (int)params[0];
        if (nb < 1 || nparams != nb + 2) { return fail(MCIG_ERR_INVALID_ARGUMENT, "X2BLOCK bad param count"); }
        for (int k = 0; k < nb; ++k) {
            if ((int)params[1 + k] < 0 || (int)params[2 + k] > ndim || (int)params[1 + k] > (int)params[2 + k]) {
                return fail(MCIG_ERR_INVALID_ARGUMENT, "X2BLOCK bad bounds");
            }
        }
        o->nobs = nb;
        break;
    }
    default: return fail(MCIG_ERR_INVALID_ARGUMENT, "unknown observable kind");
    }
    return MCIG_OK;
}

static void obs_free(obsdef *o)
{
    free(o->params);
    memset(o, 0, sizeof(*o));
}

/* observableFunction of the matching test classes */
static void obs_eval(const obsdef *o, const double *x, double *out)
{
    const int nd = o->ndim;
    switch (o->kind) {
    case MCIG_OBS_LOGPDF: { /* log of the product of the sampling functions: -sum_k (sum of proto_k) */
        double s = 0., pv[256];
        for (int k = 0; o->pdf && k < *o->npdf; ++k) {
            pdf_proto(&o->pdf[k], x, pv);
            s = s - fold_sum(pv, o->pdf[k].nproto);
        }
        out[0] = s;
        break;
    }
    case MCIG_OBS_X2SUM: { /* X2Sum (:424-430) */
        double s = 0.;
        for (int i = 0; i < nd; ++i) { s = s + x[i] * x[i]; }
        out[0] = s;
        break;
    }
    case MCIG_OBS_XND: /* XND (:344-347) */
        for (int i = 0; i < nd; ++i) { out[i] = x[i]; }
        break;
    case MCIG_OBS_X2: /* X2 (:445-450) */
        for (int i = 0; i < nd; ++i) { out[i] = x[i] * x[i]; }
        break;
    case MCIG_OBS_X2MEAN: { /* XSquared (:269-272): (x0*x0 + x1*x1 + x2*x2)/3. */
        double s = x[0] * x[0];
        for (int i = 1; i < nd; ++i) { s = s + x[i] * x[i]; }
        out[0] = s / (double)nd;
        break;
    }
    case MCIG_OBS_CONST: out[0] = o->params[0]; break; /* Constval (:385-388) */
    case MCIG_OBS_XI: out[0] = x[(int)o->params[0]]; break;
    case MCIG_OBS_POLYNOM: { /* Polynom (:403-409) */
        double s = 0.;
        for (int i = 0; i < nd; ++i) { s = s + x[i]; }
        out[0] = s;
        break;
    }
    case MCIG_OBS_X2BLOCK: {
        const int nb = (int)o->params[0];
        for (int k = 0; k < nb; ++k) {
            double s = 0.;
            for (int i = (int)o->params[1 + k]; i < (int)o->params[2 + k]; ++i) { s = s + x[i] * x[i]; }
            out[k] = s;
        }
        break;
    }
    case MCIG_OBS_GAUSSX2: { /* GaussXSquared (:287-293) */
        double r2 = x[0] * x[0];
        for (int i = 1; i < nd; ++i) { r2 = r2 + x[i] * x[i]; }
        const double normf = 1. / sqrt(M_PI * M_PI * M_PI) / 3.;
        out[0] = exp(-r2) * r2 * normf;
        break;
    }
    default: break;
    }
}

/* ------------------------------------------------------------------ */
/* accumulators (AccumulatorInterface.cpp, Simple/Block/FullAccumulator.cpp) */
/* ------------------------------------------------------------------ */
typedef struct {
    const obsdef *obs;
    int type, nskip, blocksize;
    int64_t nsteps, nstore;
    double *data;
    double *vals; /* _obs_values */
    int nchanged, skipidx, bidx;
    int64_t stepidx, storeidx;
} accu;

static int64_t accu_naccu(const accu *a) { return a->nsteps > 0 ? 1 + (a->nsteps - 1) / a->nskip : 0; }

/* AccumulatorInterface::allocate (:88-96) + child _allocate */
static int accu_alloc(accu *a, const obsdef *o, int type, int blocksize, int nskip, int64_t nsteps)
{
    memset(a, 0, sizeof(*a));
    a->obs = o;
    a->type = type;
    a->nskip = nskip;
    a->blocksize = blocksize;
    if (nsteps < 1) { return fail(MCIG_ERR_INVALID_ARGUMENT, "[AccumulatorInterface::allocate] Provided number of MC steps was < 1 ."); }
    a->nsteps = nsteps;
    const int64_t naccu = accu_naccu(a);
    switch (type) {
    case MCIG_ACC_SIMPLE: a->nstore = 1; break;
    case MCIG_ACC_FULL: a->nstore = naccu; break;
    case MCIG_ACC_BLOCK: /* BlockAccumulator::_allocate (:6-17) */
        if (naccu < blocksize) { return fail(MCIG_ERR_INVALID_ARGUMENT, "[BlockAccumulator::allocate] Requested number of accumulations is smaller than the requested block size."); }
        if (naccu % blocksize != 0) { return fail(MCIG_ERR_INVALID_ARGUMENT, "[BlockAccumulator::allocate] Requested number of accumulations is not a multiple of the requested block size."); }
        a->nstore = naccu / blocksize;
        break;
    default: return fail(MCIG_ERR_INVALID_ARGUMENT, "bad accumulator");
    }
    a->data = (double *)calloc((size_t)(a->nstore * o->nobs), sizeof(double));
    a->vals = (double *)calloc((size_t)o->nobs, sizeof(double));
    a->nchanged = o->ndim; /* _init (:21-29) */
    a->skipidx = nskip - 1;
    return MCIG_OK;
}

static void accu_free(accu *a)
{
    free(a->data);
    free(a->vals);
    a->data = NULL;
    a->vals = NULL;
}

static void accu_store(accu *a)
{
    const int n = a->obs->nobs;
    switch (a->type) {
    case MCIG_ACC_SIMPLE: /* SimpleAccumulator::_accumulate (:14-19) */
        for (int i = 0; i < n; ++i) { a->data[i] = a->data[i] + a->vals[i]; }
        break;
    case MCIG_ACC_BLOCK: /* BlockAccumulator::_accumulate (:20-30) */
        for (int i = 0; i < n; ++i) { a->data[a->storeidx + i] = a->data[a->storeidx + i] + a->vals[i]; }
        if (++a->bidx == a->blocksize) {
            a->bidx = 0;
            a->storeidx += n;
        }
        break;
    case MCIG_ACC_FULL: /* FullAccumulator::_accumulate (:14-18) */
        memcpy(a->data + a->storeidx, a->vals, (size_t)n * sizeof(double));
        a->storeidx += n;
        break;
    default: break;
    }
}

/* AccumulatorInterface::accumulate (:99-114) with _processFull (:40-53) / _processOld (:31-38) */
static void accu_accumulate(accu *a, const double *xnew, int accepted)
{
    if (accepted || a->nchanged > 0) {
        a->nchanged = a->obs->ndim;
        if (++a->skipidx == a->nskip) {
            a->skipidx = 0;
            obs_eval(a->obs, xnew, a->vals);
            a->nchanged = 0;
            accu_store(a);
        }
    } else {
        if (++a->skipidx == a->nskip) {
            a->skipidx = 0;
            accu_store(a);
        }
    }
    ++a->stepidx;
}

/* AccumulatorInterface::finalize (:117-122) + child _finalize */
static int accu_finalize(accu *a)
{
    if (a->stepidx != a->nsteps) { return fail(MCIG_ERR_RUNTIME, "[AccumulatorInterface::finalize] step count mismatch"); }
    const int n = a->obs->nobs;
    if (a->type == MCIG_ACC_SIMPLE) { /* SimpleAccumulator::_finalize (:22-29) */
        const double normf = 1. / (double)accu_naccu(a);
        for (int i = 0; i < n; ++i) { a->data[i] = a->data[i] * normf; }
    } else if (a->type == MCIG_ACC_BLOCK) { /* BlockAccumulator::_finalize (:33-41) */
        const double normf = 1. / a->blocksize;
        for (int64_t i = 0; i < a->nstore * n; ++i) { a->data[i] = a->data[i] * normf; }
    }
    return MCIG_OK;
}

/* ------------------------------------------------------------------ */
/* estimators (src/Estimators.cpp, src/MJBlocker.cpp)                   */
/* ------------------------------------------------------------------ */

/* MultiDimUncorrelatedEstimator (Estimators.cpp:125-155).  The wrapper
 * UncorrelatedEstimator (:250-258) sends ndim == 1 to OneDimUncorrelatedEstimator
 * (:36-56), which divides by (n - 1.) where the N-D form multiplies by 1/(n - 1.);
 * one_d selects that rounding. */
static int est_uncorrelated_impl(int64_t n, int nd, const double *x, double *avg, double *err, int one_d)
{
    if (n < 2) { return fail(MCIG_ERR_INVALID_ARGUMENT, "[UncorrelatedEstimator] n must be larger than 1"); }
    const double SMALLEST_ERROR = 1.e-300;
    for (int j = 0; j < nd; ++j) { avg[j] = 0.; err[j] = 0.; }
    for (int64_t i = 0; i < n; ++i) {
        for (int j = 0; j < nd; ++j) {
            avg[j] = avg[j] + x[i * nd + j];
            err[j] = err[j] + x[i * nd + j] * x[i * nd + j];
        }
    }
    const double norm = 1. / n;
    const double norm2 = 1. / (n - 1.);
    for (int j = 0; j < nd; ++j) {
        avg[j] = avg[j] * norm;
        err[j] = err[j] * norm - avg[j] * avg[j];
        if (one_d) { err[j] = (err[j] > SMALLEST_ERROR) ? sqrt(err[j] / (n - 1.)) : 0.; }
        else { err[j] = (err[j] > SMALLEST_ERROR) ? sqrt(err[j] * norm2) : 0.; }
    }
    return MCIG_OK;
}

static int est_uncorrelated(int64_t n, int nd, const double *x, double *avg, double *err)
{
    return est_uncorrelated_impl(n, nd, x, avg, err, nd == 1);
}

/* block means then the uncorrelated estimator; one_d as above
 * (OneDimBlockEstimator :59-76 / MultiDimBlockEstimator :158-185) */
static int block_estimate_impl(int64_t n, int nd, const double *x, int64_t nblocks, double *avg, double *err, int one_d);

/* MultiDimBlockEstimator (Estimators.cpp:158-185) */
int orc_block_estimate(int64_t n, int nd, const double *x, int64_t nblocks, double *avg, double *err)
{
    return block_estimate_impl(n, nd, x, nblocks, avg, err, 0);
}

static int block_estimate_impl(int64_t n, int nd, const double *x, int64_t nblocks, double *avg, double *err, int one_d)
{
    if (n < nblocks) { return fail(MCIG_ERR_INVALID_ARGUMENT, "MultiDimBlockEstimator: n must be >= nblocks"); }
    const int64_t nper = n / nblocks;
    const double norm = 1. / nper;
    double *av = (double *)calloc((size_t)(nblocks * nd), sizeof(double));
    for (int64_t b = 0; b < nblocks; ++b) {
        for (int64_t i = b * nper; i < (b + 1) * nper; ++i) {
            for (int j = 0; j < nd; ++j) { av[b * nd + j] = av[b * nd + j] + x[i * nd + j]; }
        }
    }
    for (int64_t i = 0; i < nblocks * nd; ++i) { av[i] = av[i] * norm; }
    const int rc = est_uncorrelated_impl(nblocks, nd, av, avg, err, one_d);
    free(av);
    return rc;
}

/* calcErrDelta (Estimators.cpp:9-31) */
static double calc_err_delta(int mode, const double *e /* 9 values, centre at 4 */)
{
    const int im = 4;
    switch (mode) {
    case 1: return (-0.5 * e[im - 1] + 0.5 * e[im + 1]);
    case 2: return ((1. / 12.) * e[im - 2] - (2. / 3.) * e[im - 1] + (2. / 3.) * e[im + 1] - (1. / 12.) * e[im + 2]);
    case 3: return (-(1. / 60.) * e[im - 3] + (3. / 20.) * e[im - 2] - 0.75 * e[im - 1] + 0.75 * e[im + 1]
                    - (3. / 20.) * e[im + 2] + (1. / 60.) * e[im + 3]);
    case 4: return ((1. / 280.) * e[im - 4] - (4. / 105.) * e[im - 3] + 0.2 * e[im - 2] - 0.8 * e[im - 1]
                    + 0.8 * e[im + 1] - 0.2 * e[im + 2] + (4. / 105.) * e[im + 3] - (1. / 280.) * e[im + 4]);
    default: return 0.;
    }
}

/* MultiDimFCBlockerEstimator (Estimators.cpp:191-246); 1-D (:82-122) is identical arithmetic */
static int est_fcblocker(int64_t n, int nd, const double *x, double *avg, double *err)
{
    enum { MIN_BLOCKS = 6, MAX_BLOCKS = 50, MAX_PLATEAU_AVERAGE = 4 };
    if (n < MAX_BLOCKS) { return fail(MCIG_ERR_INVALID_ARGUMENT, "FCBlockerEstimator: n must be >= 50"); }
    const int nav = MAX_BLOCKS - MIN_BLOCKS + 1;
    double *av = (double *)malloc((size_t)(nav * nd) * sizeof(double));
    double *er = (double *)malloc((size_t)(nav * nd) * sizeof(double));
    for (int i1 = 0; i1 < nav; ++i1) {
        block_estimate_impl(n, nd, x, i1 + MIN_BLOCKS, av + i1 * nd, er + i1 * nd, nd == 1);
    }
    const int naccd = nav - 2 * MAX_PLATEAU_AVERAGE;
    double *acc = (double *)calloc((size_t)(naccd * nd), sizeof(double));
    double eh[9];
    for (int i2 = MAX_PLATEAU_AVERAGE; i2 < naccd + MAX_PLATEAU_AVERAGE; ++i2) {
        for (int j = 0; j < nd; ++j) {
            for (int s = -4; s < 5; ++s) { eh[s + 4] = er[(i2 + s) * nd + j]; }
            for (int i1 = 1; i1 <= MAX_PLATEAU_AVERAGE; ++i1) {
                acc[(i2 - MAX_PLATEAU_AVERAGE) * nd + j] = acc[(i2 - MAX_PLATEAU_AVERAGE) * nd + j] + calc_err_delta(i1, eh);
            }
        }
    }
    for (int j = 0; j < nd; ++j) {
        int imin = 0;
        for (int i2 = 1; i2 < naccd; ++i2) {
            if (fabs(acc[i2 * nd + j]) < fabs(acc[imin * nd + j])) { imin = i2; }
        }
        const int k = imin + MAX_PLATEAU_AVERAGE;
        avg[j] = 0.2 * (av[(k - 2) * nd + j] + av[(k - 1) * nd + j] + av[k * nd + j] + av[(k + 1) * nd + j] + av[(k + 2) * nd + j]);
        err[j] = 0.2 * (er[(k - 2) * nd + j] + er[(k - 1) * nd + j] + er[k * nd + j] + er[(k + 1) * nd + j] + er[(k + 2) * nd + j]);
    }
    free(acc);
    free(er);
    free(av);
    return MCIG_OK;
}

/* chi^2 quantiles used by MJBlocker (MJBlocker.cpp:6-13): the 0.95 quantile
 * of the chi-squared distribution with k+1 degrees of freedom, k = 0..63. */
static const double MJ_QUANTILE[64] = {
    3.841459, 5.991465, 7.814728, 9.487729, 11.070498, 12.591587, 14.067140, 15.507313,
    16.918978, 18.307038, 19.675138, 21.026070, 22.362032, 23.684791, 24.995790, 26.296228,
    27.587112, 28.869299, 30.143527, 31.410433, 32.670573, 33.924438, 35.172462, 36.415029,
    37.652484, 38.885139, 40.113272, 41.337138, 42.556968, 43.772972, 44.985343, 46.194260,
    47.399884, 48.602367, 49.801850, 50.998460, 52.192320, 53.383541, 54.572228, 55.758479,
    56.942387, 58.124038, 59.303512, 60.480887, 61.656233, 62.829620, 64.001112, 65.170769,
    66.338649, 67.504807, 68.669294, 69.832160, 70.993453, 72.153216, 73.311493, 74.468324,
    75.623748, 76.777803, 77.930524, 79.081944, 80.232098, 81.381015, 82.528727, 83.675261};

/* MJBlocker::estimate (MJBlocker.cpp:127-154).  Where the reference would
 * index one level past its arrays (no level passes the test: constant data,
 * or n == 1), the last level is used instead. */
static int est_mjblocker(int64_t n, int nd, const double *xin, double *avg, double *err)
{
    if (n <= 0) { return fail(MCIG_ERR_INVALID_ARGUMENT, "[MJBlocker] ndata must be a natural number."); }
    if (((uint64_t)n & ((uint64_t)n - 1)) != 0) { return fail(MCIG_ERR_INVALID_ARGUMENT, "[MJBlocker] ndata must be a power of two."); }
    int npow = 0;
    while ((1LL << npow) < n) { ++npow; }
    double *x = (double *)malloc((size_t)(n * nd) * sizeof(double));
    double *X = (double *)malloc((size_t)(n * nd) * sizeof(double));
    const int np1 = npow > 0 ? npow : 1;
    double *var = (double *)calloc((size_t)(np1 * nd), sizeof(double));
    double *gam = (double *)calloc((size_t)(np1 * nd), sizeof(double));
    double *M = (double *)calloc((size_t)(np1 * nd), sizeof(double));
    double *Ms = (double *)calloc((size_t)(np1 * nd), sizeof(double));
    memcpy(x, xin, (size_t)(n * nd) * sizeof(double));
    /* _computeMean (:46-55) */
    for (int j = 0; j < nd; ++j) { avg[j] = 0.; }
    for (int64_t i = 0; i < n; ++i) {
        for (int j = 0; j < nd; ++j) { avg[j] = avg[j] + x[i * nd + j]; }
    }
    for (int j = 0; j < nd; ++j) { avg[j] = avg[j] / n; }
    /* _initX (:58-65) */
    for (int64_t i = 0; i < n; ++i) {
        for (int j = 0; j < nd; ++j) { X[i * nd + j] = x[i * nd + j] - avg[j]; }
    }
    int64_t nred = n;
    for (int k = 0; k < npow; ++k) {
        /* _gamma0 (:70-79) */
        double *v = var + k * nd, *g = gam + k * nd;
        for (int j = 0; j < nd; ++j) { v[j] = 0.; g[j] = 0.; }
        for (int64_t i = 0; i < nred; ++i) {
            for (int j = 0; j < nd; ++j) { v[j] = v[j] + X[i * nd + j] * X[i * nd + j]; }
        }
        for (int j = 0; j < nd; ++j) { v[j] = v[j] / nred; }
        /* _gamma1 (:82-91) */
        for (int64_t i = 0; i < nred - 1; ++i) {
            for (int j = 0; j < nd; ++j) { g[j] = g[j] + X[i * nd + j] * X[(i + 1) * nd + j]; }
        }
        for (int j = 0; j < nd; ++j) { g[j] = g[j] / nred; }
        /* _transform (:94-103) */
        for (int64_t i = 0; i < nred / 2; ++i) {
            for (int j = 0; j < nd; ++j) {
                x[i * nd + j] = 0.5 * (x[(2 * i) * nd + j] + x[(2 * i + 1) * nd + j]);
                X[i * nd + j] = x[i * nd + j] - avg[j];
            }
        }
        nred = nred / 2;
    }
    /* _generateM (:106-123) */
    for (int i = 0; i < npow; ++i) {
        for (int j = 0; j < nd; ++j) {
            const double r = gam[i * nd + j] / var[i * nd + j];
            M[(npow - i - 1) * nd + j] = (r * r) * ldexp(1.0, npow - i);
        }
    }
    for (int i = 0; i < npow; ++i) {
        for (int jj = 0; jj <= i; ++jj) {
            for (int j = 0; j < nd; ++j) { Ms[i * nd + j] = Ms[i * nd + j] + M[jj * nd + j]; }
        }
    }
    /* level choice (:131-152) */
    for (int l = 0; l < nd; ++l) {
        int k;
        for (k = npow - 1; k >= 0; --k) {
            if (Ms[k * nd + l] < MJ_QUANTILE[k]) { break; }
        }
        k = npow - (k + 1);
        if (k > npow - 1) { k = npow - 1; }
        if (k < 0) { k = 0; }
        err[l] = (npow > 0) ? sqrt(var[k * nd + l] / ldexp(1.0, npow - k)) : 0.;
    }
    free(Ms); free(M); free(gam); free(var); free(X); free(x);
    return MCIG_OK;
}

/* CorrelatedEstimator (:278-286) / factory dispatch (Factories.hpp:57-76) */
int orc_estimate(int type, int64_t n, int nd, const double *x, double *avg, double *err)
{
    switch (type) {
    case MCIG_EST_NOOP: /* NoopEstimator (:289-293) */
        for (int j = 0; j < nd; ++j) { avg[j] = x[j]; err[j] = 0.; }
        return MCIG_OK;
    case MCIG_EST_UNCORRELATED: return est_uncorrelated(n, nd, x, avg, err);
    case MCIG_EST_FCBLOCKER: return est_fcblocker(n, nd, x, avg, err);
    case MCIG_EST_MJBLOCKER: return est_mjblocker(n, nd, x, avg, err);
    case MCIG_EST_CORRELATED:
        if (n > 0 && (((uint64_t)n & ((uint64_t)n - 1)) == 0)) { return est_mjblocker(n, nd, x, avg, err); }
        return est_fcblocker(n, nd, x, avg, err);
    default: return fail(MCIG_ERR_DOMAIN, "[createEstimator] Unhandled estimator enumerator.");
    }
}

/* ------------------------------------------------------------------ */
/* the integrator                                                      */
/* ------------------------------------------------------------------ */
#define MAXPDF 8
#define MAXOBS 16

typedef struct {
    obsdef def;
    int acc_type, blocksize, nskip, flag_equil, estimator;
} obsentry;

typedef struct {
    double *x, *xn, *orig;
    int *cidx;
    int nchanged, accepted;
    double *step; /* [ntypes]: step sizes of the move (MultiStepMove: of its sub-move) */
    normstate nd_move[3]; /* the move's distribution: its normal_distribution and those of its gamma members */
    drawsrc ds;
    int64_t acc, rej;
    double *po[MAXPDF], *pn[MAXPDF];
    double *spo[MAXPDF], *spn[MAXPDF];
    uint8_t *bits;
    double *marg;  /* recorded with the bits: log(u) - log(acceptance), accepted iff <= 0 */
    int64_t nbits, capbits, main_start;
    int err;
    /* results of the last integrate */
    double *avg, *erv;
    double *obsdata[MAXOBS];
    int64_t obsdata_len[MAXOBS];
} chainst;

struct orc_mci {
    int ndim, nchains;
    /* move */
    int movetype, srrd, veclen, ntypes, *typeEnds;
    /* MultiStepMove parameters (MultiStepMove.hpp:23-74) */
    int ms_nsteps, ms_srrd, ms_veclen;
    int ms_npdf;
    pdfdef ms_pdf[MAXPDF];
    /* pdfs, observables */
    int npdf;
    pdfdef pdf[MAXPDF];
    int nobs;
    obsentry obs[MAXOBS];
    /* domain */
    int periodic;
    double *lb, *ub;
    /* settings (MCIntegrator.cpp:624-649) */
    double target;
    int nfind;
    int64_t ndecorr;
    int recording;
    chainst *ch;
};

static int nobsdim(const orc_mci *h)
{
    int n = 0;
    for (int i = 0; i < h->nobs; ++i) { n += h->obs[i].def.nobs; }
    return n;
}

static void chain_alloc_protos(orc_mci *h, chainst *c)
{
    for (int k = 0; k < MAXPDF; ++k) {
        free(c->po[k]); free(c->pn[k]); free(c->spo[k]); free(c->spn[k]);
        c->po[k] = c->pn[k] = c->spo[k] = c->spn[k] = NULL;
    }
    for (int k = 0; k < h->npdf; ++k) {
        c->po[k] = (double *)calloc((size_t)h->pdf[k].nproto, sizeof(double));
        c->pn[k] = (double *)calloc((size_t)h->pdf[k].nproto, sizeof(double));
    }
    for (int k = 0; k < h->ms_npdf; ++k) {
        c->spo[k] = (double *)calloc((size_t)h->ms_pdf[k].nproto, sizeof(double));
        c->spn[k] = (double *)calloc((size_t)h->ms_pdf[k].nproto, sizeof(double));
    }
}

orc_mci *orc_create(int ndim, int nchains)
{
    if (ndim < 1 || nchains < 1) {
        fail(MCIG_ERR_INVALID_ARGUMENT, "ndim and nchains must be >= 1");
        return NULL;
    }
    orc_mci *h = (orc_mci *)calloc(1, sizeof(orc_mci));
    h->ndim = ndim;
    h->nchains = nchains;
    h->target = 0.5;
    h->nfind = -50;
    h->ndecorr = -10000;
    h->movetype = MCIG_MOVE_ALL;
    h->srrd = MCIG_SRRD_UNIFORM;
    h->veclen = 0;
    h->ntypes = 1;
    h->typeEnds = (int *)malloc(sizeof(int));
    h->typeEnds[0] = ndim;
    h->ch = (chainst *)calloc((size_t)nchains, sizeof(chainst));
    for (int c = 0; c < nchains; ++c) {
        chainst *s = &h->ch[c];
        s->x = (double *)calloc((size_t)ndim, sizeof(double));
        s->xn = (double *)calloc((size_t)ndim, sizeof(double));
        s->orig = (double *)calloc((size_t)ndim, sizeof(double));
        s->cidx = (int *)calloc((size_t)ndim, sizeof(int));
        s->step = (double *)malloc(sizeof(double));
        s->step[0] = 0.05; /* DEFAULT_MRT2STEP (Factories.hpp:145) */
        mt_seed(&s->ds.mt, 5489ULL);
    }
    return h;
}

static void chain_free_results(orc_mci *h, chainst *c)
{
    (void)h;
    free(c->avg); free(c->erv);
    c->avg = c->erv = NULL;
    for (int o = 0; o < MAXOBS; ++o) { free(c->obsdata[o]); c->obsdata[o] = NULL; c->obsdata_len[o] = 0; }
}

void orc_destroy(orc_mci *h)
{
    if (!h) { return; }
    for (int c = 0; c < h->nchains; ++c) {
        chainst *s = &h->ch[c];
        free(s->x); free(s->xn); free(s->orig); free(s->cidx); free(s->step);
        free(s->ds.rec); free(s->bits); free(s->marg); free(s->ds.pbuf);
        for (int k = 0; k < MAXPDF; ++k) { free(s->po[k]); free(s->pn[k]); free(s->spo[k]); free(s->spn[k]); }
        chain_free_results(h, s);
    }
    for (int k = 0; k < h->npdf; ++k) { pdf_free(&h->pdf[k]); }
    for (int k = 0; k < h->ms_npdf; ++k) { pdf_free(&h->ms_pdf[k]); }
    for (int o = 0; o < h->nobs; ++o) { obs_free(&h->obs[o].def); }
    free(h->typeEnds); free(h->lb); free(h->ub);
    free(h->ch);
    free(h);
}

int orc_set_seeds(orc_mci *h, const uint64_t *seeds)
{
    for (int c = 0; c < h->nchains; ++c) { mt_seed(&h->ch[c].ds.mt, seeds[c]); }
    return MCIG_OK;
}

/* OrthoPeriodicDomain::applyDomain(double x[]) (OrthoPeriodicDomain.cpp:38-48) */
static void domain_apply_all(const orc_mci *h, double *x)
{
    if (!h->periodic) { return; }
    for (int i = 0; i < h->ndim; ++i) {
        while (x[i] < h->lb[i]) { x[i] += h->ub[i] - h->lb[i]; }
        while (x[i] > h->ub[i]) { x[i] -= h->ub[i] - h->lb[i]; }
    }
}

/* OrthoPeriodicDomain::applyDomain(WalkerState&) (:50-61) */
static void domain_apply_sel(const orc_mci *h, double *xn, int nchanged, const int *cidx)
{
    if (!h->periodic) { return; }
    for (int i = 0; i < nchanged; ++i) {
        const int k = cidx[i];
        while (xn[k] < h->lb[k]) { xn[k] += h->ub[k] - h->lb[k]; }
        while (xn[k] > h->ub[k]) { xn[k] -= h->ub[k] - h->lb[k]; }
    }
}

int orc_set_x(orc_mci *h, const double *x)
{
    for (int c = 0; c < h->nchains; ++c) {
        memcpy(h->ch[c].x, x + (size_t)c * h->ndim, (size_t)h->ndim * sizeof(double));
        domain_apply_all(h, h->ch[c].x); /* MCI::setX (MCIntegrator.cpp:600-604) */
    }
    return MCIG_OK;
}

int orc_get_x(orc_mci *h, double *x)
{
    for (int c = 0; c < h->nchains; ++c) { memcpy(x + (size_t)c * h->ndim, h->ch[c].x, (size_t)h->ndim * sizeof(double)); }
    return MCIG_OK;
}

static int nstepsizes(const orc_mci *h) { return h->ntypes; }

int orc_set_mrt2step(orc_mci *h, double v)
{
    for (int c = 0; c < h->nchains; ++c) {
        for (int i = 0; i < nstepsizes(h); ++i) { h->ch[c].step[i] = v; }
    }
    return MCIG_OK;
}

int orc_set_mrt2step_i(orc_mci *h, int i, double v)
{
    if (i < 0 || i >= nstepsizes(h)) { return MCIG_OK; } /* MCI::setMRT2Step warns only (:564-572) */
    for (int c = 0; c < h->nchains; ++c) { h->ch[c].step[i] = v; }
    return MCIG_OK;
}

int orc_get_mrt2step(orc_mci *h, int chain, int i, double *v)
{
    *v = (i >= 0 && i < nstepsizes(h)) ? h->ch[chain].step[i] : 0.; /* MCI::getMRT2Step (:581-585) */
    return MCIG_OK;
}

int orc_set_target_acceptance_rate(orc_mci *h, double r) { h->target = r; return MCIG_OK; }
int orc_set_nfind_mrt2_iterations(orc_mci *h, int n) { h->nfind = n; return MCIG_OK; }
int orc_set_ndecorrelation_steps(orc_mci *h, int64_t n) { h->ndecorr = n; return MCIG_OK; }

static void reset_steps(orc_mci *h, int ntypes, double v)
{
    for (int c = 0; c < h->nchains; ++c) {
        free(h->ch[c].step);
        h->ch[c].step = (double *)malloc((size_t)ntypes * sizeof(double));
        for (int i = 0; i < ntypes; ++i) { h->ch[c].step[i] = v; }
        for (int k = 0; k < 3; ++k) { h->ch[c].nd_move[k].avail = 0; } /* a new move object has a fresh distribution */
    }
}

/* MCI::setTrialMove(SRRDType, veclen, ntypes, typeEnds) (MCIntegrator.cpp:431-446) and
 * setTrialMove(MoveType) (:423-429) via the factories (Factories.hpp:148-227) */
int orc_set_trial_move(orc_mci *h, int movetype, int srrd, int veclen, int ntypes, const int *typeEnds)
{
    if (srrd < MCIG_SRRD_UNIFORM || srrd > MCIG_SRRD_FISHER) { return fail(MCIG_ERR_INVALID_ARGUMENT, "unknown SRRDType"); }
    if (movetype == MCIG_MOVE_MULTISTEP) { return orc_set_multistep_move(h, h->ndim, MCIG_SRRD_UNIFORM, 1, 0.05); }
    if (ntypes < 1) { ntypes = 1; }
    int vl = (movetype == MCIG_MOVE_VEC) ? (veclen < 1 ? 1 : veclen) : 0;
    if (vl > 0 && h->ndim % vl != 0) { return fail(MCIG_ERR_INVALID_ARGUMENT, "[MCI::setTrialMove] MCI's number of walkers must be a multiple of passed veclen."); }
    if (ntypes > 1 && typeEnds == NULL) { return fail(MCIG_ERR_INVALID_ARGUMENT, "[TypedMoveInterface] When ntypes>1, passed typeEnds must not be null."); }
    if (ntypes > 1 && vl > 0) {
        for (int i = 0; i < ntypes; ++i) {
            if (typeEnds[i] % vl != 0) { return fail(MCIG_ERR_INVALID_ARGUMENT, "[SRRDVecMove] All type end indices must be multiples of vector length."); }
        }
    }
    free(h->typeEnds);
    h->typeEnds = (int *)malloc((size_t)ntypes * sizeof(int));
    if (ntypes > 1) { memcpy(h->typeEnds, typeEnds, (size_t)ntypes * sizeof(int)); }
    else { h->typeEnds[0] = h->ndim; }
    h->movetype = (vl > 0) ? MCIG_MOVE_VEC : MCIG_MOVE_ALL;
    h->srrd = srrd;
    h->veclen = vl;
    h->ntypes = ntypes;
    reset_steps(h, ntypes, 0.05);
    return MCIG_OK;
}

/* MultiStepMove(ndim, nsteps) with a sub-move SRRDVecMove(ndim/veclen, veclen, step)
 * (MultiStepMove.hpp:23-74); its step sizes are the sub-move's. */
int orc_set_multistep_move(orc_mci *h, int nsteps, int sub_srrd, int sub_veclen, double sub_step)
{
    if (sub_srrd != MCIG_SRRD_UNIFORM && sub_srrd != MCIG_SRRD_GAUSSIAN) { return fail(MCIG_ERR_UNSUPPORTED, "only uniform and gaussian sub-moves"); }
    if (sub_veclen < 1 || h->ndim % sub_veclen != 0) { return fail(MCIG_ERR_INVALID_ARGUMENT, "bad sub-move vector length"); }
    for (int k = 0; k < h->ms_npdf; ++k) { pdf_free(&h->ms_pdf[k]); }
    h->ms_npdf = 0;
    h->movetype = MCIG_MOVE_MULTISTEP;
    h->ms_nsteps = nsteps;
    h->ms_srrd = sub_srrd;
    h->ms_veclen = sub_veclen;
    h->ntypes = 1;
    free(h->typeEnds);
    h->typeEnds = (int *)malloc(sizeof(int));
    h->typeEnds[0] = h->ndim;
    reset_steps(h, 1, sub_step);
    return MCIG_OK;
}

int orc_multistep_add_pdf(orc_mci *h, int kind, const double *params, int nparams)
{
    if (h->movetype != MCIG_MOVE_MULTISTEP) { return fail(MCIG_ERR_INVALID_ARGUMENT, "no multi-step move set"); }
    if (h->ms_npdf >= MAXPDF) { return fail(MCIG_ERR_INVALID_ARGUMENT, "too many sub-pdfs"); }
    int rc = pdf_init(&h->ms_pdf[h->ms_npdf], kind, h->ndim, params, nparams);
    if (rc) { return rc; }
    ++h->ms_npdf;
    return MCIG_OK;
}

int orc_add_sampling_function(orc_mci *h, int kind, const double *params, int nparams)
{
    if (h->npdf >= MAXPDF) { return fail(MCIG_ERR_INVALID_ARGUMENT, "too many sampling functions"); }
    int rc = pdf_init(&h->pdf[h->npdf], kind, h->ndim, params, nparams);
    if (rc) { return rc; }
    ++h->npdf;
    return MCIG_OK;
}

int orc_pop_sampling_function(orc_mci *h)
{
    if (h->npdf > 0) { pdf_free(&h->pdf[--h->npdf]); }
    return MCIG_OK;
}

int orc_clear_sampling_functions(orc_mci *h)
{
    while (h->npdf > 0) { pdf_free(&h->pdf[--h->npdf]); }
    return MCIG_OK;
}

/* MCI::addObservable (MCIntegrator.cpp:451-465) with createAccumulator (Factories.hpp:24-38) */
int orc_add_observable(orc_mci *h, int kind, const double *params, int nparams, int blocksize, int nskip,
                       int flag_equil, int estimator)
{
    if (h->nobs >= MAXOBS) { return fail(MCIG_ERR_INVALID_ARGUMENT, "too many observables"); }
    if (blocksize < 0) { blocksize = 0; }
    if (nskip < 1) { nskip = 1; }
    if (flag_equil && estimator == MCIG_EST_NOOP) {
        return fail(MCIG_ERR_INVALID_ARGUMENT, "[MCI::addObservable] Requested automatic observable equilibration requires estimator with error calculation.");
    }
    if (estimator < MCIG_EST_NOOP || estimator > MCIG_EST_MJBLOCKER) { return fail(MCIG_ERR_DOMAIN, "[createEstimator] Unhandled estimator enumerator."); }
    obsentry *e = &h->obs[h->nobs];
    int rc = obs_init(&e->def, kind, h->ndim, params, nparams);
    if (rc) { return rc; }
    e->def.pdf = h->pdf;
    e->def.npdf = &h->npdf;
    e->acc_type = (blocksize == 0) ? MCIG_ACC_SIMPLE : (blocksize == 1 ? MCIG_ACC_FULL : MCIG_ACC_BLOCK);
    e->blocksize = blocksize;
    e->nskip = nskip;
    e->flag_equil = flag_equil;
    e->estimator = estimator;
    ++h->nobs;
    return MCIG_OK;
}

int orc_pop_observable(orc_mci *h)
{
    if (h->nobs > 0) { obs_free(&h->obs[--h->nobs].def); }
    return MCIG_OK;
}

int orc_clear_observables(orc_mci *h)
{
    while (h->nobs > 0) { obs_free(&h->obs[--h->nobs].def); }
    return MCIG_OK;
}

int orc_get_nobsdim(orc_mci *h) { return nobsdim(h); }

int orc_set_irange(orc_mci *h, const double *lb, const double *ub)
{
    for (int i = 0; i < h->ndim; ++i) {
        if (!(ub[i] > lb[i])) { return fail(MCIG_ERR_INVALID_ARGUMENT, "[OrthoPeriodicDomain::checkBounds] All upper bounds must be truly greater than their corresponding lower bounds."); }
    }
    free(h->lb); free(h->ub);
    h->lb = (double *)malloc((size_t)h->ndim * sizeof(double));
    h->ub = (double *)malloc((size_t)h->ndim * sizeof(double));
    memcpy(h->lb, lb, (size_t)h->ndim * sizeof(double));
    memcpy(h->ub, ub, (size_t)h->ndim * sizeof(double));
    h->periodic = 1;
    for (int c = 0; c < h->nchains; ++c) { domain_apply_all(h, h->ch[c].x); }
    return MCIG_OK;
}

int orc_reset_domain(orc_mci *h)
{
    h->periodic = 0;
    return MCIG_OK;
}

int orc_set_record(orc_mci *h, int on)
{
    h->recording = on;
    for (int c = 0; c < h->nchains; ++c) {
        h->ch[c].ds.recording = on;
        h->ch[c].ds.rec_len = 0;
        h->ch[c].nbits = 0;
        h->ch[c].main_start = -1;
    }
    return MCIG_OK;
}

int64_t orc_get_tape(orc_mci *h, int chain, double *out, int64_t maxn)
{
    const chainst *c = &h->ch[chain];
    if (out) {
        const int64_t n = c->ds.rec_len < maxn ? c->ds.rec_len : maxn;
        memcpy(out, c->ds.rec, (size_t)n * sizeof(double));
    }
    return c->ds.rec_len;
}

int64_t orc_get_accept_bits(orc_mci *h, int chain, uint8_t *out, int64_t maxn, int64_t *main_start)
{
    const chainst *c = &h->ch[chain];
    if (out) {
        const int64_t n = c->nbits < maxn ? c->nbits : maxn;
        memcpy(out, c->bits, (size_t)n);
    }
    if (main_start) { *main_start = c->main_start; }
    return c->nbits;
}

int orc_set_replay(orc_mci *h, const double *tape, int64_t stride, const int64_t *lens)
{
    for (int c = 0; c < h->nchains; ++c) {
        h->ch[c].ds.tape = tape ? tape + (size_t)c * stride : NULL;
        h->ch[c].ds.tape_len = tape ? lens[c] : 0;
        h->ch[c].ds.tape_pos = 0;
        h->ch[c].ds.exhausted = 0;
    }
    return MCIG_OK;
}

/* Draws from the device kernels' Philox streams instead of the engine: chain c of this
 * oracle is device chain chain0 + c, key (seed lo, seed hi), step counter ctr0[c] (NULL:
 * 0).  layout 1: the float kernels' draws (mcig_common.cuh move_draws<float>, accept
 * on (0, 1]) evaluated in double from the same Philox words; layout 2: the double
 * kernels' draws (move_draws<double>, accept_draw<double>).  All-coordinate, vector and
 * MultiStepMove moves with uniform or Gaussian draws; layout 0 returns to the engine. */
int orc_set_philox(orc_mci *h, uint64_t seed, int64_t chain0, const uint64_t *ctr0, int layout)
{
    if (layout < 0 || layout > 2) { return fail(MCIG_ERR_INVALID_ARGUMENT, "layout must be 0, 1 or 2"); }
    const int srrd = h->movetype == MCIG_MOVE_MULTISTEP ? h->ms_srrd : h->srrd;
    if (layout && srrd != MCIG_SRRD_UNIFORM && srrd != MCIG_SRRD_GAUSSIAN) {
        return fail(MCIG_ERR_UNSUPPORTED, "Philox draws: moves with uniform or Gaussian draws");
    }
    for (int c = 0; c < h->nchains; ++c) {
        drawsrc *d = &h->ch[c].ds;
        d->philox = layout;
        d->pkey[0] = (uint32_t)seed;
        d->pkey[1] = (uint32_t)(seed >> 32);
        d->pchain = (uint32_t)(chain0 + c);
        d->pctr = ctr0 ? ctr0[c] : 0;
        d->pmove = h->movetype;
        d->psrrd = h->srrd;
        d->pveclen = h->veclen;
        d->pndim = h->ndim;
        d->pms_nsteps = h->ms_nsteps;
        d->pms_srrd = h->ms_srrd;
        d->pms_veclen = h->ms_veclen;
        free(d->pbuf);
        d->pbuf = layout ? (double *)calloc((size_t)(h->ms_nsteps + 1) * (h->ndim + 2), sizeof(double)) : NULL;
        d->pbuf_n = d->pbuf_pos = 0;
    }
    return MCIG_OK;
}

/* the chains' Philox step counters (steps taken since orc_set_philox set them) */
int orc_get_philox_counters(orc_mci *h, uint64_t *ctr)
{
    for (int c = 0; c < h->nchains; ++c) { ctr[c] = h->ch[c].ds.pctr; }
    return MCIG_OK;
}

/* per-chain step sizes steps[nchains][ntypes] (a chain restarted at another's state) */
int orc_set_chain_steps(orc_mci *h, const double *steps)
{
    for (int c = 0; c < h->nchains; ++c) {
        for (int t = 0; t < nstepsizes(h); ++t) { h->ch[c].step[t] = steps[(size_t)c * nstepsizes(h) + t]; }
    }
    return MCIG_OK;
}

/* the recorded steps' margins log(u) - log(acceptance) (accepted iff <= 0), in the order of
 * orc_get_accept_bits */
int64_t orc_get_margins(orc_mci *h, int chain, double *out, int64_t maxn)
{
    const chainst *c = &h->ch[chain];
    if (out) {
        const int64_t n = c->nbits < maxn ? c->nbits : maxn;
        memcpy(out, c->marg, (size_t)n * sizeof(double));
    }
    return c->nbits;
}

static void push_bit_margin(chainst *c, int b, double m)
{
    if (c->nbits == c->capbits) {
        c->capbits = c->capbits ? 2 * c->capbits : 4096;
        c->bits = (uint8_t *)realloc(c->bits, (size_t)c->capbits);
        c->marg = (double *)realloc(c->marg, (size_t)c->capbits * sizeof(double));
    }
    c->marg[c->nbits] = m;
    c->bits[c->nbits++] = (uint8_t)b;
}

static void push_bit(chainst *c, int b) { push_bit_margin(c, b, b ? -INFINITY : INFINITY); }

/* step size of x-index i (TypedMoveInterface::getStepSizeIndex, TypedMoveInterface.hpp:40-48) */
static int type_of(const orc_mci *h, int i)
{
    for (int t = 0; t < h->ntypes; ++t) {
        if (i < h->typeEnds[t]) { return t; }
    }
    return h->ntypes - 1;
}

/* SRRDVecMove::trialMove (SRRDVecMove.hpp:75-96) */
static void vec_move(const orc_mci *h, chainst *c, int srrd, int veclen, normstate *nd)
{
    const int nvecs = h->ndim / veclen;
    const int vidx = draw_index(&c->ds, nvecs);
    const int x0 = vidx * veclen;
    const int t = type_of(h, x0);
    for (int i = 0; i < veclen; ++i) {
        c->xn[x0 + i] = c->xn[x0 + i] + c->step[t] * draw_srrd(&c->ds, srrd, nd);
        c->cidx[i] = x0 + i;
    }
    c->nchanged = veclen;
}

/* SamplingFunctionContainer::computeAcceptance (SamplingFunctionContainer.cpp:41-48) */
static double pdfcont_accept(int npdf, const pdfdef *pdf, chainst *c, double **po, double **pn)
{
    double a = 1.;
    for (int k = 0; k < npdf; ++k) { a *= pdf_compute_acceptance(&pdf[k], c->xn, c->nchanged, c->cidx, po[k], pn[k]); }
    return a;
}

static void pdfcont_init(int npdf, const pdfdef *pdf, const double *x, double **po, double **pn)
{
    for (int k = 0; k < npdf; ++k) { /* ProtoFunctionInterface::initializeProtoValues (:40-44) */
        pdf_proto(&pdf[k], x, pn[k]);
        memcpy(po[k], pn[k], (size_t)pdf[k].nproto * sizeof(double));
    }
}

static void pdfcont_copy(int npdf, const pdfdef *pdf, double **dst, double **src)
{
    for (int k = 0; k < npdf; ++k) { memcpy(dst[k], src[k], (size_t)pdf[k].nproto * sizeof(double)); }
}

/* SamplingFunctionContainer::getOldSamplingFunction (SamplingFunctionContainer.cpp:32-39) */
static double pdfcont_old_value(int npdf, const pdfdef *pdf, double **po)
{
    double v = 1.;
    for (int k = 0; k < npdf; ++k) { v *= pdf_value(&pdf[k], po[k]); }
    return v;
}

/* MultiStepMove::trialMove (src/MultiStepMove.cpp:6-47) */
static double multistep_move(const orc_mci *h, chainst *c)
{
    const int nd = h->ndim;
    memcpy(c->orig, c->x, (size_t)nd * sizeof(double));
    pdfcont_init(h->ms_npdf, h->ms_pdf, c->x, c->spo, c->spn);
    const double oldPDF = pdfcont_old_value(h->ms_npdf, h->ms_pdf, c->spo);
    for (int s = 0; s < h->ms_nsteps; ++s) {
        vec_move(h, c, h->ms_srrd, h->ms_veclen, c->nd_move);
        const double pdfAcc = pdfcont_accept(h->ms_npdf, h->ms_pdf, c, c->spo, c->spn);
        const int acc = (draw_u01(&c->ds) <= pdfAcc * 1.);
        if (acc) {
            pdfcont_copy(h->ms_npdf, h->ms_pdf, c->spo, c->spn);
            memcpy(c->x, c->xn, (size_t)nd * sizeof(double));
        } else {
            pdfcont_copy(h->ms_npdf, h->ms_pdf, c->spn, c->spo);
            memcpy(c->xn, c->x, (size_t)nd * sizeof(double));
        }
    }
    const double newPDF = pdfcont_old_value(h->ms_npdf, h->ms_pdf, c->spo);
    memcpy(c->x, c->orig, (size_t)nd * sizeof(double));
    c->nchanged = nd;
    return oldPDF / newPDF;
}

/* MCI::doStepMRT2 (MCIntegrator.cpp:326-360) */
static void step_mrt2(const orc_mci *h, chainst *c)
{
    const int nd = h->ndim;
    double moveAcc = 1.;
    if (h->movetype == MCIG_MOVE_ALL) { /* SRRDAllMove::trialMove (SRRDAllMove.hpp:67-80) */
        int xi = 0;
        for (int t = 0; t < h->ntypes; ++t) {
            while (xi < h->typeEnds[t]) {
                c->xn[xi] = c->xn[xi] + c->step[t] * draw_srrd(&c->ds, h->srrd, c->nd_move);
                ++xi;
            }
        }
        c->nchanged = nd;
    } else if (h->movetype == MCIG_MOVE_VEC) {
        vec_move(h, c, h->srrd, h->veclen, c->nd_move);
    } else {
        moveAcc = multistep_move(h, c);
    }
    if (c->nchanged < nd) { domain_apply_sel(h, c->xn, c->nchanged, c->cidx); }
    else { domain_apply_all(h, c->xn); }
    const double pdfAcc = pdfcont_accept(h->npdf, h->pdf, c, c->po, c->pn);
    const double u = draw_u01(&c->ds);
    c->accepted = (u <= pdfAcc * moveAcc);
    if (c->accepted) { ++c->acc; } else { ++c->rej; }
    if (h->recording) { push_bit_margin(c, c->accepted, log(u) - log(pdfAcc * moveAcc)); }
    if (c->accepted) {
        pdfcont_copy(h->npdf, h->pdf, c->po, c->pn);
        memcpy(c->x, c->xn, (size_t)nd * sizeof(double));
    } else {
        pdfcont_copy(h->npdf, h->pdf, c->pn, c->po);
        memcpy(c->xn, c->x, (size_t)nd * sizeof(double));
    }
}

/* MCI::doStepRandom (MCIntegrator.cpp:362-376) with OrthoPeriodicDomain::scaleToDomain (:63-68) */
static void step_random(const orc_mci *h, chainst *c)
{
    for (int i = 0; i < h->ndim; ++i) { c->xn[i] = draw_u01(&c->ds); }
    for (int i = 0; i < h->ndim; ++i) { c->xn[i] = h->lb[i] + c->xn[i] * (h->ub[i] - h->lb[i]); }
    c->nchanged = h->ndim;
    c->accepted = 1;
    ++c->acc;
    if (h->recording) { push_bit(c, 1); }
    memcpy(c->x, c->xn, (size_t)h->ndim * sizeof(double));
}

/* MCI::initializeSampling (MCIntegrator.cpp:252-271) */
static void init_sampling(const orc_mci *h, chainst *c)
{
    c->acc = 0;
    c->rej = 0;
    memcpy(c->xn, c->x, (size_t)h->ndim * sizeof(double));
    c->nchanged = h->ndim;
    for (int i = 0; i < h->ndim; ++i) { c->cidx[i] = i; }
    c->accepted = 1;
    pdfcont_init(h->npdf, h->pdf, c->x, c->po, c->pn);
}

/* MCI::sample(npoints) (MCIntegrator.cpp:273-288) and sample(npoints, container, flagMC) (:290-321) */
static void sample(const orc_mci *h, chainst *c, int64_t n, accu *acc, int nacc)
{
    init_sampling(h, c);
    for (int64_t r = 0; r < n; ++r) {
        if (h->npdf > 0) { step_mrt2(h, c); }
        else { step_random(h, c); }
        for (int k = 0; k < nacc; ++k) { accu_accumulate(&acc[k], c->xn, c->accepted); }
    }
    for (int k = 0; k < nacc; ++k) { accu_finalize(&acc[k]); }
}

static double acc_rate(const chainst *c)
{
    return (c->acc > 0) ? (double)c->acc / ((double)c->acc + (double)c->rej) : 0.; /* MCI::getAcceptanceRate (:587-592) */
}

/* MCI::findMRT2Step (MCIntegrator.cpp:87-168), one rank */
static void find_mrt2step(const orc_mci *h, chainst *c)
{
    const int nstep = nstepsizes(h);
    const double d = sqrt(40000. * h->ndim);
    const int64_t MIN_STAT = (int64_t)(d > 100. ? d : 100.);
    const int MIN_CONS = 5;
    const double TOLERANCE = 0.05;
    const double SMALLEST = FLT_MIN;
    const double half = h->periodic ? 0. : 0.5 * (2. * (double)FLT_MAX); /* UnboundDomain sizes (UnboundDomain.hpp:34) */
    int cons = 0, counter = 0;
    while ((h->nfind < 0 && cons < MIN_CONS) || counter < h->nfind) {
        sample(h, c, MIN_STAT, NULL, 0);
        const double rate = acc_rate(c);
        if (fabs(rate - h->target) < TOLERANCE) { ++cons; } else { cons = 0; }
        double f = rate / h->target;
        f = (f > 0.5) ? f : 0.5;
        f = (f < 2.) ? f : 2.;
        for (int i = 0; i < nstep; ++i) { c->step[i] = c->step[i] * f; }
        for (int i = 0; i < h->ndim; ++i) {
            const int t = type_of(h, i);
            const double lim = h->periodic ? 0.5 * (h->ub[i] - h->lb[i]) : half;
            if (c->step[t] > lim) { c->step[t] = lim; }
        }
        for (int j = 0; j < nstep; ++j) {
            if (c->step[j] < SMALLEST) { c->step[j] = SMALLEST; }
        }
        ++counter;
        if (h->nfind < 0 && counter >= abs(h->nfind)) { break; }
    }
}

/* MCI::initialDecorrelation (MCIntegrator.cpp:171-247), one rank */
static int initial_decorrelation(const orc_mci *h, chainst *c)
{
    if (h->ndecorr > 0) {
        sample(h, c, h->ndecorr, NULL, 0);
        return MCIG_OK;
    }
    if (h->ndecorr == 0) { return MCIG_OK; }
    /* automatic: temporary container of the flag_equil observables, Full + Correlated */
    accu acc[MAXOBS];
    int idx[MAXOBS], ne = 0, nod = 0;
    for (int o = 0; o < h->nobs; ++o) {
        if (h->obs[o].flag_equil) { idx[ne++] = o; nod += h->obs[o].def.nobs; }
    }
    const double d = sqrt(40000. * h->ndim);
    const int64_t MIN_NMC = (int64_t)(d > 100. ? d : 100.);
    for (int k = 0; k < ne; ++k) {
        int rc = accu_alloc(&acc[k], &h->obs[idx[k]].def, MCIG_ACC_FULL, 1, 1, MIN_NMC);
        if (rc) { return rc; }
    }
    double *oa = (double *)calloc((size_t)(nod + 1), sizeof(double)), *oe = (double *)calloc((size_t)(nod + 1), sizeof(double));
    double *na = (double *)calloc((size_t)(nod + 1), sizeof(double)), *ne_ = (double *)calloc((size_t)(nod + 1), sizeof(double));
    int rc = MCIG_OK;
#define RESET_ACCS()                                                                                        \
    for (int k = 0; k < ne; ++k) {                                                                          \
        memset(acc[k].data, 0, (size_t)(acc[k].nstore * acc[k].obs->nobs) * sizeof(double));               \
        acc[k].stepidx = 0; acc[k].storeidx = 0; acc[k].bidx = 0; acc[k].skipidx = 0;                       \
        acc[k].nchanged = acc[k].obs->ndim;                                                                 \
    }
#define ESTIMATE(A, E)                                                                                      \
    {                                                                                                       \
        int off = 0;                                                                                        \
        for (int k = 0; k < ne && !rc; ++k) {                                                               \
            rc = orc_estimate(MCIG_EST_CORRELATED, acc[k].nstore, acc[k].obs->nobs, acc[k].data, A + off, E + off); \
            off += acc[k].obs->nobs;                                                                        \
        }                                                                                                   \
    }
    RESET_ACCS();
    sample(h, c, MIN_NMC, acc, ne);
    ESTIMATE(oa, oe);
    int loop = 1;
    int64_t count = 0;
    while (loop && !rc) {
        loop = 0;
        RESET_ACCS();
        sample(h, c, MIN_NMC, acc, ne);
        count += MIN_NMC;
        if (count >= llabs(h->ndecorr)) { break; } /* reference prints a warning here (:219-222) */
        ESTIMATE(na, ne_);
        for (int i = 0; i < nod; ++i) {
            if (fabs(oa[i] - na[i]) > 2 * sqrt(oe[i] * oe[i] + ne_[i] * ne_[i])) { loop = 1; break; }
        }
        memcpy(oa, na, (size_t)nod * sizeof(double));
        memcpy(oe, ne_, (size_t)nod * sizeof(double));
    }
#undef RESET_ACCS
#undef ESTIMATE
    for (int k = 0; k < ne; ++k) { accu_free(&acc[k]); }
    free(oa); free(oe); free(na); free(ne_);
    return rc;
}

typedef struct {
    orc_mci *h;
    int c0, c1;
    int64_t nmc;
    int do_find, do_decorr;
    int rc;
} job;

/* MCI::integrate (MCIntegrator.cpp:43-82) for one chain */
static int integrate_chain(orc_mci *h, int ci, int64_t nmc, int do_find, int do_decorr)
{
    chainst *c = &h->ch[ci];
    chain_alloc_protos(h, c);
    if (h->npdf > 0) {
        if (do_find) { find_mrt2step(h, c); }
        if (do_decorr) {
            int rc = initial_decorrelation(h, c);
            if (rc) { return rc; }
        }
    }
    chain_free_results(h, c);
    const int nod = nobsdim(h);
    c->avg = (double *)calloc((size_t)(nod + 1), sizeof(double));
    c->erv = (double *)calloc((size_t)(nod + 1), sizeof(double));
    if (nmc <= 0) { return MCIG_OK; }
    accu acc[MAXOBS];
    for (int o = 0; o < h->nobs; ++o) {
        int rc = accu_alloc(&acc[o], &h->obs[o].def, h->obs[o].acc_type, h->obs[o].blocksize, h->obs[o].nskip, nmc);
        if (rc) {
            for (int k = 0; k < o; ++k) { accu_free(&acc[k]); }
            return rc;
        }
    }
    if (h->recording) { c->main_start = c->nbits; }
    sample(h, c, nmc, acc, h->nobs);
    int off = 0, rc = MCIG_OK;
    for (int o = 0; o < h->nobs; ++o) {
        if (!rc) { rc = orc_estimate(h->obs[o].estimator, acc[o].nstore, acc[o].obs->nobs, acc[o].data, c->avg + off, c->erv + off); }
        off += acc[o].obs->nobs;
        c->obsdata_len[o] = acc[o].nstore * acc[o].obs->nobs;
        c->obsdata[o] = acc[o].data;
        acc[o].data = NULL;
        accu_free(&acc[o]);
    }
    if (h->npdf == 0) { /* volume scaling (:70-77) */
        double vol = 1.;
        for (int i = 0; i < h->ndim; ++i) { vol *= (h->ub[i] - h->lb[i]); }
        for (int i = 0; i < nod; ++i) { c->avg[i] *= vol; c->erv[i] *= vol; }
    }
    if (c->ds.exhausted) { return fail(MCIG_ERR_RUNTIME, "replay tape exhausted"); }
    return rc;
}

static void *job_run(void *arg)
{
    job *j = (job *)arg;
    j->rc = MCIG_OK;
    for (int c = j->c0; c < j->c1 && !j->rc; ++c) { j->rc = integrate_chain(j->h, c, j->nmc, j->do_find, j->do_decorr); }
    return NULL;
}

int orc_integrate(orc_mci *h, int64_t nmc, double *avg, double *err, int do_find, int do_decorr,
                  double *chain_avg, double *chain_err, int nthreads)
{
    if (h->npdf == 0 && !h->periodic) {
        return fail(MCIG_ERR_DOMAIN, "[MCI::integrate] Integrating over an infinite domain requires a sampling function.");
    }
    if (nthreads < 1) { nthreads = 1; }
    if (nthreads > h->nchains) { nthreads = h->nchains; }
    job *jobs = (job *)calloc((size_t)nthreads, sizeof(job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].h = h;
        jobs[t].c0 = (int)((int64_t)h->nchains * t / nthreads);
        jobs[t].c1 = (int)((int64_t)h->nchains * (t + 1) / nthreads);
        jobs[t].nmc = nmc;
        jobs[t].do_find = do_find;
        jobs[t].do_decorr = do_decorr;
    }
    if (nthreads == 1) { job_run(&jobs[0]); }
    else {
        for (int t = 0; t < nthreads; ++t) { pthread_create(&th[t], NULL, job_run, &jobs[t]); }
        for (int t = 0; t < nthreads; ++t) { pthread_join(th[t], NULL); }
    }
    int rc = MCIG_OK;
    for (int t = 0; t < nthreads; ++t) {
        if (jobs[t].rc && !rc) { rc = jobs[t].rc; }
    }
    free(th);
    free(jobs);
    if (rc) { return rc; }
    if (nmc <= 0) { return MCIG_OK; }
    const int nod = nobsdim(h);
    /* MPIMCI::integrate reduction (src/MPIMCI.cpp:85-92): mean of averages, sqrt(sum err^2)/n */
    for (int i = 0; i < nod; ++i) {
        double sa = 0., se = 0.;
        for (int c = 0; c < h->nchains; ++c) {
            sa += h->ch[c].avg[i];
            se += h->ch[c].erv[i] * h->ch[c].erv[i];
        }
        avg[i] = sa / h->nchains;
        err[i] = sqrt(se) / h->nchains;
    }
    if (chain_avg) {
        for (int c = 0; c < h->nchains; ++c) { memcpy(chain_avg + (size_t)c * nod, h->ch[c].avg, (size_t)nod * sizeof(double)); }
    }
    if (chain_err) {
        for (int c = 0; c < h->nchains; ++c) { memcpy(chain_err + (size_t)c * nod, h->ch[c].erv, (size_t)nod * sizeof(double)); }
    }
    return MCIG_OK;
}

double orc_get_acceptance_rate(orc_mci *h)
{
    int64_t a = 0, r = 0;
    for (int c = 0; c < h->nchains; ++c) { a += h->ch[c].acc; r += h->ch[c].rej; }
    return (a > 0) ? (double)a / ((double)a + (double)r) : 0.;
}

int orc_get_counts(orc_mci *h, int64_t *acc, int64_t *rej)
{
    for (int c = 0; c < h->nchains; ++c) { acc[c] = h->ch[c].acc; rej[c] = h->ch[c].rej; }
    return MCIG_OK;
}

int64_t orc_get_obs_data(orc_mci *h, int o, double *out, int64_t maxn)
{
    if (o < 0 || o >= h->nobs) { return -1; }
    const int64_t len = h->ch[0].obsdata_len[o];
    if (out) {
        for (int c = 0; c < h->nchains; ++c) {
            if ((c + 1) * len > maxn) { break; }
            memcpy(out + (size_t)c * len, h->ch[c].obsdata[o], (size_t)len * sizeof(double));
        }
    }
    return len * h->nchains;
}

int64_t orc_accumulate_walk(int obs_kind, const double *params, int nparams, int ndim, int blocksize, int nskip,
                            int64_t nsteps, const double *xs, const uint8_t *accepted, double *data, int64_t maxn)
{
    obsdef o;
    if (obs_init(&o, obs_kind, ndim, params, nparams)) { return -1; }
    if (blocksize < 0) { blocksize = 0; }
    if (nskip < 1) { nskip = 1; }
    const int type = (blocksize == 0) ? MCIG_ACC_SIMPLE : (blocksize == 1 ? MCIG_ACC_FULL : MCIG_ACC_BLOCK);
    accu a;
    if (accu_alloc(&a, &o, type, blocksize, nskip, nsteps)) { obs_free(&o); return -1; }
    for (int64_t i = 0; i < nsteps; ++i) { accu_accumulate(&a, xs + (size_t)i * ndim, accepted[i]); }
    accu_finalize(&a);
    const int64_t n = a.nstore * o.nobs;
    if (data) { memcpy(data, a.data, (size_t)(n < maxn ? n : maxn) * sizeof(double)); }
    accu_free(&a);
    obs_free(&o);
    return n;
}
