/*
 * oracle.c — serial CPU restatement of the reference's per-time-step dengue simulation.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline; see oracle.h). Written
 * from the reference's semantics, one agent / one event at a time in the reference's serial
 * order, with every random number taken from a keyed Philox4x32-10 stream:
 *   counter = { entity, step, (stream << 24) | sub, (xsub << 16) | instance },
 *   key     = { seed & 0xffffffff, seed >> 32 }.
 * u01(x) = ((x >> 8) + 1) * 2^-24 in (0, 1] (the range of curand_uniform);
 * bounded(x, n) = (x * n) >> 32 (stands in for curand() % n).
 *
 * Compile with -ffp-contract=off: every float expression below is evaluated exactly as
 * written, in IEEE single precision, as the device code is (-fmad=false).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- random stream */

enum {
    ST_INIT_H = 0, ST_INIT_M = 1, ST_SEED_H = 2, ST_SEED_M = 3, ST_PERM = 4,
    ST_H_REBIRTH = 5, ST_M_TILE = 6, ST_M_REBIRTH = 7,
    ST_FOI_HM = 8, ST_FOI_HM_LOCAL = 9, ST_FOI_HM_LONG = 10,
    ST_FOI_MH = 11, ST_FOI_MH_LOCAL = 12, ST_FOI_MH_LONG = 13,
    ST_INF_M_START = 14, ST_INF_M_TARGET = 15, ST_INF_M_EXP = 16,
    ST_INF_H_START = 17, ST_INF_H_TARGET = 18, ST_INF_H_EXP = 19,
    ST_INTRO_N = 20, ST_INTRO_TARGET = 21, ST_INTRO_EXP = 22
};

/* Philox4x32-10, Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as easy as 1, 2, 3"
 * (SC'11): ten rounds of two 32x32->64 multiplies, the key bumped by the Weyl constants
 * between rounds. */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void oracle_draw4(uint64_t seed, uint32_t instance, uint32_t stream, uint32_t entity, uint32_t step,
                  uint32_t sub, uint32_t xsub, uint32_t out[4])
{
    uint32_t ctr[4] = {entity, step, (stream << 24) | (sub & 0xFFFFFFu), (xsub << 16) | (instance & 0xFFFFu)};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    oracle_philox4x32_10(ctr, key, out);
}

static float u01(uint32_t x) { return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f); }
static uint32_t bounded(uint32_t x, uint32_t n) { return (uint32_t)(((uint64_t)x * n) >> 32); }

/* decimalResolve (cpp/nepidemic.cu:13-24): round up with probability frac(v). Returns the
 * rounded value as a float; callers convert. */
static float resolve(float v, uint32_t x)
{
    float fl = floorf(v);
    float frac = v - fl;
    return (u01(x) <= frac) ? ceilf(v) : fl;
}

static uint32_t perm_mix(uint32_t x, const uint32_t k[4], uint32_t mask, uint32_t h)
{
    for (int r = 0; r < 4; ++r) {
        x = (x * 0x9E3779B1u + k[r]) & mask;
        x ^= x >> h;
    }
    return x;
}

/* Bijection of [0, n): a keyed mix on the smallest power-of-two domain, cycle-walked back
 * into [0, n). Element j < k of the permutation is the j-th seeded individual. The reference
 * seeds the first k census indices (cpp/epidemicinitial.cu:48-49, 88-89), whose communities
 * are random; with a community-sorted census k distinct uniform picks are the equivalent. */
uint32_t oracle_perm(uint64_t seed, uint32_t instance, uint32_t species, uint32_t n, uint32_t j)
{
    if (n <= 1) return j;
    uint32_t b = 1;
    while (b < 32 && (1ull << b) < n) ++b;
    uint32_t mask = (b == 32) ? 0xFFFFFFFFu : ((1u << b) - 1u);
    uint32_t h = (b + 1) / 2;
    uint32_t k[4];
    oracle_draw4(seed, instance, ST_PERM, species, 0, 0, 0, k);
    uint32_t y = perm_mix(j, k, mask, h);
    while (y >= n) y = perm_mix(y, k, mask, h);
    return y;
}

/* ---------------------------------------------------------------- state */

struct oracle_sim {
    arbo_sim_param p;
    uint32_t S, P, N, M, T, tiles, instance;
    uint64_t seed;
    uint32_t t;
    uint32_t *csr_loc, *csr_to;
    uint32_t *nsize, *msize, *nloc, *mloc, *ncomm, *mcomm;
    float *cdfh, *cdfm, *survh, *survm, *etab;
    uint32_t ah, am, yh, dm;
    /* census */
    int32_t *n_age, *n_exposed, *n_recovery, *n_dage;
    float *n_ple;
    uint8_t *n_status, *n_strain, *n_imm;
    int32_t *m_age, *m_exposed, *m_dage;
    float *m_ple;
    uint8_t *m_dead, *m_status, *m_strain;
    int32_t *ledger;
    /* counters */
    uint32_t *infh, *infm, *inc, *ncnt, *mcnt, *transh, *transm;
    uint32_t diag[4];
    /* series */
    uint32_t *s_ninc, *s_ninf, *s_one, *s_ncount, *s_mcount, *s_minf, *s_spatial;
};

static void draw(const oracle_sim* o, uint32_t stream, uint32_t entity, uint32_t step, uint32_t sub,
                 uint32_t xsub, uint32_t out[4])
{
    oracle_draw4(o->seed, o->instance, stream, entity, step, sub, xsub, out);
}

/* Human bi-Weibull CDF at integer age (cpp/ndemographic.cu:13-29), evaluated in double and
 * rounded once to float. */
static float cdf_h_value(const arbo_sim_param* p, uint32_t a)
{
    double x = pow((double)a * (double)p->nScaleInfantMortality, (double)p->nShapeInfantMortality);
    if ((double)a >= (double)p->nLocWeibull)
        x += pow(((double)a - (double)p->nLocWeibull) / (double)p->nScaleLifeExpectancy,
                 (double)p->nShapeLifeExpectancy);
    return (float)(1.0 - exp(-x));
}

/* Mosquito Weibull CDF (cpp/mdemographic.cu:13-17). */
static float cdf_m_value(const arbo_sim_param* p, uint32_t a)
{
    double x = pow((double)a / (double)p->mScaleLifeExpectancy, (double)p->mShapeLifeExpectancy);
    return (float)(1.0 - exp(-x));
}

/* A CDF table runs from age 0 until its value first reaches 1.0f or until max_age; ages past
 * the end read the last entry (exact: the CDF is non-decreasing and bounded by 1). */
static float* build_cdf(const arbo_sim_param* p, int human, uint32_t max_age, uint32_t* size)
{
    float* t = (float*)malloc(sizeof(float) * ((size_t)max_age + 1));
    uint32_t n = 0;
    for (uint32_t a = 0; a <= max_age; ++a) {
        float v = human ? cdf_h_value(p, a) : cdf_m_value(p, a);
        t[n++] = v;
        if (v >= 1.0f) break;
    }
    *size = n;
    return t;
}

static float cdf_at(const float* t, uint32_t n, int32_t a)
{
    uint32_t i = (a < 0) ? 0u : (uint32_t)a;
    return t[i < n ? i : n - 1];
}

/* First age whose CDF reaches ple (INT32_MAX if none): the age at which the death test
 * "ple <= CDF(age)" first holds. Bookkeeping only — the oracle's own death test compares
 * ple with the table every step, as the reference does. */
static int32_t death_age(const float* t, uint32_t n, float ple)
{
    if (!(t[n - 1] >= ple)) return INT32_MAX;
    uint32_t lo = 0, hi = n - 1; /* t[hi] >= ple */
    while (lo < hi) {
        uint32_t mid = (lo + hi) / 2;
        if (t[mid] >= ple) hi = mid; else lo = mid + 1;
    }
    return (int32_t)lo;
}

static uint32_t comm_of(const uint32_t* loc, uint32_t P, uint32_t i)
{
    uint32_t lo = 0, hi = P; /* largest c with loc[c] <= i */
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) / 2;
        if (loc[mid] <= i) lo = mid; else hi = mid;
    }
    return lo;
}

oracle_sim* oracle_create(const arbo_sim_param* p, const arbo_csr* csr, const uint32_t* n_comm_size,
                          const uint32_t* m_comm_size, uint32_t max_time, uint64_t seed, uint32_t instance)
{
    oracle_sim* o = (oracle_sim*)calloc(1, sizeof(oracle_sim));
    o->p = *p;
    o->S = p->nStrains;
    o->P = csr->subPopTotal;
    o->N = (uint32_t)p->nSize;
    o->M = p->mSize;
    o->T = max_time;
    o->tiles = (o->M + ARBO_MOSQUITO_TILE - 1) / ARBO_MOSQUITO_TILE;
    o->seed = seed;
    o->instance = instance;
    uint32_t P = o->P, S = o->S, N = o->N, M = o->M, T = o->T;

    o->csr_loc = (uint32_t*)malloc(sizeof(uint32_t) * (P + 1));
    memcpy(o->csr_loc, csr->loc, sizeof(uint32_t) * (P + 1));
    o->csr_to = (uint32_t*)malloc(sizeof(uint32_t) * (csr->nnz ? csr->nnz : 1));
    if (csr->nnz) memcpy(o->csr_to, csr->to, sizeof(uint32_t) * csr->nnz);

    o->nsize = (uint32_t*)malloc(sizeof(uint32_t) * P);
    o->msize = (uint32_t*)malloc(sizeof(uint32_t) * P);
    memcpy(o->nsize, n_comm_size, sizeof(uint32_t) * P);
    memcpy(o->msize, m_comm_size, sizeof(uint32_t) * P);
    o->nloc = (uint32_t*)malloc(sizeof(uint32_t) * (P + 1));
    o->mloc = (uint32_t*)malloc(sizeof(uint32_t) * (P + 1));
    o->nloc[0] = 0; o->mloc[0] = 0;
    for (uint32_t c = 0; c < P; ++c) {
        o->nloc[c + 1] = o->nloc[c] + o->nsize[c];
        o->mloc[c + 1] = o->mloc[c] + o->msize[c];
    }
    o->ncomm = (uint32_t*)malloc(sizeof(uint32_t) * (N ? N : 1));
    o->mcomm = (uint32_t*)malloc(sizeof(uint32_t) * (M ? M : 1));
    for (uint32_t i = 0; i < N; ++i) o->ncomm[i] = comm_of(o->nloc, P, i);
    for (uint32_t i = 0; i < M; ++i) o->mcomm[i] = comm_of(o->mloc, P, i);

    /* Tables. Human ages reach at most 365*Y + 364 at init plus one per step. */
    o->yh = p->nMaxInitialAgeYears;
    o->dm = p->mMaxInitialAge;
    o->cdfh = build_cdf(p, 1, 365u * o->yh + 364u + T + 1u, &o->ah);
    o->cdfm = build_cdf(p, 0, o->dm + T + 1u, &o->am);
    /* Cumulative survival sums (cpp/demographicintial.cu:48-83): yearly for humans, daily for
     * mosquitoes, accumulated in float in index order. */
    o->survh = (float*)malloc(sizeof(float) * (o->yh + 1));
    o->survh[0] = 1.0f - cdf_at(o->cdfh, o->ah, 0);
    for (uint32_t y = 1; y <= o->yh; ++y)
        o->survh[y] = o->survh[y - 1] + (1.0f - cdf_at(o->cdfh, o->ah, (int32_t)(365u * y)));
    o->survm = (float*)malloc(sizeof(float) * (o->dm + 1));
    o->survm[0] = 1.0f - cdf_at(o->cdfm, o->am, 0);
    for (uint32_t d = 1; d <= o->dm; ++d)
        o->survm[d] = o->survm[d - 1] + (1.0f - cdf_at(o->cdfm, o->am, (int32_t)d));

    /* Seasonal expected mosquito population, capped at the slot count. */
    o->etab = (float*)malloc(sizeof(float) * (T + 1));
    for (uint32_t t = 0; t <= T; ++t) {
        double e = (double)p->mosBaseRatio * (double)p->nSize *
                   (1.0 + (double)p->seasonAmp * sin(2.0 * 3.14159265358979323846 *
                                                      ((double)t - (double)p->seasonPhase) / 365.0));
        if (e > (double)M) e = (double)M;
        if (e < 0.0) e = 0.0;
        o->etab[t] = (float)e;
    }

    size_t SP = (size_t)S * P;
    o->n_age = (int32_t*)calloc(N ? N : 1, 4);
    o->n_exposed = (int32_t*)calloc(N ? N : 1, 4);
    o->n_recovery = (int32_t*)calloc(N ? N : 1, 4);
    o->n_dage = (int32_t*)calloc(N ? N : 1, 4);
    o->n_ple = (float*)calloc(N ? N : 1, 4);
    o->n_status = (uint8_t*)calloc(N ? N : 1, 1);
    o->n_strain = (uint8_t*)calloc(N ? N : 1, 1);
    o->n_imm = (uint8_t*)calloc(N ? N : 1, 1);
    o->m_age = (int32_t*)calloc(M ? M : 1, 4);
    o->m_exposed = (int32_t*)calloc(M ? M : 1, 4);
    o->m_dage = (int32_t*)calloc(M ? M : 1, 4);
    o->m_ple = (float*)calloc(M ? M : 1, 4);
    o->m_dead = (uint8_t*)calloc(M ? M : 1, 1);
    o->m_status = (uint8_t*)calloc(M ? M : 1, 1);
    o->m_strain = (uint8_t*)calloc(M ? M : 1, 1);
    o->ledger = (int32_t*)calloc(o->tiles ? o->tiles : 1, 4);
    o->infh = (uint32_t*)calloc(SP, 4);
    o->infm = (uint32_t*)calloc(SP, 4);
    o->inc = (uint32_t*)calloc(SP, 4);
    o->transh = (uint32_t*)calloc(SP, 4);
    o->transm = (uint32_t*)calloc(SP, 4);
    o->ncnt = (uint32_t*)calloc(P, 4);
    o->mcnt = (uint32_t*)calloc(P, 4);
    size_t R = (size_t)T + 1;
    o->s_ninc = (uint32_t*)calloc(R * S, 4);
    o->s_ninf = (uint32_t*)calloc(R * S, 4);
    o->s_one = (uint32_t*)calloc(R * S, 4);
    o->s_minf = (uint32_t*)calloc(R * S, 4);
    o->s_ncount = (uint32_t*)calloc(R, 4);
    o->s_mcount = (uint32_t*)calloc(R, 4);
    o->s_spatial = p->recordSpatial ? (uint32_t*)calloc(R * SP, 4) : NULL;
    return o;
}

void oracle_destroy(oracle_sim* o)
{
    if (!o) return;
    void* ptrs[] = {o->csr_loc, o->csr_to, o->nsize, o->msize, o->nloc, o->mloc, o->ncomm, o->mcomm,
                    o->cdfh, o->cdfm, o->survh, o->survm, o->etab, o->n_age, o->n_exposed, o->n_recovery,
                    o->n_dage, o->n_ple, o->n_status, o->n_strain, o->n_imm, o->m_age, o->m_exposed,
                    o->m_dage, o->m_ple, o->m_dead, o->m_status, o->m_strain, o->ledger, o->infh, o->infm,
                    o->inc, o->transh, o->transm, o->ncnt, o->mcnt, o->s_ninc, o->s_ninf, o->s_one,
                    o->s_minf, o->s_ncount, o->s_mcount, o->s_spatial};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
    free(o);
}

void oracle_set_expected(oracle_sim* o, const float* e, uint32_t n)
{
    for (uint32_t t = 0; t <= o->T && t < n; ++t) {
        float v = e[t];
        if (v > (float)o->M) v = (float)o->M;
        if (!(v >= 0.0f)) v = 0.0f;
        o->etab[t] = v;
    }
}

uint32_t oracle_time(const oracle_sim* o) { return o->t; }

/* dataCollect (cpp/datacollect.cu:79-189): sums over communities into series row r. */
static void collect(oracle_sim* o, uint32_t r)
{
    uint32_t S = o->S, P = o->P;
    for (uint32_t s = 0; s < S; ++s) {
        uint32_t ninf = 0, ninc = 0, minf = 0;
        for (uint32_t c = 0; c < P; ++c) {
            ninf += o->infh[s * P + c];
            ninc += o->inc[s * P + c];
            minf += o->infm[s * P + c];
        }
        o->s_ninf[r * S + s] = ninf;
        o->s_ninc[r * S + s] = ninc;
        o->s_minf[r * S + s] = minf;
        o->s_one[r * S + s] = o->infh[s * P + 0];
    }
    uint32_t nc = 0, mc = 0;
    for (uint32_t c = 0; c < P; ++c) { nc += o->ncnt[c]; mc += o->mcnt[c]; }
    o->s_ncount[r] = nc;
    o->s_mcount[r] = mc;
    if (o->s_spatial) memcpy(o->s_spatial + (size_t)r * S * P, o->infh, sizeof(uint32_t) * S * P);
}

/* demographicInitialization + epidemicInitial (cpp/demographicintial.cu:86-297,
 * cpp/epidemicinitial.cu:27-99). */
void oracle_init(oracle_sim* o)
{
    const arbo_sim_param* p = &o->p;
    uint32_t S = o->S, P = o->P, N = o->N, M = o->M, T = o->T;
    uint32_t r[4], r1[4], r2[4];
    o->t = 0;
    memset(o->diag, 0, sizeof(o->diag));
    memset(o->infh, 0, sizeof(uint32_t) * S * P);
    memset(o->infm, 0, sizeof(uint32_t) * S * P);
    memset(o->inc, 0, sizeof(uint32_t) * S * P);
    memset(o->transh, 0, sizeof(uint32_t) * S * P);
    memset(o->transm, 0, sizeof(uint32_t) * S * P);
    size_t R = (size_t)T + 1;
    memset(o->s_ninc, 0, R * S * 4); memset(o->s_ninf, 0, R * S * 4); memset(o->s_one, 0, R * S * 4);
    memset(o->s_minf, 0, R * S * 4); memset(o->s_ncount, 0, R * 4); memset(o->s_mcount, 0, R * 4);
    if (o->s_spatial) memset(o->s_spatial, 0, R * S * P * 4);

    /* Humans (cpp/demographicintial.cu:109-179). */
    for (uint32_t j = 0; j < N; ++j) {
        draw(o, ST_INIT_H, j, 0, 0, 0, r);
        draw(o, ST_INIT_H, j, 0, 1, 0, r1);
        draw(o, ST_INIT_H, j, 0, 2, 0, r2);
        uint32_t d[12] = {r[0], r[1], r[2], r[3], r1[0], r1[1], r1[2], r1[3], r2[0], r2[1], r2[2], r2[3]};
        float randCSF = o->survh[o->yh] * u01(d[0]);
        uint32_t y = 0;
        while (y < o->yh && !(randCSF <= o->survh[y])) ++y;
        int32_t age = (int32_t)(365u * y + bounded(d[1], 365u));
        float base = cdf_at(o->cdfh, o->ah, age != 0 ? age - 1 : 0);
        float ple = (1.0f - base) * u01(d[2]) + base;
        uint8_t imm = 0;
        for (uint32_t s = 0; s < S; ++s)
            if (u01(d[3 + s]) < p->initialSeroPrev) imm |= (uint8_t)(1u << s);
        o->n_age[j] = age;
        o->n_ple[j] = ple;
        o->n_dage[j] = death_age(o->cdfh, o->ah, ple);
        o->n_status[j] = 0;
        o->n_strain[j] = 0;
        o->n_imm[j] = imm;
        o->n_exposed[j] = 0;
        o->n_recovery[j] = 0;
    }
    for (uint32_t c = 0; c < P; ++c) o->ncnt[c] = o->nsize[c];

    /* Mosquitoes (cpp/demographicintial.cu:221-296). */
    float alive_p = o->etab[0] / (float)M;
    for (uint32_t b = 0; b < o->tiles; ++b) o->ledger[b] = 0;
    for (uint32_t c = 0; c < P; ++c) o->mcnt[c] = o->msize[c];
    for (uint32_t j = 0; j < M; ++j) {
        draw(o, ST_INIT_M, j, 0, 0, 0, r);
        o->m_status[j] = 0;
        o->m_strain[j] = 0;
        o->m_exposed[j] = 0;
        if (!(u01(r[0]) < alive_p)) {
            o->m_dead[j] = 1;
            o->m_age[j] = 0;
            o->m_ple[j] = 0.0f;
            o->m_dage[j] = 0;
            o->ledger[j / ARBO_MOSQUITO_TILE] += 1;
            o->mcnt[o->mcomm[j]] -= 1;
        } else {
            float randCSF = o->survm[o->dm] * u01(r[1]);
            uint32_t a = 0;
            while (a < o->dm && !(randCSF <= o->survm[a])) ++a;
            float base = cdf_at(o->cdfm, o->am, a != 0 ? (int32_t)a - 1 : 0);
            float ple = (1.0f - base) * u01(r[2]) + base;
            o->m_dead[j] = 0;
            o->m_age[j] = (int32_t)a;
            o->m_ple[j] = ple;
            o->m_dage[j] = death_age(o->cdfm, o->am, ple);
        }
    }

    /* Seeded infections (cpp/epidemicinitial.cu:27-99). */
    uint32_t kh = (uint32_t)p->nInitialInf;
    if (kh > N) kh = N;
    for (uint32_t j = 0; j < kh; ++j) {
        uint32_t i = oracle_perm(o->seed, o->instance, 0, N, j);
        draw(o, ST_SEED_H, j, 0, 0, 0, r);
        uint32_t s = bounded(r[0], S);
        o->n_status[i] = 2;
        o->n_strain[i] = (uint8_t)s;
        o->n_imm[i] |= (uint8_t)(1u << s);
        uint32_t rr = (uint32_t)resolve(p->recovery, r[2]);
        uint32_t m = (rr > 1u) ? rr - 1u : 1u;
        int32_t dur = (int32_t)(bounded(r[1], m) + 1u);
        o->n_recovery[i] = (p->quirks & ARBO_QUIRK_SEED_RECOVERY_DURATION) ? dur : o->n_age[i] + dur;
        o->infh[s * P + o->ncomm[i]] += 1;
    }
    uint32_t km = (uint32_t)p->mInitialInf;
    if (km > M) km = M;
    for (uint32_t j = 0; j < km; ++j) {
        uint32_t i = oracle_perm(o->seed, o->instance, 1, M, j);
        if (o->m_dead[i] && !(p->quirks & ARBO_QUIRK_SEED_DEAD_MOSQUITO)) continue;
        draw(o, ST_SEED_M, j, 0, 0, 0, r);
        uint32_t s = bounded(r[0], S);
        o->m_status[i] = 2;
        o->m_strain[i] = (uint8_t)s;
        o->infm[s * P + o->mcomm[i]] += 1;
    }
    collect(o, 0);
}

/* nBlockBirthDeath (cpp/ndemographic.cu:32-105). */
static void demog_humans(oracle_sim* o, uint32_t t)
{
    uint32_t P = o->P;
    uint32_t r[4];
    for (uint32_t i = 0; i < o->N; ++i) {
        int32_t a = ++o->n_age[i];
        uint8_t st = o->n_status[i];
        uint32_t c = o->ncomm[i];
        if (o->n_ple[i] > cdf_at(o->cdfh, o->ah, a)) {
            if (st == 2 && o->n_recovery[i] < a) {
                o->infh[o->n_strain[i] * P + c] -= 1;
                o->n_status[i] = 0;
            } else if (st == 1 && o->n_exposed[i] < a) {
                o->inc[o->n_strain[i] * P + c] += 1;
                o->infh[o->n_strain[i] * P + c] += 1;
                o->n_status[i] = 2;
            }
        } else {
            if (st == 2) o->infh[o->n_strain[i] * P + c] -= 1;
            draw(o, ST_H_REBIRTH, i >> 2, t, 0, 0, r);
            o->n_age[i] = 0;
            o->n_status[i] = 0;
            o->n_ple[i] = u01(r[i & 3]);
            o->n_dage[i] = death_age(o->cdfh, o->ah, o->n_ple[i]);
            o->n_imm[i] = 0;
        }
    }
}

/* mBlockBirthDeath (cpp/mdemographic.cu:22-150) on logical 128-slot tiles: deaths, the
 * tile's stochastic birth quota from the carried dead count, rebirth of dead slots in a fixed
 * order, then the net change of each community's alive count. The reference reborns whichever
 * dead slots win a shared-memory ticket race (cpp/mdemographic.cu:135); here the lowest-index
 * dead slots of the tile are reborn first. Draws: the quota of tile b is component b&3 of the
 * call keyed (b>>2, t); the r-th reborn slot of tile b takes component r&3 of the call keyed
 * (b, t, r>>2). */
static void demog_mosquitoes(oracle_sim* o, uint32_t t)
{
    uint32_t M = o->M, P = o->P;
    float E = o->etab[t + 1];
    uint32_t r[4];
    int32_t net[ARBO_MOSQUITO_TILE];
    for (uint32_t b = 0; b < o->tiles; ++b) {
        uint32_t i0 = b * ARBO_MOSQUITO_TILE;
        uint32_t bt = M - i0 < ARBO_MOSQUITO_TILE ? M - i0 : ARBO_MOSQUITO_TILE;
        uint32_t deaths = 0;
        for (uint32_t k = 0; k < bt; ++k) {
            uint32_t i = i0 + k;
            net[k] = 0;
            if (o->m_dead[i]) continue;
            int32_t a = ++o->m_age[i];
            uint8_t st = o->m_status[i];
            uint32_t c = o->mcomm[i];
            if (o->m_ple[i] <= cdf_at(o->cdfm, o->am, a)) {
                if (st == 2) o->infm[o->m_strain[i] * P + c] -= 1;
                o->m_dead[i] = 1;
                net[k] = -1;
                deaths += 1;
            } else if (st == 1 && o->m_exposed[i] < a) {
                o->infm[o->m_strain[i] * P + c] += 1;
                o->m_status[i] = 2;
            }
        }
        uint32_t L = (uint32_t)o->ledger[b] + deaths;
        float fbt = (float)bt;
        float x = E * fbt;
        x = x / (float)M;
        x = x - fbt;
        x = x + (float)L;
        draw(o, ST_M_TILE, b >> 2, t, 0, 0, r);
        int32_t births = (int32_t)resolve(x, r[b & 3]);
        o->ledger[b] = (int32_t)L - births;
        int32_t rank = 0;
        for (uint32_t k = 0; k < bt; ++k) {
            uint32_t i = i0 + k;
            if (!o->m_dead[i]) continue;
            if (rank < births) {
                draw(o, ST_M_REBIRTH, b, t, (uint32_t)rank >> 2, 0, r);
                o->m_age[i] = 0;
                o->m_dead[i] = 0;
                o->m_status[i] = 0;
                o->m_ple[i] = u01(r[rank & 3]);
                o->m_dage[i] = death_age(o->cdfm, o->am, o->m_ple[i]);
                net[k] += 1;
            }
            rank += 1;
        }
        for (uint32_t k = 0; k < bt; ++k)
            if (net[k]) o->mcnt[o->mcomm[i0 + k]] += (uint32_t)net[k];
    }
}

/* Split of a source's events (cpp/nepidemic.cu:86-136): a noDistance share stays home, a
 * longDistance share of the rest goes to a uniform community, the remainder to a uniform
 * neighbour of the CSR row. An isolated community keeps all its events. */
static void scatter(oracle_sim* o, uint32_t* trans, uint32_t s, uint32_t c, uint32_t n, const uint32_t rr[4],
                    uint32_t st_local, uint32_t st_long, uint32_t t)
{
    uint32_t P = o->P, pidx = s * P + c, r[4];
    uint32_t loc = o->csr_loc[c];
    uint32_t deg = o->csr_loc[c + 1] - loc;
    uint32_t stay;
    if (deg > 0) {
        stay = (uint32_t)resolve((float)n * o->p.noDistance, rr[1]);
        n -= stay;
        uint32_t lng = (uint32_t)resolve((float)n * o->p.longDistance, rr[2]);
        n -= lng;
        for (uint32_t e = 0; e < n; ++e) {
            draw(o, st_local, pidx, t, e >> 2, 0, r);
            uint32_t dest = o->csr_to[loc + bounded(r[e & 3], deg)];
            trans[s * P + dest] += 1;
        }
        for (uint32_t e = 0; e < lng; ++e) {
            draw(o, st_long, pidx, t, e >> 2, 0, r);
            trans[s * P + bounded(r[e & 3], P)] += 1;
        }
    } else {
        stay = n;
    }
    trans[pidx] += stay;
}

/* nVisitingInfected / mVisitingInfected (cpp/nepidemic.cu:28-142, cpp/mepidemic.cu:28-138). */
static void force_of_infection(oracle_sim* o, uint32_t t)
{
    const arbo_sim_param* p = &o->p;
    uint32_t S = o->S, P = o->P, r[4];
    for (uint32_t s = 0; s < S; ++s) {
        for (uint32_t c = 0; c < P; ++c) {
            uint32_t pidx = s * P + c;
            if (o->infh[pidx] > 0) {
                draw(o, ST_FOI_HM, pidx, t, 0, 0, r);
                float ratio = (float)o->mcnt[c] / (float)o->ncnt[c];
                float x = ratio * p->bitingRate;
                x = x * p->nmBitingSuccess;
                x = x * (float)o->infh[pidx];
                uint32_t n = (uint32_t)resolve(x, r[0]);
                scatter(o, o->transm, s, c, n, r, ST_FOI_HM_LOCAL, ST_FOI_HM_LONG, t);
            }
            if (o->infm[pidx] > 0) {
                draw(o, ST_FOI_MH, pidx, t, 0, 0, r);
                float x = p->bitingRate * p->mnBitingSuccess;
                x = x * (float)o->infm[pidx];
                uint32_t n = (uint32_t)resolve(x, r[0]);
                scatter(o, o->transh, s, c, n, r, ST_FOI_MH_LOCAL, ST_FOI_MH_LONG, t);
            }
        }
    }
}

static void infect_human(oracle_sim* o, uint32_t i, uint32_t s, const uint32_t r[4])
{
    o->n_status[i] = 1;
    o->n_strain[i] = (uint8_t)s;
    o->n_imm[i] |= (uint8_t)(1u << s);
    int32_t ex = (int32_t)resolve((float)o->n_age[i] + o->p.nExposed, r[0]);
    o->n_exposed[i] = ex;
    o->n_recovery[i] = (int32_t)resolve((float)ex + o->p.recovery, r[1]);
}

static int human_eligible(const oracle_sim* o, uint32_t i, uint32_t s)
{
    return o->n_status[i] == 0 && !((o->n_imm[i] >> s) & 1u);
}

/* nmTransmission (cpp/mepidemic.cu:143-246) and mnTransmission (cpp/nepidemic.cu:146-319):
 * per community, serotypes from a random start, events in order. A mosquito event retries
 * dead slots (capped at maxTargetAttempt; an exhausted event is dropped and counted); a human
 * event is spent on whoever it hits. After each serotype's events come the external
 * introductions, retried until they land (at most maxIntroAttempt attempts). */
static void infections(oracle_sim* o, uint32_t t)
{
    const arbo_sim_param* p = &o->p;
    uint32_t S = o->S, P = o->P, r[4];
    for (uint32_t c = 0; c < P; ++c) {
        if (o->mcnt[c] == 0) continue;
        draw(o, ST_INF_M_START, c, t, 0, 0, r);
        uint32_t s = bounded(r[0], S);
        for (uint32_t j = 0; j < S; ++j) {
            uint32_t pidx = s * P + c;
            uint32_t k = o->transm[pidx];
            for (uint32_t e = 0; e < k; ++e) {
                uint32_t slot = 0;
                int found = 0;
                for (uint32_t a = 0; a < p->maxTargetAttempt; ++a) {
                    draw(o, ST_INF_M_TARGET, pidx, t, e, a >> 2, r);
                    slot = o->mloc[c] + bounded(r[a & 3], o->msize[c]);
                    if (!o->m_dead[slot]) { found = 1; break; }
                }
                if (!found) { o->diag[0] += 1; continue; }
                if (o->m_status[slot] == 0) {
                    draw(o, ST_INF_M_EXP, pidx, t, e >> 2, 0, r);
                    o->m_status[slot] = 1;
                    o->m_strain[slot] = (uint8_t)s;
                    o->m_exposed[slot] = (int32_t)resolve((float)o->m_age[slot] + p->mExposed, r[e & 3]);
                }
            }
            s = (s + 1) % S;
        }
    }
    for (uint32_t c = 0; c < P; ++c) {
        if (o->nsize[c] == 0) continue;
        draw(o, ST_INF_H_START, c, t, 0, 0, r);
        uint32_t s = bounded(r[0], S);
        for (uint32_t j = 0; j < S; ++j) {
            uint32_t pidx = s * P + c;
            uint32_t k = o->transh[pidx];
            for (uint32_t e = 0; e < k; ++e) {
                draw(o, ST_INF_H_TARGET, pidx, t, e >> 2, 0, r);
                uint32_t i = o->nloc[c] + bounded(r[e & 3], o->nsize[c]);
                if (human_eligible(o, i, s)) {
                    draw(o, ST_INF_H_EXP, pidx, t, e, 0, r);
                    infect_human(o, i, s, r);
                }
            }
            draw(o, ST_INTRO_N, pidx, t, 0, 0, r);
            uint32_t ne = (uint32_t)resolve(p->externalInfection / (float)P, r[0]);
            uint32_t a = 0;
            while (ne > 0 && a < p->maxIntroAttempt) {
                draw(o, ST_INTRO_TARGET, pidx, t, a >> 2, 0, r);
                uint32_t i = o->nloc[c] + bounded(r[a & 3], o->nsize[c]);
                if (human_eligible(o, i, s)) {
                    draw(o, ST_INTRO_EXP, pidx, t, a, 0, r);
                    infect_human(o, i, s, r);
                    ne -= 1;
                }
                a += 1;
            }
            if (ne > 0) o->diag[1] += 1;
            s = (s + 1) % S;
        }
    }
    memset(o->transh, 0, sizeof(uint32_t) * S * P);
    memset(o->transm, 0, sizeof(uint32_t) * S * P);
}

/* One iteration of the time loop (cpp/simulation.cpp:115-155). The series row of time t+1 is
 * taken right after the demographic passes: the epidemic pass changes no counter, so this is
 * the reference's dataCollect at the top of the next iteration. */
void oracle_step(oracle_sim* o, uint32_t nsteps)
{
    for (uint32_t k = 0; k < nsteps && o->t < o->T; ++k) {
        uint32_t t = o->t;
        demog_humans(o, t);
        demog_mosquitoes(o, t);
        collect(o, t + 1);
        memset(o->inc, 0, sizeof(uint32_t) * o->S * o->P);
        force_of_infection(o, t);
        infections(o, t);
        o->t = t + 1;
        o->diag[3] = o->t;
    }
}

void* oracle_census(oracle_sim* o, int field, uint32_t* n)
{
    *n = field <= ARBO_CENSUS_N_DEATH_AGE ? o->N : o->M;
    switch (field) {
    case ARBO_CENSUS_N_AGE: return o->n_age;
    case ARBO_CENSUS_N_EXPOSED: return o->n_exposed;
    case ARBO_CENSUS_N_IMMUNITY: return o->n_imm;
    case ARBO_CENSUS_N_STATUS: return o->n_status;
    case ARBO_CENSUS_N_PLE: return o->n_ple;
    case ARBO_CENSUS_N_RECOVERY: return o->n_recovery;
    case ARBO_CENSUS_N_STRAIN: return o->n_strain;
    case ARBO_CENSUS_N_DEATH_AGE: return o->n_dage;
    case ARBO_CENSUS_M_AGE: return o->m_age;
    case ARBO_CENSUS_M_DEAD: return o->m_dead;
    case ARBO_CENSUS_M_EXPOSED: return o->m_exposed;
    case ARBO_CENSUS_M_STATUS: return o->m_status;
    case ARBO_CENSUS_M_PLE: return o->m_ple;
    case ARBO_CENSUS_M_STRAIN: return o->m_strain;
    case ARBO_CENSUS_M_DEATH_AGE: return o->m_dage;
    default: *n = 0; return NULL;
    }
}

void* oracle_counters(oracle_sim* o, int kind, uint32_t* n)
{
    uint32_t SP = o->S * o->P;
    switch (kind) {
    case ARBO_COUNTER_N_INFECTED_SUBPOP: *n = SP; return o->infh;
    case ARBO_COUNTER_M_INFECTED_SUBPOP: *n = SP; return o->infm;
    case ARBO_COUNTER_N_INCIDENCE_SUBPOP: *n = SP; return o->inc;
    case ARBO_COUNTER_N_SUBPOP_COUNT: *n = o->P; return o->ncnt;
    case ARBO_COUNTER_M_SUBPOP_COUNT: *n = o->P; return o->mcnt;
    case ARBO_COUNTER_N_SUBPOP_LOC: *n = o->P + 1; return o->nloc;
    case ARBO_COUNTER_M_SUBPOP_LOC: *n = o->P + 1; return o->mloc;
    case ARBO_COUNTER_M_DEAD_COUNT: *n = o->tiles; return o->ledger;
    case ARBO_COUNTER_DIAG: *n = 4; return o->diag;
    default: *n = 0; return NULL;
    }
}

void* oracle_series(oracle_sim* o, int kind, uint32_t* n)
{
    uint32_t R = o->T + 1;
    switch (kind) {
    case ARBO_SERIES_N_INCIDENCE: *n = R * o->S; return o->s_ninc;
    case ARBO_SERIES_N_INFECTED: *n = R * o->S; return o->s_ninf;
    case ARBO_SERIES_ONE_SUBPOP: *n = R * o->S; return o->s_one;
    case ARBO_SERIES_N_COUNT: *n = R; return o->s_ncount;
    case ARBO_SERIES_M_COUNT: *n = R; return o->s_mcount;
    case ARBO_SERIES_M_INFECTED: *n = R * o->S; return o->s_minf;
    case ARBO_SERIES_INFECTED_SUBPOP: *n = o->s_spatial ? R * o->S * o->P : 0; return o->s_spatial;
    default: *n = 0; return NULL;
    }
}

float* oracle_table(oracle_sim* o, int which, uint32_t* n)
{
    switch (which) {
    case 0: *n = o->ah; return o->cdfh;
    case 1: *n = o->am; return o->cdfm;
    case 2: *n = o->yh + 1; return o->survh;
    case 3: *n = o->dm + 1; return o->survm;
    case 4: *n = o->T + 1; return o->etab;
    default: *n = 0; return NULL;
    }
}
