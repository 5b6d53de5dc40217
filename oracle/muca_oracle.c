/*
 * muca_oracle.c -- CPU oracle (test infrastructure only; see muca_oracle.h).
 *
 * Every function restates one reference routine literally: same integer and
 * floating-point types, same operation order, same Philox keys and counters.
 * Build with -ffp-contract=off so that no multiply-add is fused (the
 * reference's x86 builds have no FMA contraction).
 */
#define _GNU_SOURCE
#include "muca_oracle.h"
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Philox4x32-R.  Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11, section 3.2; Random123 philox.h:232-250 (round
 * multipliers and Weyl key increments), :284-302 (round and key bump),
 * :311-320 (R-round unroll: bump the key before every round but the first). */
#define PHX_M0 0xD2511F53u
#define PHX_M1 0xCD9E8D57u
#define PHX_W0 0x9E3779B9u
#define PHX_W1 0xBB67AE85u

void orc_philox4x32(unsigned rounds, const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t x0 = ctr[0], x1 = ctr[1], x2 = ctr[2], x3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (unsigned r = 0; r < rounds; ++r) {
        if (r) { k0 += PHX_W0; k1 += PHX_W1; }
        uint64_t p0 = (uint64_t)PHX_M0 * x0;
        uint64_t p1 = (uint64_t)PHX_M1 * x2;
        uint32_t y0 = (uint32_t)(p1 >> 32) ^ x1 ^ k0;
        uint32_t y1 = (uint32_t)p1;
        uint32_t y2 = (uint32_t)(p0 >> 32) ^ x3 ^ k1;
        uint32_t y3 = (uint32_t)p0;
        x0 = y0; x1 = y1; x2 = y2; x3 = y3;
    }
    out[0] = x0; out[1] = x1; out[2] = x2; out[3] = x3;
}

/* u01fixedpt<float>(uint32): (1 | (r >> 8)) * 2^-24 (uniform.hpp:195-205;
 * excess = 32 - 24 = 8 bits dropped).  Exact in float. */
float orc_u01fixedpt_f32(uint32_t r) { return (float)((r >> 8) | 1u) * 5.9604644775390625e-08f; }

/* u01fixedpt<double>(uint32): excess < 0, falls through to u01<double>:
 * r * 2^-32 + 2^-33 (uniform.hpp:144-153).  Exact in double. */
double orc_u01fixedpt_f64(uint32_t r) { return (double)r * 2.3283064365386962890625e-10 + 1.16415321826934814453125e-10; }

/* Initial spin: (u < 1/3.0) + (u < 2/3.0) - 1, float u compared in double
 * (muca_delta_multigpu.cu:350). */
int orc_init_spin(uint32_t r)
{
    double u = (double)orc_u01fixedpt_f32(r);
    return (u < 1 / 3.0) + (u < 2 / 3.0) - 1;
}

/* ------------------------------------------------------------------------ */
/* Neighbour table (right, left, up, down) and sweep order, restating
 * muca_delta_multigpu.cu:157-175 with unsigned arithmetic as written.      */
void orc_sweep_tables(unsigned L, uint32_t *naver, uint32_t *index)
{
    unsigned N = L * L;
    for (unsigned i = 0; i < N; i++) {
        int right = (int)i + 1;
        int left = (int)i - 1;
        int up = (int)(i + L);
        int down = (int)i - (int)L;
        if (right % (int)L == 0) right = right - (int)L;
        if (i % L == 0) left = left + (int)L;
        if (up > (int)N - 1) up = up - (int)N;
        if (down < 0) down = down + (int)N;
        naver[4 * i] = (uint32_t)right;
        naver[4 * i + 1] = (uint32_t)left;
        naver[4 * i + 2] = (uint32_t)up;
        naver[4 * i + 3] = (uint32_t)down;
        index[i] = ((unsigned)(0 == ((i / (N / 2)) % 2)) * (2 * i)) % N
                 + ((unsigned)(1 == ((i / (N / 2)) % 2)) * (2 * i + 1)) % N;
    }
}

/* ------------------------------------------------------------------------ */
orc_init_scheme orc_scheme_weight(unsigned jack, unsigned gpu)
{   /* key {10*WORK + mm*2, 0xdecafbad}, ctr {j*2, SEED, 0xBADCAB1E, 0xBADC0DED}, ++c[0] */
    orc_init_scheme s = {10u, 2u * jack, 0xdecafbadu, {2u * gpu, 100u, 0xBADCAB1Eu, 0xBADC0DEDu}, 0u, 7u};
    return s;
}
orc_init_scheme orc_scheme_produce(unsigned gpu)
{   /* key {WORK*10, 0xdecafbad}, ctr {gpu*1000, SEED, 0, 0xBADCAFE3}, ++c[2] */
    orc_init_scheme s = {10u, 0u, 0xdecafbadu, {1000u * gpu, 100u, 0u, 0xBADCAFE3u}, 2u, 7u};
    return s;
}
orc_init_scheme orc_scheme_produce_cpu(unsigned l)
{   /* key {WORKER*2000 + l*2, 0xdecafbad}, ctr {0, SEED, 0xBADCAB1E, 0xBADC0DED}, ++c[0] */
    orc_init_scheme s = {2000u, 2u * l, 0xdecafbadu, {0u, 100u, 0xBADCAB1Eu, 0xBADC0DEDu}, 0u, 7u};
    return s;
}
orc_init_scheme orc_scheme_muca_mag(unsigned jack)
{   /* key {10*WORKER + mm*10000, 0xdecafbad}, ctr {0, SEED, 0xBADCAB1E, 0xBADC0DED}, ++c[0] */
    orc_init_scheme s = {10u, 10000u * jack, 0xdecafbadu, {0u, 100u, 0xBADCAB1Eu, 0xBADC0DEDu}, 0u, 7u};
    return s;
}

void orc_init_lattice(unsigned L, unsigned chain0, unsigned nchains, const orc_init_scheme *s, int8_t *lat)
{
    unsigned N = L * L;
    for (unsigned c = 0; c < nchains; c++) {
        unsigned W = chain0 + c;
        uint32_t key[2] = {s->key0_mul * W + s->key0_add, s->key1};
        uint32_t ctr[4] = {s->ctr0[0], s->ctr0[1], s->ctr0[2], s->ctr0[3]};
        uint32_t r[4] = {0, 0, 0, 0};
        for (unsigned i = 0; i < N; i++) {
            if (i % 4 == 0) {
                ++ctr[s->ctr_word];
                orc_philox4x32(s->rounds, ctr, key, r);
            }
            lat[(size_t)c * N + i] = (int8_t)orc_init_spin(r[i % 4]);
        }
    }
}

/* Graded initial spins (an extension of this project, no reference
 * counterpart): the Philox words of orc_init_lattice, each spin nonzero iff
 * (r >> 8) * 2 cpd < (2W + 1) * 2^24, the sign from bit 0 of r (1: +1). */
void orc_init_lattice_graded(unsigned L, unsigned chain0, unsigned nchains, unsigned cpd, const orc_init_scheme *s,
                             int8_t *lat)
{
    unsigned N = L * L;
    for (unsigned c = 0; c < nchains; c++) {
        unsigned W = chain0 + c;
        uint32_t key[2] = {s->key0_mul * W + s->key0_add, s->key1};
        uint32_t ctr[4] = {s->ctr0[0], s->ctr0[1], s->ctr0[2], s->ctr0[3]};
        uint32_t r[4] = {0, 0, 0, 0};
        for (unsigned i = 0; i < N; i++) {
            if (i % 4 == 0) {
                ++ctr[s->ctr_word];
                orc_philox4x32(s->rounds, ctr, key, r);
            }
            uint32_t w = r[i % 4];
            int nz = (uint64_t)(w >> 8) * (2ull * cpd) < ((2ull * W + 1ull) << 24);
            lat[(size_t)c * N + i] = (int8_t)(nz ? ((w & 1u) ? 1 : -1) : 0);
        }
    }
}

/* total_energy (muca_delta_multigpu.cu:548-571): sum_i -s_i * sum(nb) >> 1 */
void orc_chain_energies(unsigned L, unsigned nchains, const int8_t *lat, int32_t *ej, int32_t *edel, int32_t *mag)
{
    unsigned N = L * L;
    uint32_t *nv = (uint32_t *)malloc(sizeof(uint32_t) * 4 * N);
    uint32_t *ix = (uint32_t *)malloc(sizeof(uint32_t) * N);
    orc_sweep_tables(L, nv, ix);
    for (unsigned c = 0; c < nchains; c++) {
        const int8_t *s = lat + (size_t)c * N;
        int sum = 0, d = 0, m = 0;
        for (unsigned i = 0; i < N; i++) {
            sum += -s[i] * (s[nv[4 * i]] + s[nv[4 * i + 1]] + s[nv[4 * i + 2]] + s[nv[4 * i + 3]]);
            d += s[i] * s[i];
            m += s[i];
        }
        if (ej) ej[c] = sum >> 1;
        if (edel) edel[c] = d;
        if (mag) mag[c] = m;
    }
    free(nv);
    free(ix);
}

/* ------------------------------------------------------------------------ */
/* One Metropolis attempt exactly as written in the reference kernels
 * (muca_delta_multigpu.cu:762-786, produce2_multigpu.cu:464-487): the site
 * takes the trial value new*(old==0)+old while dE is formed, then the final
 * value is stored.  Returns old/new/dE/dDel through pointers.               */
static inline void propose(int8_t *s, const uint32_t *nv, unsigned idx, uint32_t r3,
                           int *old_s, int *new_s, int *dE, int *dDel)
{
    int ns = s[idx] + 2 * (orc_u01fixedpt_f32(r3) < 0.5) - 1;
    int os = s[idx];
    ns = ns - 3 * (ns == 2) + 3 * (ns == -2);
    s[idx] = (int8_t)(ns * (os == 0) + os);
    *dE = ((os == 0) + os * (ns - os)) * (-s[idx]) *
          (s[nv[4 * idx]] + s[nv[4 * idx + 1]] + s[nv[4 * idx + 2]] + s[nv[4 * idx + 3]]);
    *dDel = ns * ns - os * os;
    *old_s = os;
    *new_s = ns;
}

/* Acceptance logarithm log(u01fixedpt<float>(r)).  The GPU kernels compute
 * it with CUDA's logf (muca_delta_multigpu.cu:781,816,
 * produce2_multigpu.cu:446,481), the CPU programs with libm's
 * (muca_mag.cpp:347,382).  Without a table this is libm's logf, which
 * differs from CUDA's by one ulp for some u; with the table of CUDA's values
 * (tab[k] for u = (2k+1) 2^-24, k = r >> 9, made by devlogf.cu) the decision
 * is the device's. */
static const float *g_logf_tab = NULL;

void orc_set_logf_table(const float *tab) { g_logf_tab = tab; }

void orc_libm_logf_table(float *tab)
{
    for (uint32_t k = 0; k < (1u << 23); ++k) tab[k] = logf(orc_u01fixedpt_f32(k << 9));
}

static inline float accept_logf(uint32_t r)
{
    return g_logf_tab ? g_logf_tab[r >> 9] : logf(orc_u01fixedpt_f32(r));
}

/* Metropolis term of the weight sweep.  The reference fixes beta = 2 and
 * forms -dE*2 as an int (muca_delta_multigpu.cu:810); orc_set_beta(b > 0)
 * uses the FP32 value (float)(-(b * dE)) instead, as the batched engine does
 * for any beta (for b = 2 the two are the same float). */
static int g_beta_on = 0;
static float g_btab[17];

void orc_set_beta(double beta)
{
    g_beta_on = beta > 0.0;
    for (int d = -8; d <= 8; ++d) g_btab[d + 8] = (float)(-(beta * (double)d));
}

static inline float beta_term(int dE) { return g_beta_on ? g_btab[dE + 8] : (float)(-dE * 2); }

/* Kernel mcs of muca_delta_multigpu.cu:737-829 for one chain. */
static void weight_chain(unsigned L, const uint32_t *nv, const uint32_t *ix, unsigned W, int8_t *s,
                         int32_t *ej, int32_t *edel, const float *w, uint64_t *hist,
                         uint32_t iter, uint32_t seed, uint64_t therm, uint64_t nup, unsigned rounds)
{
    unsigned N = L * L;
    uint32_t k1[2] = {2u * W, 0xdecafbadu};
    uint32_t k3[2] = {2u * W + 50000u, 0x11cafeadu};
    uint32_t c[4] = {0u, seed, iter, 0xBADC0DEDu};
    uint32_t r1[4] = {0, 0, 0, 0}, r3[4] = {0, 0, 0, 0};
    int energy = *ej, E = *edel;
    for (int phase = 0; phase < 2; phase++) {
        uint64_t n = phase ? nup : therm;
        for (uint64_t i = 0; i < n; i++) {
            if (i % 4 == 0) {
                ++c[0];
                orc_philox4x32(rounds, c, k1, r1);
                orc_philox4x32(rounds, c, k3, r3);
            }
            unsigned idx = ix[i % N];
            int os, ns, dE, dDel;
            propose(s, nv, idx, r3[i % 4], &os, &ns, &dE, &dDel);
            float diff = beta_term(dE) + w[E + dDel] - w[E];
            if (diff >= 0) {
                s[idx] = (int8_t)ns; energy += dE; E += dDel;
            } else if (accept_logf(r1[i % 4]) < diff) {
                s[idx] = (int8_t)ns; energy += dE; E += dDel;
            } else {
                s[idx] = (int8_t)os;
            }
            if (phase) hist[E] += 1;
        }
    }
    *ej = energy;
    *edel = E;
}

/* Kernel mcs of produce2_multigpu.cu:401-496 for one chain. */
static void produce_chain(unsigned L, const uint32_t *nv, const uint32_t *ix, unsigned W, int8_t *s,
                          int32_t *ej, int32_t *edel, int32_t *mag, const double *w, uint64_t *hist2d,
                          uint32_t iter, uint32_t seed, uint64_t therm, uint64_t nup, unsigned rounds)
{
    unsigned N = L * L;
    uint32_t k1[2] = {W, 0xdecafbadu};
    uint32_t k3[2] = {W + 40000u, 0xdecafeadu};
    uint32_t c[4] = {0u, seed, iter, 0xBADC0DEDu};
    uint32_t r1[4] = {0, 0, 0, 0}, r3[4] = {0, 0, 0, 0};
    int energy = *ej, E = *edel, M = *mag;
    for (int phase = 0; phase < 2; phase++) {
        uint64_t n = phase ? nup : therm;
        for (uint64_t i = 0; i < n; i++) {
            if (i % 4 == 0) {
                ++c[0];
                orc_philox4x32(rounds, c, k1, r1);
                orc_philox4x32(rounds, c, k3, r3);
            }
            unsigned idx = ix[i % N];
            int os, ns, dE, dDel;
            propose(s, nv, idx, r3[i % 4], &os, &ns, &dE, &dDel);
            int dM = ns - os;
            double diff = -dE * 2 + w[E + dDel] - w[E];
            if (diff >= 0) {
                s[idx] = (int8_t)ns; energy += dE; E += dDel; M += dM;
            } else if (accept_logf(r1[i % 4]) < diff) {
                s[idx] = (int8_t)ns; energy += dE; E += dDel; M += dM;
            } else {
                s[idx] = (int8_t)os;
            }
            if (phase) hist2d[(M + E * E + 2 * E) / 2] += 1;
        }
    }
    *ej = energy;
    *edel = E;
    *mag = M;
}

typedef struct sweep_job {
    int kind;  /* 0 weight, 1 produce */
    unsigned L, chain0, c_lo, c_hi, rounds;
    int8_t *lat;
    int32_t *ej, *edel, *mag;
    const float *wf;
    const double *wd;
    uint64_t *hist;      /* private histogram of this job */
    size_t hist_len;
    uint32_t iter, seed;
    uint64_t therm, nup;
    const uint32_t *nv, *ix;
} sweep_job;

static void *sweep_worker(void *arg)
{
    sweep_job *j = (sweep_job *)arg;
    unsigned N = j->L * j->L;
    for (unsigned c = j->c_lo; c < j->c_hi; c++) {
        if (j->kind == 0)
            weight_chain(j->L, j->nv, j->ix, j->chain0 + c, j->lat + (size_t)c * N, j->ej + c, j->edel + c,
                         j->wf, j->hist, j->iter, j->seed, j->therm, j->nup, j->rounds);
        else
            produce_chain(j->L, j->nv, j->ix, j->chain0 + c, j->lat + (size_t)c * N, j->ej + c, j->edel + c,
                          j->mag + c, j->wd, j->hist, j->iter, j->seed, j->therm, j->nup, j->rounds);
    }
    return NULL;
}

static void run_sweeps(sweep_job *base, unsigned nchains, uint64_t *hist_out, int nthreads)
{
    unsigned N = base->L * base->L;
    uint32_t *nv = (uint32_t *)malloc(sizeof(uint32_t) * 4 * N);
    uint32_t *ix = (uint32_t *)malloc(sizeof(uint32_t) * N);
    orc_sweep_tables(base->L, nv, ix);
    base->nv = nv;
    base->ix = ix;
    if (nthreads < 1) nthreads = 1;
    if ((unsigned)nthreads > nchains) nthreads = (int)(nchains ? nchains : 1);
    sweep_job *jobs = (sweep_job *)calloc((size_t)nthreads, sizeof(sweep_job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = *base;
        jobs[t].c_lo = (unsigned)((uint64_t)nchains * t / nthreads);
        jobs[t].c_hi = (unsigned)((uint64_t)nchains * (t + 1) / nthreads);
        jobs[t].hist = (t == 0) ? hist_out : (uint64_t *)calloc(base->hist_len, sizeof(uint64_t));
    }
    for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, sweep_worker, &jobs[t]);
    sweep_worker(&jobs[0]);
    for (int t = 1; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        for (size_t b = 0; b < base->hist_len; b++) hist_out[b] += jobs[t].hist[b];
        free(jobs[t].hist);
    }
    free(jobs);
    free(th);
    free(nv);
    free(ix);
}

void orc_weight_sweep(unsigned L, unsigned chain0, unsigned nchains, int8_t *lat, int32_t *ej, int32_t *edel,
                      const float *w, uint64_t *hist, uint32_t iter, uint32_t seed, uint64_t therm, uint64_t nup,
                      unsigned rounds, int nthreads)
{
    sweep_job b;
    memset(&b, 0, sizeof b);
    b.kind = 0; b.L = L; b.chain0 = chain0; b.rounds = rounds; b.lat = lat; b.ej = ej; b.edel = edel;
    b.wf = w; b.hist_len = (size_t)L * L + 1; b.iter = iter; b.seed = seed; b.therm = therm; b.nup = nup;
    run_sweeps(&b, nchains, hist, nthreads);
}

void orc_produce_sweep(unsigned L, unsigned chain0, unsigned nchains, int8_t *lat, int32_t *ej, int32_t *edel,
                       int32_t *mag, const double *w, uint64_t *hist2d, uint32_t iter, uint32_t seed,
                       uint64_t therm, uint64_t nup, unsigned rounds, int nthreads)
{
    sweep_job b;
    memset(&b, 0, sizeof b);
    size_t N = (size_t)L * L;
    b.kind = 1; b.L = L; b.chain0 = chain0; b.rounds = rounds; b.lat = lat; b.ej = ej; b.edel = edel;
    b.mag = mag; b.wd = w; b.hist_len = (N + 1) * (N + 2) / 2; b.iter = iter; b.seed = seed;
    b.therm = therm; b.nup = nup;
    run_sweeps(&b, nchains, hist2d, nthreads);
}

/* produce.cpp:421-511 */
void orc_produce_cpu_mcs(unsigned L, unsigned worker, int8_t *s, int32_t *ej, int32_t *edel, int32_t *mag,
                         const double *w, uint64_t *hist, uint32_t iter, uint32_t seed, uint64_t therm, uint64_t nup)
{
    unsigned N = L * L;
    uint32_t *nv = (uint32_t *)malloc(sizeof(uint32_t) * 4 * N);
    uint32_t *ix = (uint32_t *)malloc(sizeof(uint32_t) * N);
    orc_sweep_tables(L, nv, ix);
    uint32_t k1[2] = {10u * worker, 0xdecafbadu};
    uint32_t k3[2] = {10u * worker + 1000u, 0x11cafeadu};
    uint32_t c[4] = {0u, 10000u * seed, 2u * iter, 0xBADC0DEDu};
    uint32_t r1[4] = {0, 0, 0, 0}, r3[4] = {0, 0, 0, 0};
    for (size_t i = 0; i < (size_t)N + 1; i++) hist[i] = 0;
    int energy = *ej, E = *edel, M = *mag;
    for (int phase = 0; phase < 2; phase++) {
        uint64_t n = phase ? nup : therm;
        for (uint64_t i = 0; i < n; i++) {
            if (i % 4 == 0) {
                ++c[0];
                orc_philox4x32(7, c, k1, r1);
                orc_philox4x32(7, c, k3, r3);
            }
            if (phase) hist[(M + E * E + 2 * E) / 2] += 1;
            unsigned idx = ix[i % N];
            int os, ns, dE, dDel;
            propose(s, nv, idx, r3[i % 4], &os, &ns, &dE, &dDel);
            int dM = ns - os;
            double diff = -dE * 2 + w[E + dDel] - w[E];
            if (diff >= 0) {
                s[idx] = (int8_t)ns; energy += dE; E += dDel; M += dM;
            } else if (log(orc_u01fixedpt_f64(r1[i % 4])) < diff) {
                s[idx] = (int8_t)ns; energy += dE; E += dDel; M += dM;
            } else {
                s[idx] = (int8_t)os;
            }
        }
    }
    *ej = energy; *edel = E; *mag = M;
    free(nv);
    free(ix);
}

/* muca_mag.cpp:312-393 */
void orc_muca_mag_mcs(unsigned L, unsigned worker, int8_t *s, int32_t *ej, int32_t *edel, const double *w,
                      uint64_t *hist, uint32_t iter, uint32_t seed, uint64_t therm, uint64_t nup)
{
    unsigned N = L * L;
    uint32_t *nv = (uint32_t *)malloc(sizeof(uint32_t) * 4 * N);
    uint32_t *ix = (uint32_t *)malloc(sizeof(uint32_t) * N);
    orc_sweep_tables(L, nv, ix);
    uint32_t k1[2] = {10u * worker + 1000u * seed, 0xdecafbadu};
    uint32_t k2[2] = {100u * worker + 4000u * seed, 0x20202041u};
    uint32_t k3[2] = {1000u * worker + 10000u * seed, 0x11cafeadu};
    uint32_t c[4] = {0u, 0xbadbad11u, 2u * iter, 0xBADC0DEDu};
    uint32_t r1[4] = {0}, r2[4] = {0}, r3[4] = {0};
    for (unsigned i = 0; i < N + 1; i++) hist[i] = 0;
    int energy = *ej, E = *edel;
    for (int phase = 0; phase < 2; phase++) {
        uint64_t n = phase ? nup : therm;
        for (uint64_t i = 0; i < n; i++) {
            if (i % 4 == 0) {
                ++c[0];
                orc_philox4x32(7, c, k1, r1);
                orc_philox4x32(7, c, k2, r2);
                orc_philox4x32(7, c, k3, r3);
            }
            unsigned idx = (unsigned)(orc_u01fixedpt_f32(r2[i % 4]) * (float)N);
            int os, ns, dE, dDel;
            propose(s, nv, idx, r3[i % 4], &os, &ns, &dE, &dDel);
            double diff = -dE * 2 + w[E + dDel] - w[E];
            if (diff >= 0) {
                s[idx] = (int8_t)ns; energy += dE; E += dDel;
            } else if (accept_logf(r1[i % 4]) < diff) {
                s[idx] = (int8_t)ns; energy += dE; E += dDel;
            } else {
                s[idx] = (int8_t)os;
            }
            if (phase) hist[E] += 1;
        }
    }
    *ej = energy; *edel = E;
    free(nv);
    free(ix);
}

/* ------------------------------------------------------------------------ */
void orc_hist_range(const uint64_t *hist, unsigned N, int *start, int *end)
{
    int i;
    *start = (int)N + 1;
    *end = 0;
    for (i = 0; i < (int)N + 1; i++) {
        if (hist[i] > 1) { if (i < *start) *start = i; break; }
    }
    for (i = (int)N + 1; i-- > 0;) {
        if (hist[i] > 1) { if (i > *end) *end = i; break; }
    }
    if (*start > *end) { *start = 0; *end = 0; }
}

double orc_kull_leibler(const uint64_t *hist, unsigned N)
{
    double num_bin = 0, num_event = 0, kld = 0, P, Q;
    for (int i = 0; i < (int)N + 1; i++)
        if (hist[i] > 0) { num_event = num_event + (double)hist[i]; num_bin = num_bin + 1.0; }
    for (int i = 0; i < (int)N + 1; i++) {
        if (hist[i] > 0) {
            P = (double)hist[i] / num_event;
            Q = 1.0 / num_bin;
            kld = kld + P * log(P / Q);
        }
    }
    return kld;
}

void orc_update_trivial_gpu(const uint64_t *h, unsigned N, double *lnw)
{
    for (unsigned i = 0; i <= N; i++) if (h[i] > 1) lnw[i] = lnw[i] - log((double)h[i]);
    double tmp = lnw[0];
    for (unsigned i = 0; i <= N; i++) lnw[i] = lnw[i] - tmp;
}

void orc_update_trivial_cpu(const uint64_t *h, unsigned N, double *lnw)
{
    for (unsigned i = 0; i <= N; ++i) if (h[i] > 0) lnw[i] = lnw[i] - log((double)h[i]);
    double temp = lnw[0];
    for (unsigned i = 0; i <= N; ++i) if (h[i] > 0) lnw[i] = lnw[i] - temp;
}

void orc_weight_recursion(const uint64_t *hist, unsigned N, double *p_acc, int hist_start, int hist_end, double *lnw)
{
    double *bf = (double *)malloc(sizeof(double) * (N + 1));
    for (unsigned i = 0; i <= N; i++) bf[i] = lnw[i];
    for (int i = hist_start; i < hist_end; i++) {
        if ((hist[i] != 0) & (hist[i + 1] != 0)) {
            double p = (double)(hist[i] * hist[i + 1]) / (double)(hist[i] + hist[i + 1]);
            double k = p / (p + p_acc[i]);
            double delta_S = -bf[i] + bf[i + 1] + k * log((double)hist[i] / (double)hist[i + 1]);
            lnw[i + 1] = lnw[i] + delta_S;
            p_acc[i] = p_acc[i] + p;
        }
    }
    free(bf);
}

/* Flatness as min_i H[i] / mean_i H[i] over all N+1 bins (no reference
 * routine; E_Delta covers every bin of [0,N]).                            */
void orc_flatness(const uint64_t *h, unsigned N, double *min_over_mean, int *start, int *end)
{
    uint64_t mn = h[0];
    long double s = 0;
    for (unsigned i = 0; i <= N; i++) { if (h[i] < mn) mn = h[i]; s += h[i]; }
    double mean = (double)(s / (long double)(N + 1));
    *min_over_mean = mean > 0 ? (double)mn / mean : 0.0;
    orc_hist_range(h, N, start, end);
}

void orc_jackknife(const double *M_jacks, unsigned JACKS, double *avg_M, double *error_M)
{
    double avg = 0;
    for (unsigned i = 0; i < JACKS; i++) avg += M_jacks[i];
    double *M_i = (double *)malloc(sizeof(double) * (JACKS ? JACKS : 1));
    for (unsigned i = 0; i < JACKS; i++) M_i[i] = (avg - M_jacks[i]) / (double)(JACKS - 1);
    avg = avg / (double)JACKS;
    double dev = 0;
    for (unsigned i = 0; i < JACKS; i++) dev += (avg - M_i[i]) * (avg - M_i[i]);
    dev = (JACKS - 1) * dev / (double)(JACKS);
    dev = sqrt(dev);
    *avg_M = avg;
    *error_M = dev;
    free(M_i);
}

void orc_weight_shift(double beta, double delta, unsigned N, double *lnw)
{
    double mx = -INFINITY;
    for (unsigned i = 0; i < N + 1; i++) {
        double v = -lnw[i] - beta * delta * i;
        if (i == 0 || v > mx) mx = v;
    }
    for (unsigned i = 0; i < N + 1; i++) lnw[i] = lnw[i] + mx;
}

void orc_boltz(double beta, double delta, unsigned N, const double *lnw, double *boltz, int use_expl)
{
    for (unsigned j = 0; j < N + 1; j++) {
        double a = -beta * delta * j - lnw[j];
        boltz[j] = use_expl ? (double)expl(a) : exp(a);
    }
}

/* produce2_multigpu.cu:498-518 (long double sums), plus the fourth moment
 * for the Binder cumulant U4 = 1 - <M^4> / (3 <M^2>^2) (an extension).    */
void orc_observables(double beta, unsigned N, const uint64_t *h, const double *boltz, double out[7])
{
    long double sum = 0, M1 = 0, M2 = 0, M4 = 0;
    unsigned i;
    int m;
    for (i = 0; i <= N; i++) {
        for (m = -(int)i; m <= (int)i; m = m + 2) {
            uint64_t H = h[(i * i + 2 * i + (unsigned)m) / 2];
            uint64_t am = (uint64_t)(m < 0 ? -m : m);
            sum = sum + (double)H * boltz[i];
            M1 = M1 + (double)(am * H) * boltz[i];
            M2 = M2 + (double)((uint64_t)(m * m) * H) * boltz[i];
            M4 = M4 + (long double)((double)((uint64_t)(m * m) * H) * boltz[i]) * (long double)m * m;
        }
    }
    long double mabs = M1 / sum;
    long double chi = (M2 / sum - (M1 / sum) * (M1 / sum)) * beta / (long double)N;
    long double m2 = M2 / sum, m4 = M4 / sum;
    out[0] = (double)mabs;
    out[1] = (double)chi;
    out[2] = (double)(1.0L - m4 / (3.0L * m2 * m2));
    out[3] = (double)sum;
    out[4] = (double)M1;
    out[5] = (double)M2;
    out[6] = (double)M4;
}

/* ------------------------------------------------------------------------ */
unsigned orc_weight_run(const orc_weight_opts *o, int8_t *lat, int32_t *ej, int32_t *edel, double *lnw,
                        double *p_acc, double *rec, unsigned rec_cap, int *converged)
{
    unsigned N = o->L * o->L;
    float *w = (float *)malloc(sizeof(float) * (N + 1));
    uint64_t *h = (uint64_t *)malloc(sizeof(uint64_t) * (N + 1));
    unsigned width = o->width_start ? o->width_start : 10, NUPDATES = o->starting_M;
    int reach = 0;
    uint64_t total_run = 0;
    double prev_mm = 0.0;
    *converged = 0;
    for (unsigned i = 0; i <= N; i++) w[i] = (float)lnw[i];
    unsigned k;
    for (k = 0; k < o->max_iter; k++) {
        {
            /* the schedule at the top of the loop (muca_delta_multigpu.cu:379-382),
               with the doubling schedules and the cap as options; schedule 3
               doubles once the previous iteration's histogram also had every
               bin at >= 5 % of the mean */
            uint64_t nx = NUPDATES;
            unsigned cap = o->nup_max;
            if ((o->sched == 2 && k > 0) || (o->sched == 1 && width == N) ||
                (o->sched == 3 && width == N && k > 0 && prev_mm >= 0.05)) {
                nx = 2ull * NUPDATES;
                if (cap == 0) cap = 1u << 30;
            } else if ((o->sched == 0 || o->sched == 3) && width == N) {
                const unsigned nu = NUPDATES + 1;
                nx = (unsigned)(nu * 1.01);
            } else if (o->sched == 4 || (o->sched == 5 && width == N)) {
                nx = (uint64_t)((double)NUPDATES * 1.05);
                if (cap == 0) cap = 1u << 30;
            }
            if (cap != 0 && nx > cap) nx = cap > NUPDATES ? cap : NUPDATES;
            NUPDATES = (unsigned)nx;
        }
        total_run += (uint64_t)NUPDATES * o->nchains;
        memset(h, 0, sizeof(uint64_t) * (N + 1));
        if (o->algo == 1) {
            /* every rank's mcs, then the histogram Reduce (muca_mag.cpp:140-141) */
            uint64_t *hc = (uint64_t *)malloc(sizeof(uint64_t) * (N + 1));
            for (unsigned c = 0; c < o->nchains; ++c) {
                orc_muca_mag_mcs(o->L, c, lat + (size_t)c * N, ej + c, edel + c, lnw, hc, (uint32_t)k, o->jack, 0,
                                 NUPDATES);
                for (unsigned i = 0; i <= N; i++) h[i] += hc[i];
            }
            free(hc);
        } else {
            orc_weight_sweep(o->L, 0, o->nchains, lat, ej, edel, w, h, (uint32_t)k, 100u + 1000u * o->gpu, N,
                             NUPDATES, o->rounds, o->nthreads);
        }
        int hs, he;
        orc_hist_range(h, N, &hs, &he);
        unsigned width_temp = (unsigned)(he - hs);
        if (width_temp > width) width = width_temp;
        double dkl = orc_kull_leibler(h, N);
        double mm;
        int a, b;
        orc_flatness(h, N, &mm, &a, &b);
        prev_mm = mm;
        if (k < rec_cap) {
            rec[k * 5 + 0] = width_temp;
            rec[k * 5 + 1] = dkl;
            rec[k * 5 + 2] = NUPDATES;
            rec[k * 5 + 3] = (double)total_run;
            rec[k * 5 + 4] = mm;
        }
        if (width == N && !reach) reach = 1;
        if (o->flat_minmean ? (mm >= 0.5) : (width == N && dkl < 1e-4)) { *converged = 1; k++; break; }
        if (!o->hold_until_full || width == N) {
            if (o->recursive == 2) {
                orc_update_trivial_cpu(h, N, lnw);
            } else if (o->recursive) {
                orc_weight_recursion(h, N, p_acc, hs, he, lnw);
                double tmp = lnw[0];
                for (unsigned i = 0; i <= N; i++) lnw[i] = lnw[i] - tmp;
            } else {
                orc_update_trivial_gpu(h, N, lnw);
            }
            for (unsigned i = 0; i <= N; i++) w[i] = (float)lnw[i];
        }
    }
    free(w);
    free(h);
    return k;
}
