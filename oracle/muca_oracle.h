/*
 * muca_oracle.h -- CPU oracle for the MUCA multicanonical hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (null2p/MUCA) used as the checker for the CUDA implementation in
 * muca_gb300/.  Only tests/, __graft_entry__.smoke() and the cpu_baseline leg
 * of bench.py may load it.  The product never links or calls it.
 *
 * Parity pins (see tests/): Philox4x32-7/-10 known-answer vectors from
 * Random123/examples/kat_vectors:24-29, u01fixedpt vectors from
 * Random123/examples/ut_uniform_kat_vectors.dat, the reference CPU programs
 * (produce.cpp, muca_mag.cpp) and the reference host functions of
 * muca_delta_multigpu.cu / produce2_multigpu.cu compiled from their own
 * sources into oracle/_ref, and the reference GPU kernels compiled from their
 * own sources into cubins that the GPU tests launch beside ours.
 *
 * Layout convention: lattices are [chain][site] int8, site = row*L + col.
 * "WORKER" below is the reference's global thread index == chain id.
 */
#ifndef MUCA_ORACLE_H
#define MUCA_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- RNG (Random123 philox.h:284-320 round/bumpkey; uniform.hpp:195-205) ---- */
void     orc_philox4x32(unsigned rounds, const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float    orc_u01fixedpt_f32(uint32_t r);
double   orc_u01fixedpt_f64(uint32_t r);
int      orc_init_spin(uint32_t r);

/* ---- lattice tables (muca_delta_multigpu.cu:157-175) ---- */
void orc_sweep_tables(unsigned L, uint32_t *naver /*4N*/, uint32_t *index /*N*/);

/* ---- initial lattices ----
 * key = {key0_mul*WORKER + key0_add, key1}; ctr = ctr0[0..3]; before every
 * 4th site the counter word ctr_word is incremented; site i takes r.v[i%4]. */
typedef struct orc_init_scheme {
    uint32_t key0_mul, key0_add, key1;
    uint32_t ctr0[4];
    uint32_t ctr_word;
    uint32_t rounds;
} orc_init_scheme;
/* scheme of muca_delta_multigpu.cu:340-351 (weight run, jack mm, device j) */
orc_init_scheme orc_scheme_weight(unsigned jack, unsigned gpu);
/* scheme of produce2_multigpu.cu:126-138 (production, device gpu) */
orc_init_scheme orc_scheme_produce(unsigned gpu);
/* scheme of produce.cpp:167-177 (CPU production, delta point l) */
orc_init_scheme orc_scheme_produce_cpu(unsigned l);
/* scheme of muca_mag.cpp:63-73 (CPU weight, jack mm) */
orc_init_scheme orc_scheme_muca_mag(unsigned jack);
void orc_init_lattice(unsigned L, unsigned chain0, unsigned nchains, const orc_init_scheme *s, int8_t *lat);
void orc_init_lattice_graded(unsigned L, unsigned chain0, unsigned nchains, unsigned cpd, const orc_init_scheme *s,
                             int8_t *lat);

/* E_J (computeEnergies, :69-74 + :548-571), E_Delta (:76-83), M (produce2:84-89) */
void orc_chain_energies(unsigned L, unsigned nchains, const int8_t *lat, int32_t *ej, int32_t *edel, int32_t *mag);

/* Acceptance logarithm of orc_weight_sweep / orc_produce_sweep: NULL = libm
 * logf; else tab[k] = CUDA's logf((2k+1) 2^-24) for k < 2^23 (devlogf.cu),
 * the value the reference kernels compute on the device.  The table is read,
 * not copied: it must stay alive while set. */
void orc_set_logf_table(const float *tab);
/* the same table with libm's logf (2^23 floats), to check the lookup */
void orc_libm_logf_table(float *tab);

/* beta of orc_weight_sweep: 0 = the reference's literal -dE*2; b > 0 =
 * the FP32 term (float)(-(b*dE)) of the batched engine. */
void orc_set_beta(double beta);

/* ---- sweeps ----
 * orc_weight_sweep: muca_delta_multigpu.cu:737-829 (kernel mcs), FP32 weights,
 * histogram of E_Delta after every production attempt (added to hist, u64).
 * orc_produce_sweep: produce2_multigpu.cu:401-496, FP64 weights, 2D histogram
 * at (M + E^2 + 2E)/2 after every production attempt (added to hist2d).
 * Chains [chain0, chain0+nchains) use WORKER = chain0 + c.  nthreads>1 splits
 * chains over POSIX threads (results are independent of nthreads).        */
void orc_weight_sweep(unsigned L, unsigned chain0, unsigned nchains, int8_t *lat,
                      int32_t *ej, int32_t *edel, const float *w, uint64_t *hist,
                      uint32_t iter, uint32_t seed, uint64_t therm, uint64_t nup,
                      unsigned rounds, int nthreads);
void orc_produce_sweep(unsigned L, unsigned chain0, unsigned nchains, int8_t *lat,
                       int32_t *ej, int32_t *edel, int32_t *mag, const double *w,
                       uint64_t *hist2d, uint32_t iter, uint32_t seed, uint64_t therm,
                       uint64_t nup, unsigned rounds, int nthreads);
/* produce.cpp:421-511 (CPU production mcs, one rank == one chain): keys
 * {10W, 10W+1000}, ctr {0,10000*seed,2*iter,..}, u01fixedpt<double>, histogram
 * recorded BEFORE each production attempt, and only hist[0..N] zeroed first. */
void orc_produce_cpu_mcs(unsigned L, unsigned worker, int8_t *lat, int32_t *ej, int32_t *edel,
                         int32_t *mag, const double *w, uint64_t *hist2d, uint32_t iter,
                         uint32_t seed, uint64_t therm, uint64_t nup);
/* muca_mag.cpp:312-393 (CPU weight mcs): random site, 3 Philox streams,
 * FP64 diff; zeroes hist[0..N] then records E_Delta after every attempt. */
void orc_muca_mag_mcs(unsigned L, unsigned worker, int8_t *lat, int32_t *ej, int32_t *edel,
                      const double *w, uint64_t *hist, uint32_t iter, uint32_t seed,
                      uint64_t therm, uint64_t nup);

/* ---- host math (FP64) ---- */
void   orc_hist_range(const uint64_t *h, unsigned N, int *start, int *end);          /* :573-596 */
double orc_kull_leibler(const uint64_t *h, unsigned N);                              /* :598-618 */
void   orc_update_trivial_gpu(const uint64_t *h, unsigned N, double *lnw);           /* :466-476 */
void   orc_update_trivial_cpu(const uint64_t *h, unsigned N, double *lnw);           /* muca_mag.cpp:178-183 */
void   orc_weight_recursion(const uint64_t *h, unsigned N, double *p_acc, int start, int end,
                            double *lnw);                                             /* :833-859 */
void   orc_flatness(const uint64_t *h, unsigned N, double *min_over_mean, int *start, int *end);
void   orc_jackknife(const double *x, unsigned J, double *avg, double *err);         /* :620-635 */
void   orc_weight_shift(double beta, double delta, unsigned N, double *lnw);         /* produce2:391-400 */
void   orc_boltz(double beta, double delta, unsigned N, const double *lnw, double *boltz, int use_expl);
/* produce2_multigpu.cu:498-518 in long double; out = {<|M|>, chi, U4, sum, M1, M2, M4} */
void   orc_observables(double beta, unsigned N, const uint64_t *hist2d, const double *boltz, double out[7]);

/* ---- one reference weight-estimation run (muca_delta_multigpu.cu:329-477) ----
 * Runs iterations until converged or max_iter.  lnw (N+1) holds the initial
 * FP64 weight on entry and the final one on exit.  Per-iteration records are
 * written to rec[k*5 + {width_temp, D_KL, NUPDATES, total_run, min/mean}] for
 * k < rec_cap.  Returns the number of iterations run; *converged set. */
typedef struct orc_weight_opts {
    unsigned L, nchains, jack, gpu, starting_M;
    int recursive;        /* 0 trivial (GPU flavour), 1 weight_recursion, 2 trivial (CPU flavour,
                             muca_mag.cpp:179-182) */
    int hold_until_full;  /* 0: reference GPU behaviour (always update) */
    int flat_minmean;     /* 0: width==N && D_KL<1e-4 ; 1: min/mean >= 0.5 */
    unsigned max_iter;
    unsigned rounds;
    int nthreads;
    unsigned width_start; /* initial running width; 0 = 10 (the reference keeps the previous jack's) */
    unsigned sched;       /* NUPDATES schedule: 0 reference ((NUP+1)*1.01 once width==N), 1 doubling
                             once width==N, 2 doubling every iteration from the first, 3 as 0 and
                             doubling once the last histogram had every bin >= 5 % of the mean */
    unsigned nup_max;     /* cap of NUPDATES: 0 = none for schedule 0, 2^30 otherwise; never decreases.
                             Schedule 4: NUP*1.05 every iteration, the first included (muca_mag.cpp:131) */
    unsigned algo;        /* 0: the GPU weight kernel (sweep order, FP32 weights, therm N);
                             1: the CPU program's random-site mcs (muca_mag.cpp:312-393) per chain,
                             WORKER = chain, seed = jack, therm 0, FP64 weights */
} orc_weight_opts;
unsigned orc_weight_run(const orc_weight_opts *o, int8_t *lat, int32_t *ej, int32_t *edel,
                        double *lnw, double *p_acc, double *rec, unsigned rec_cap, int *converged);

#ifdef __cplusplus
}
#endif
#endif
