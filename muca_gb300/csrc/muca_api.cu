// muca_api.cu -- the C ABI of include/muca.h on top of the GB300 kernels.
//
// A context owns every device buffer of one simulation: the packed lattices
// of all chains, per-chain E_J / E_Delta / M, the FP64 master weights and
// the FP32 shadow the weight sweep reads, the u64 histogram(s), and the
// device-resident run state.  All work is enqueued on the context's stream.
#include "../../include/muca.h"
#include "muca_device.cuh"
#include "muca_internal.h"

#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace muca;

struct muca_ctx {
    muca_params prm{};
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sms = 0, max_thr_sm = 0;
    size_t smem_optin = 0;
    uint32_t L = 0, N = 0, WPR = 0, ndev = 1, cpd = 0, nchains = 0, rounds = 7, mode = 0, dev0 = 0;
    SweepPlan plan{};
    size_t lat_words = 0, hist_len = 0;
    uint32_t *d_lat = nullptr;
    int32_t *d_ej = nullptr, *d_edel = nullptr, *d_mag = nullptr;
    double *d_lnw = nullptr, *d_pacc = nullptr, *d_lnw_obs = nullptr;
    float *d_w32 = nullptr;
    unsigned long long *d_hist = nullptr;
    uint32_t *d_index = nullptr, *d_naver = nullptr;
    HistStatsDev *d_stats = nullptr, *h_stats = nullptr;
    UpdScratch *d_upd = nullptr;  // the multi-block weight update
    RunCtl *d_ctl = nullptr, *h_ctl = nullptr;
    IterRecordDev *d_recs = nullptr;
    size_t recs_cap = 0;
    double *d_obs_part = nullptr, *d_obs_out = nullptr, *h_obs_out = nullptr;
    double *d_jk = nullptr;
    size_t jk_cap = 0;
    int8_t *d_tmp = nullptr;
    unsigned long long *d_bad = nullptr, *h_bad = nullptr;
    unsigned int *d_err = nullptr, *h_err = nullptr;
    uint64_t device_bytes = 0;
    double log_eps = 0, log_eps_measured = 0;
    double log_eps_table = 1e30;  // host_logf: twice max |__logf(u) - the host table's log(u)|
    uint32_t algo = 0;
    float *d_logf_tab = nullptr;  // random-site algorithm with host_logf: the host libm's logf
    RecScratch rec{};             // the multi-block recursion's dS_i and pair flags (weight mode)
    long long wait_cycles = 0;    // bound of the sweep's device-side waits (0 = default)
    uint32_t hooks = 0;           // test hooks of the sweep (kHook*)
    std::string err;
};

namespace {

std::string g_create_err;

muca_status fail(muca_ctx *c, muca_status st, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf; else g_create_err = buf;
    return st;
}

#define CUDA_TRY(c, x)                                                                          \
    do {                                                                                        \
        cudaError_t _e = (x);                                                                   \
        if (_e != cudaSuccess) return fail((c), MUCA_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(_e)); \
    } while (0)

template <typename T>
cudaError_t dmalloc(muca_ctx *c, T **p, size_t n)
{
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e == cudaSuccess) c->device_bytes += n * sizeof(T);
    return e;
}

void free_all(muca_ctx *c)
{
    void *dp[] = {c->d_lat, c->d_ej, c->d_edel, c->d_mag, c->d_lnw, c->d_lnw_obs, c->d_pacc, c->d_w32, c->d_hist,
                  c->d_index, c->d_naver, c->d_stats, c->d_ctl, c->d_recs, c->d_obs_part, c->d_obs_out,
                  c->d_jk, c->d_tmp, c->d_bad, c->d_err, c->d_logf_tab, c->d_upd, c->rec.ds, c->rec.valid};
    for (void *p : dp)
        if (p) cudaFree(p);
    void *hp[] = {c->h_stats, c->h_ctl, c->h_obs_out, c->h_bad, c->h_err};
    for (void *p : hp)
        if (p) cudaFreeHost(p);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
}

// the host-side tables of muca_delta_multigpu.cu:157-175 (for the generic kernel)
void build_tables(uint32_t L, std::vector<uint32_t> &naver, std::vector<uint32_t> &index)
{
    const uint32_t N = L * L;
    naver.assign(4 * (size_t)N, 0);
    index.assign(N, 0);
    for (uint32_t i = 0; i < N; i++) {
        int right = (int)i + 1, left = (int)i - 1, up = (int)(i + L), down = (int)i - (int)L;
        if (right % (int)L == 0) right -= (int)L;
        if (i % L == 0) left += (int)L;
        if (up > (int)N - 1) up -= (int)N;
        if (down < 0) down += (int)N;
        naver[4 * i] = right; naver[4 * i + 1] = left; naver[4 * i + 2] = up; naver[4 * i + 3] = down;
        index[i] = ((uint32_t)(0 == ((i / (N / 2)) % 2)) * (2 * i)) % N
                 + ((uint32_t)(1 == ((i / (N / 2)) % 2)) * (2 * i + 1)) % N;
    }
}

muca_status ensure_tmp(muca_ctx *c)
{
    if (!c->d_tmp) CUDA_TRY(c, dmalloc(c, &c->d_tmp, (size_t)c->nchains * c->N));
    return MUCA_OK;
}

muca_status recompute_energies(muca_ctx *c)
{
    CUDA_TRY(c, launch_energies(c->d_lat, c->d_ej, c->d_edel, c->d_mag, c->L, c->WPR, c->plan.cpb, c->nchains,
                                c->stream));
    return MUCA_OK;
}

muca_status check_err(muca_ctx *c)
{
    CUDA_TRY(c, cudaMemcpyAsync(c->h_err, c->d_err, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (*c->h_err) {
        const unsigned int e = *c->h_err;
        cudaMemsetAsync(c->d_err, 0, sizeof(unsigned int), c->stream);
        return fail(c, MUCA_ERR_TIMEOUT, "a bounded device wait gave up (error word 0x%x); results are invalid", e);
    }
    return MUCA_OK;
}

SweepArgs sweep_args(muca_ctx *c, uint32_t iter, uint32_t seed_base, uint32_t seed_dev_mul, uint64_t therm,
                     uint64_t nup)
{
    SweepArgs a{};
    a.lat = c->d_lat;
    a.ej = c->d_ej;
    a.edel = c->d_edel;
    a.mag = c->d_mag;
    a.w = c->mode == MUCA_MODE_WEIGHT ? (const void *)c->d_w32 : (const void *)c->d_lnw;
    a.hist = c->d_hist;
    a.index = c->d_index;
    a.naver = c->d_naver;
    a.L = c->L;
    a.N = c->N;
    a.WPR = c->WPR;
    a.nchains = c->nchains;
    a.chains_per_dev = c->cpd;
    a.seed_base = seed_base + seed_dev_mul * c->dev0;  // device dev0 + d uses base + mul*(dev0+d)
    a.seed_dev_mul = seed_dev_mul;
    a.iter = iter;
    a.therm = therm;
    a.nup = nup;
    if (c->mode == MUCA_MODE_WEIGHT) {
        // muca_delta_multigpu.cu:740-741
        a.k1_mul = 2; a.k1_add = 0; a.k1_hi = 0xdecafbadu;
        a.k3_mul = 2; a.k3_add = 50000; a.k3_hi = 0x11cafeadu;
    } else {
        // produce2_multigpu.cu:406-408
        a.k1_mul = 1; a.k1_add = 0; a.k1_hi = 0xdecafbadu;
        a.k3_mul = 1; a.k3_add = 40000; a.k3_hi = 0xdecafeadu;
    }
    a.log_eps = c->log_eps;
    a.err = c->d_err;
    a.dyn = nullptr;
    a.wait_cycles = c->wait_cycles;
    a.hooks = c->hooks;
    return a;
}

// Arguments of the random-site sweep (muca_mag.cpp:312-318): WORKER = chain
// (offset by the first emulated device's chains), `seed` = the jack index.
RandomArgs random_args(muca_ctx *c, uint32_t iter, uint32_t seed, uint64_t therm, uint64_t nup)
{
    RandomArgs a{};
    a.lat = c->d_lat;
    a.ej = c->d_ej;
    a.edel = c->d_edel;
    a.w = c->d_lnw;
    a.hist = c->d_hist;
    a.L = c->L;
    a.N = c->N;
    a.WPR = c->WPR;
    a.nchains = c->nchains;
    a.worker0 = 0;  // WORKER = chain: the CPU program's ranks; dev_offset does not apply
    a.seed = seed;
    a.iter = iter;
    a.therm = therm;
    a.nup = nup;
    a.logf_tab = c->d_logf_tab;
    a.dyn = nullptr;
    a.inv_L = (uint32_t)(((1ull << 32) + c->L - 1) / c->L);
    // muca_set_log_bracket widens either bound
    a.log_eps = c->d_logf_tab ? (c->log_eps_table > c->log_eps ? c->log_eps_table : c->log_eps) : c->log_eps;
    return a;
}

}  // namespace

extern "C" {

const char *muca_last_error(const muca_ctx *c) { return c ? c->err.c_str() : g_create_err.c_str(); }

muca_status muca_default_chains(int32_t device, uint32_t *out)
{
    if (!out) return fail(nullptr, MUCA_ERR_BAD_ARG, "out is NULL");
    int thr = 0, sms = 0;
    CUDA_TRY(nullptr, cudaDeviceGetAttribute(&thr, cudaDevAttrMaxThreadsPerMultiProcessor, device));
    CUDA_TRY(nullptr, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    *out = (uint32_t)(thr * sms);
    return MUCA_OK;
}

muca_status muca_create(const muca_params *p, muca_ctx **out)
{
    if (!p || !out) return fail(nullptr, MUCA_ERR_BAD_ARG, "params/out is NULL");
    *out = nullptr;
    if (p->L < 2 || p->L > 128) return fail(nullptr, MUCA_ERR_BAD_ARG, "L=%u outside 2..128", p->L);
    if (p->mode > MUCA_MODE_PRODUCE) return fail(nullptr, MUCA_ERR_BAD_ARG, "mode=%u", p->mode);
    const uint32_t rounds = p->rounds ? p->rounds : 7;
    if (rounds != 7 && rounds != 10) return fail(nullptr, MUCA_ERR_BAD_ARG, "rounds=%u (7 or 10)", rounds);
    muca_ctx *c = new muca_ctx();
    c->prm = *p;
    c->device = p->device;
    c->L = p->L;
    c->N = p->L * p->L;
    c->WPR = (p->L + 15) / 16;
    c->ndev = p->ndev ? p->ndev : 1;
    c->dev0 = p->dev_offset;
    c->rounds = rounds;
    c->mode = p->mode;
    auto bail = [&](muca_status st) {
        g_create_err = c->err;
        free_all(c);
        delete c;
        return st;
    };
#define CREATE_TRY(x)                                                                               \
    do {                                                                                            \
        cudaError_t _e = (x);                                                                       \
        if (_e != cudaSuccess) { fail(c, MUCA_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(_e)); return bail(MUCA_ERR_CUDA); } \
    } while (0)
    CREATE_TRY(cudaSetDevice(c->device));
    int optin = 0;
    CREATE_TRY(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device));
    CREATE_TRY(cudaDeviceGetAttribute(&c->max_thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, c->device));
    CREATE_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    c->smem_optin = (size_t)optin;
    c->cpd = p->nchains ? p->nchains : (uint32_t)(c->max_thr_sm * c->sms);
    const uint64_t total = (uint64_t)c->cpd * c->ndev;
    if (total == 0 || total > (1ull << 26)) {
        fail(c, MUCA_ERR_BAD_ARG, "chains=%llu outside 1..2^26", (unsigned long long)total);
        return bail(MUCA_ERR_BAD_ARG);
    }
    c->nchains = (uint32_t)total;
    if (p->kernel > 3) {
        fail(c, MUCA_ERR_BAD_ARG, "kernel=%u (0..3)", p->kernel);
        return bail(MUCA_ERR_BAD_ARG);
    }
    if (p->kernel >= 2 && !(p->L % 8 == 0 && p->L >= 8)) {
        fail(c, MUCA_ERR_BAD_ARG, "kernel %u needs L %% 8 == 0", p->kernel);
        return bail(MUCA_ERR_BAD_ARG);
    }
    if (p->algorithm > MUCA_ALGO_RANDOM_SITE) {
        fail(c, MUCA_ERR_BAD_ARG, "algorithm=%u (0..1)", p->algorithm);
        return bail(MUCA_ERR_BAD_ARG);
    }
    if (p->algorithm == MUCA_ALGO_RANDOM_SITE && (p->mode != MUCA_MODE_WEIGHT || p->L < 3 || c->ndev != 1)) {
        fail(c, MUCA_ERR_BAD_ARG, "the random-site algorithm needs weight mode, L >= 3 and one device");
        return bail(MUCA_ERR_BAD_ARG);
    }
    c->algo = p->algorithm;
    const int want_kernel = p->kernel == 0 ? -1 : (int)p->kernel - 1;
    c->plan = c->algo == MUCA_ALGO_RANDOM_SITE
                  ? plan_random(c->L, c->nchains, c->smem_optin, c->sms)
                  : plan_sweep((int)c->mode, (int)rounds, c->L, c->nchains, c->smem_optin, c->sms, want_kernel);
    c->plan.rounds = (int)rounds;
    if (c->plan.smem > c->smem_optin) {
        fail(c, MUCA_ERR_BAD_ARG, "L=%u needs %zu B of shared memory per block (device has %zu)", c->L, c->plan.smem,
             c->smem_optin);
        return bail(MUCA_ERR_BAD_ARG);
    }
    if (p->stream) {
        c->stream = (cudaStream_t)p->stream;
    } else {
        CREATE_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    const uint32_t N = c->N;
    c->lat_words = (size_t)c->plan.blocks * c->plan.cpb * c->L * c->WPR;
    c->hist_len = c->mode == MUCA_MODE_WEIGHT ? (size_t)N + 1 : (size_t)(N + 1) * (N + 2) / 2;
    CREATE_TRY(dmalloc(c, &c->d_lat, c->lat_words));
    CREATE_TRY(dmalloc(c, &c->d_ej, c->nchains));
    CREATE_TRY(dmalloc(c, &c->d_edel, c->nchains));
    CREATE_TRY(dmalloc(c, &c->d_mag, c->nchains));
    CREATE_TRY(dmalloc(c, &c->d_lnw, (size_t)N + 1));
    CREATE_TRY(dmalloc(c, &c->d_pacc, (size_t)N + 1));
    CREATE_TRY(dmalloc(c, &c->d_lnw_obs, (size_t)N + 1));
    CREATE_TRY(cudaMemsetAsync(c->d_lnw_obs, 0, ((size_t)N + 1) * 8, c->stream));
    CREATE_TRY(dmalloc(c, &c->d_w32, (size_t)N + 1));
    CREATE_TRY(dmalloc(c, &c->d_hist, c->hist_len));
    CREATE_TRY(dmalloc(c, &c->d_stats, 1));
    CREATE_TRY(dmalloc(c, &c->d_upd, 1));
    CREATE_TRY(cudaMemsetAsync(c->d_upd, 0, sizeof(UpdScratch), c->stream));
    if (c->mode == MUCA_MODE_WEIGHT) {
        CREATE_TRY(dmalloc(c, &c->rec.ds, (size_t)N));
        CREATE_TRY(dmalloc(c, &c->rec.valid, (size_t)N));
    }
    CREATE_TRY(dmalloc(c, &c->d_ctl, 1));
    CREATE_TRY(dmalloc(c, &c->d_bad, 1));
    CREATE_TRY(dmalloc(c, &c->d_err, 1));
    CREATE_TRY(cudaMallocHost((void **)&c->h_err, sizeof(unsigned int)));
    CREATE_TRY(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned int), c->stream));
    CREATE_TRY(cudaMallocHost((void **)&c->h_stats, sizeof(HistStatsDev)));
    CREATE_TRY(cudaMallocHost((void **)&c->h_ctl, sizeof(RunCtl)));
    CREATE_TRY(cudaMallocHost((void **)&c->h_bad, sizeof(unsigned long long)));
    CREATE_TRY(cudaMallocHost((void **)&c->h_obs_out, 4 * sizeof(double)));
    CREATE_TRY(cudaMemsetAsync(c->d_lat, 0x55, c->lat_words * 4, c->stream));  // all spins 0
    CREATE_TRY(cudaMemsetAsync(c->d_ej, 0, c->nchains * 4, c->stream));
    CREATE_TRY(cudaMemsetAsync(c->d_edel, 0, c->nchains * 4, c->stream));
    CREATE_TRY(cudaMemsetAsync(c->d_mag, 0, c->nchains * 4, c->stream));
    CREATE_TRY(cudaMemsetAsync(c->d_lnw, 0, ((size_t)N + 1) * 8, c->stream));
    CREATE_TRY(cudaMemsetAsync(c->d_pacc, 0, ((size_t)N + 1) * 8, c->stream));
    CREATE_TRY(cudaMemsetAsync(c->d_w32, 0, ((size_t)N + 1) * 4, c->stream));
    CREATE_TRY(cudaMemsetAsync(c->d_hist, 0, c->hist_len * 8, c->stream));
    if (c->plan.kernel == kKernelGeneric) {  // its sweep order and neighbours come from tables
        std::vector<uint32_t> nv, ix;
        build_tables(c->L, nv, ix);
        CREATE_TRY(dmalloc(c, &c->d_index, ix.size()));
        CREATE_TRY(dmalloc(c, &c->d_naver, nv.size()));
        CREATE_TRY(cudaMemcpyAsync(c->d_index, ix.data(), ix.size() * 4, cudaMemcpyHostToDevice, c->stream));
        CREATE_TRY(cudaMemcpyAsync(c->d_naver, nv.data(), nv.size() * 4, cudaMemcpyHostToDevice, c->stream));
    }
    {
        // the bound of the fast acceptance test, measured once per device
        // (cached under a lock: contexts may be created on several threads)
        if (c->device < 0 || c->device >= 64) { fail(c, MUCA_ERR_BAD_ARG, "device %d", c->device); return bail(MUCA_ERR_BAD_ARG); }
        CREATE_TRY(device_log_eps(c->device, c->stream, &c->log_eps));
        c->log_eps_measured = c->log_eps;
    }
    if (c->algo == MUCA_ALGO_RANDOM_SITE) {
        if (random_sweep_smem(c->L, c->plan.cpb, false) > c->smem_optin) {
            fail(c, MUCA_ERR_BAD_ARG, "L=%u: FP64 weights and histogram exceed shared memory", c->L);
            return bail(MUCA_ERR_BAD_ARG);
        }
        if (p->host_logf) {
            // the CPU program's acceptance log, logf(u) of this host's libm for every
            // u = (2k+1) 2^-24 that u01fixedpt<float> can return
            std::vector<float> tab((size_t)1 << 23);
            for (uint32_t k = 0; k < (1u << 23); ++k) tab[k] = logf((float)(2u * k + 1u) * 5.9604644775390625e-8f);
            CREATE_TRY(dmalloc(c, &c->d_logf_tab, tab.size()));
            CREATE_TRY(cudaMemcpyAsync(c->d_logf_tab, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, c->stream));
            CREATE_TRY(cudaStreamSynchronize(c->stream));  // `tab` is pageable
            // the fast test's bound against this table, measured over every entry
            float m = 0.0f;
            CREATE_TRY(measure_table_bracket(c->d_logf_tab, &m, c->stream));
            c->log_eps_table = (m >= 0.0f && m < 1e-2f) ? 2.0 * (double)m + 1e-30 : 1e30;
        }
    }
    CREATE_TRY(cudaStreamSynchronize(c->stream));
#undef CREATE_TRY
    *out = c;
    return MUCA_OK;
}

muca_status muca_destroy(muca_ctx *c)
{
    if (!c) return MUCA_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_all(c);
    delete c;
    return MUCA_OK;
}

muca_status muca_get_info(const muca_ctx *c, muca_info *o)
{
    if (!c || !o) return fail(nullptr, MUCA_ERR_BAD_ARG, "NULL argument");
    o->L = c->L;
    o->N = c->N;
    o->nchains_total = c->nchains;
    o->chains_per_block = c->plan.cpb;
    o->blocks = c->plan.blocks;
    o->lattice_in_smem = c->plan.lat_smem;
    o->hist_in_smem = c->mode == MUCA_MODE_WEIGHT;
    o->weights_in_smem = 1;
    o->smem_bytes = (uint32_t)c->plan.smem;
    o->sms = (uint32_t)c->sms;
    o->device_bytes = c->device_bytes;
    o->log_bracket = c->log_eps;
    o->kernel = (uint32_t)c->plan.kernel + 1;
    o->threads_per_block = c->plan.threads;
    return MUCA_OK;
}

muca_status muca_set_log_bracket(muca_ctx *c, double bracket)
{
    if (!c) return fail(nullptr, MUCA_ERR_BAD_ARG, "ctx is NULL");
    if (!(bracket >= c->log_eps_measured && bracket <= 1e30))
        return fail(c, MUCA_ERR_BAD_ARG, "log bracket %g outside [%g, 1e30] (the measured bound and up)", bracket,
                    c->log_eps_measured);
    c->log_eps = bracket;
    return MUCA_OK;
}

muca_status muca_set_wait_limit(muca_ctx *c, uint64_t cycles)
{
    if (!c) return fail(nullptr, MUCA_ERR_BAD_ARG, "ctx is NULL");
    if (cycles > (1ull << 40)) return fail(c, MUCA_ERR_BAD_ARG, "wait limit %llu cycles above 2^40",
                                           (unsigned long long)cycles);
    c->wait_cycles = (long long)cycles;
    return MUCA_OK;
}

muca_status muca_set_test_hooks(muca_ctx *c, uint32_t hooks)
{
    if (!c) return fail(nullptr, MUCA_ERR_BAD_ARG, "ctx is NULL");
    if (hooks & ~(uint32_t)(MUCA_HOOK_SILENT_PRODUCER | MUCA_HOOK_FLUSH_ROWS))
        return fail(c, MUCA_ERR_BAD_ARG, "unknown hook bits 0x%x", hooks);
    static_assert(MUCA_HOOK_SILENT_PRODUCER == kHookSilentProducer && MUCA_HOOK_FLUSH_ROWS == kHookFlushRows,
                  "hook bits");
    c->hooks = hooks;
    return MUCA_OK;
}

muca_status muca_init_chains(muca_ctx *c, uint32_t scheme, uint32_t jack)
{
    if (!c) return fail(nullptr, MUCA_ERR_BAD_ARG, "ctx is NULL");
    InitArgs ia{};
    ia.rounds = 7;
    switch (scheme) {
    case MUCA_INIT_WEIGHT:  // muca_delta_multigpu.cu:342-347
    case MUCA_INIT_GRADED:
        ia.key0_mul = 10; ia.key0_jack_mul = 2; ia.key1 = 0xdecafbadu;
        ia.ctr0[1] = 100; ia.ctr0[2] = 0xBADCAB1Eu; ia.ctr0[3] = 0xBADC0DEDu;
        ia.ctr0_dev_mul[0] = 2; ia.ctr_word = 0;
        ia.graded = scheme == MUCA_INIT_GRADED;
        break;
    case MUCA_INIT_PRODUCE:  // produce2_multigpu.cu:129-134
        ia.key0_mul = 10; ia.key1 = 0xdecafbadu;
        ia.ctr0[1] = 100; ia.ctr0[3] = 0xBADCAFE3u;
        ia.ctr0_dev_mul[0] = 1000; ia.ctr_word = 2;
        break;
    case MUCA_INIT_CHAIN_COUNTER:
        ia.key0_add = 2024; ia.key1_jack_mul = 1; ia.rounds = 10; ia.chain_in_ctr = 1;
        break;
    case MUCA_INIT_ORDERED:
        ia.ordered = 1;
        break;
    case MUCA_INIT_MUCA_MAG:  // muca_mag.cpp:64-65
        ia.key0_mul = 10; ia.key0_jack_mul = 10000; ia.key1 = 0xdecafbadu;
        ia.ctr0[1] = 100; ia.ctr0[2] = 0xBADCAB1Eu; ia.ctr0[3] = 0xBADC0DEDu;
        ia.ctr_word = 0;
        break;
    default:
        return fail(c, MUCA_ERR_BAD_ARG, "init scheme %u", scheme);
    }
    CUDA_TRY(c, cudaSetDevice(c->device));
    // emulated device index = dev0 + chain / cpd enters the init counter
    for (int j = 0; j < 4; ++j) ia.ctr0[j] += ia.ctr0_dev_mul[j] * c->dev0;
    ia.chain_offset = c->dev0 * c->cpd;
    CUDA_TRY(c, launch_init(c->d_lat, c->L, c->WPR, c->plan.cpb, c->nchains, c->cpd, jack, ia, c->stream));
    return recompute_energies(c);
}

muca_status muca_set_lattice(muca_ctx *c, const int8_t *lat, size_t n)
{
    if (!c || !lat) return fail(c, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n != (size_t)c->nchains * c->N) return fail(c, MUCA_ERR_BAD_ARG, "n=%zu, expected %zu", n, (size_t)c->nchains * c->N);
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (muca_status st = ensure_tmp(c)) return st;
    CUDA_TRY(c, cudaMemcpyAsync(c->d_tmp, lat, n, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(c->d_bad, 0, 8, c->stream));
    CUDA_TRY(c, launch_validate(c->d_tmp, n, c->d_bad, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(c->h_bad, c->d_bad, 8, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (*c->h_bad) return fail(c, MUCA_ERR_BAD_ARG, "%llu lattice values outside {-1,0,1}", *c->h_bad);
    CUDA_TRY(c, launch_pack(c->d_lat, c->d_tmp, c->L, c->WPR, c->plan.cpb, c->nchains, c->stream));
    return recompute_energies(c);
}

muca_status muca_get_lattice(muca_ctx *c, int8_t *lat, size_t n)
{
    if (!c || !lat) return fail(c, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n != (size_t)c->nchains * c->N) return fail(c, MUCA_ERR_BAD_ARG, "n=%zu, expected %zu", n, (size_t)c->nchains * c->N);
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (muca_status st = ensure_tmp(c)) return st;
    CUDA_TRY(c, launch_unpack(c->d_lat, c->d_tmp, c->L, c->WPR, c->plan.cpb, c->nchains, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(lat, c->d_tmp, n, cudaMemcpyDeviceToHost, c->stream));
    return check_err(c);
}

muca_status muca_get_chain_state(muca_ctx *c, int32_t *ej, int32_t *edel, int32_t *mag, size_t n)
{
    if (!c) return fail(nullptr, MUCA_ERR_BAD_ARG, "ctx is NULL");
    if (n != c->nchains) return fail(c, MUCA_ERR_BAD_ARG, "n=%zu, expected %u", n, c->nchains);
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (ej) CUDA_TRY(c, cudaMemcpyAsync(ej, c->d_ej, n * 4, cudaMemcpyDeviceToHost, c->stream));
    if (edel) CUDA_TRY(c, cudaMemcpyAsync(edel, c->d_edel, n * 4, cudaMemcpyDeviceToHost, c->stream));
    if (mag) CUDA_TRY(c, cudaMemcpyAsync(mag, c->d_mag, n * 4, cudaMemcpyDeviceToHost, c->stream));
    return check_err(c);
}

muca_status muca_set_weights(muca_ctx *c, const double *lnw, size_t n)
{
    if (!c || !lnw) return fail(c, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n != (size_t)c->N + 1) return fail(c, MUCA_ERR_BAD_ARG, "n=%zu, expected N+1=%u", n, c->N + 1);
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(lnw[i])) return fail(c, MUCA_ERR_BAD_ARG, "weight %zu is not finite", i);
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaMemcpyAsync(c->d_lnw, lnw, n * 8, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(c->d_lnw_obs, c->d_lnw, n * 8, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(c, launch_weights_to_f32(c->d_lnw, c->d_w32, (uint32_t)n, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MUCA_OK;
}

muca_status muca_get_weights(muca_ctx *c, double *lnw, size_t n)
{
    if (!c || !lnw) return fail(c, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n != (size_t)c->N + 1) return fail(c, MUCA_ERR_BAD_ARG, "n=%zu, expected N+1=%u", n, c->N + 1);
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaMemcpyAsync(lnw, c->d_lnw, n * 8, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MUCA_OK;
}

static muca_status do_sweep(muca_ctx *c, uint32_t iter, uint32_t seed_base, uint32_t seed_dev_mul, uint64_t therm,
                            uint64_t nup, bool clear)
{
    if (!c) return fail(nullptr, MUCA_ERR_BAD_ARG, "ctx is NULL");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (clear) CUDA_TRY(c, cudaMemsetAsync(c->d_hist, 0, c->hist_len * 8, c->stream));
    if (c->algo == MUCA_ALGO_RANDOM_SITE) {
        const RandomArgs a = random_args(c, iter, seed_base, therm, nup);
        CUDA_TRY(c, launch_sweep_random(a, c->plan.cpb, c->plan.blocks, (int)c->rounds, c->smem_optin, c->stream));
        return MUCA_OK;
    }
    const SweepArgs a = sweep_args(c, iter, seed_base, seed_dev_mul, therm, nup);
    CUDA_TRY(c, launch_sweep(c->plan, a, c->stream));
    return MUCA_OK;
}

muca_status muca_sweep(muca_ctx *c, uint32_t iter, uint32_t seed_base, uint32_t seed_dev_mul, uint64_t therm,
                       uint64_t nup)
{
    return do_sweep(c, iter, seed_base, seed_dev_mul, therm, nup, true);
}

muca_status muca_sweep_accumulate(muca_ctx *c, uint32_t iter, uint32_t seed_base, uint32_t seed_dev_mul,
                                  uint64_t therm, uint64_t nup)
{
    return do_sweep(c, iter, seed_base, seed_dev_mul, therm, nup, false);
}

muca_status muca_clear_histogram(muca_ctx *c)
{
    if (!c) return fail(nullptr, MUCA_ERR_BAD_ARG, "ctx is NULL");
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaMemsetAsync(c->d_hist, 0, c->hist_len * 8, c->stream));
    return MUCA_OK;
}

muca_status muca_get_histogram(muca_ctx *c, uint64_t *h, size_t n)
{
    if (!c || !h) return fail(c, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n != c->hist_len) return fail(c, MUCA_ERR_BAD_ARG, "n=%zu, expected %zu", n, c->hist_len);
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaMemcpyAsync(h, c->d_hist, n * 8, cudaMemcpyDeviceToHost, c->stream));
    return check_err(c);
}

muca_status muca_set_histogram(muca_ctx *c, const uint64_t *h, size_t n)
{
    if (!c || !h) return fail(c, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n != c->hist_len) return fail(c, MUCA_ERR_BAD_ARG, "n=%zu, expected %zu", n, c->hist_len);
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaMemcpyAsync(c->d_hist, h, n * 8, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MUCA_OK;
}

static void stats_out(const HistStatsDev &s, muca_hist_stats *o)
{
    o->start = s.start;
    o->end = s.end;
    o->width = s.width;
    o->visited = s.visited;
    o->events = s.events;
    o->min_count = s.min_count;
    o->d_kl = s.d_kl;
    o->min_over_mean = s.min_over_mean;
}

static muca_status update_impl(muca_ctx *c, int rule, muca_hist_stats *st)
{
    if (!c) return fail(nullptr, MUCA_ERR_BAD_ARG, "ctx is NULL");
    if (c->mode != MUCA_MODE_WEIGHT) return fail(c, MUCA_ERR_STATE, "weight statistics need a weight-mode context");
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, launch_weight_update(c->d_hist, c->N, c->d_lnw, c->d_w32, c->d_pacc, rule, c->d_stats, c->stream, c->d_upd,
                                     &c->rec));
    if (!st) return MUCA_OK;  // enqueue only
    CUDA_TRY(c, cudaMemcpyAsync(c->h_stats, c->d_stats, sizeof(HistStatsDev), cudaMemcpyDeviceToHost, c->stream));
    if (muca_status e = check_err(c)) return e;
    stats_out(*c->h_stats, st);
    return MUCA_OK;
}

muca_status muca_histogram_stats(muca_ctx *c, muca_hist_stats *st)
{
    if (!st) return fail(c, MUCA_ERR_BAD_ARG, "stats is NULL");
    return update_impl(c, -1, st);
}

muca_status muca_update_weights(muca_ctx *c, uint32_t rule, muca_hist_stats *st)
{
    if (rule > MUCA_UPDATE_RECURSION) return fail(c, MUCA_ERR_BAD_ARG, "rule %u", rule);
    return update_impl(c, (int)rule, st);
}

muca_status muca_iterate_host(muca_ctx *c, const double *lnw_in, uint32_t iter, uint32_t seed_base,
                              uint32_t seed_dev_mul, uint64_t therm, uint64_t nup, uint32_t rule, double *lnw_out,
                              uint64_t *hist_out, muca_hist_stats *st)
{
    if (!c) return fail(nullptr, MUCA_ERR_BAD_ARG, "ctx is NULL");
    if (c->mode != MUCA_MODE_WEIGHT) return fail(c, MUCA_ERR_STATE, "iterate_host needs a weight-mode context");
    if (rule > MUCA_UPDATE_RECURSION) return fail(c, MUCA_ERR_BAD_ARG, "rule %u", rule);
    const size_t n = (size_t)c->N + 1;
    if (lnw_in)
        for (size_t i = 0; i < n; ++i)
            if (!std::isfinite(lnw_in[i])) return fail(c, MUCA_ERR_BAD_ARG, "weight %zu is not finite", i);
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (lnw_in) {
        // read by the stream before this call returns (it synchronises below)
        CUDA_TRY(c, cudaMemcpyAsync(c->d_lnw, lnw_in, n * 8, cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(c->d_lnw_obs, c->d_lnw, n * 8, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(c, launch_weights_to_f32(c->d_lnw, c->d_w32, (uint32_t)n, c->stream));
    }
    if (muca_status e = do_sweep(c, iter, seed_base, seed_dev_mul, therm, nup, true)) return e;
    CUDA_TRY(c, launch_weight_update(c->d_hist, c->N, c->d_lnw, c->d_w32, c->d_pacc, (int)rule, c->d_stats, c->stream,
                                     c->d_upd, &c->rec));
    if (st) CUDA_TRY(c, cudaMemcpyAsync(c->h_stats, c->d_stats, sizeof(HistStatsDev), cudaMemcpyDeviceToHost, c->stream));
    if (lnw_out) CUDA_TRY(c, cudaMemcpyAsync(lnw_out, c->d_lnw, n * 8, cudaMemcpyDeviceToHost, c->stream));
    if (hist_out) CUDA_TRY(c, cudaMemcpyAsync(hist_out, c->d_hist, n * 8, cudaMemcpyDeviceToHost, c->stream));
    if (muca_status e = check_err(c)) return e;  // the one synchronisation
    if (st) stats_out(*c->h_stats, st);
    return MUCA_OK;
}

static muca_status run_impl(muca_ctx *c, const muca_run_opts *o, muca_run_result *res, muca_iter_record *recs,
                            size_t cap, muca_iter_callback cb, void *user)
{
    if (!c || !o) return fail(c, MUCA_ERR_BAD_ARG, "NULL argument");
    if (c->mode != MUCA_MODE_WEIGHT) return fail(c, MUCA_ERR_STATE, "weight run needs a weight-mode context");
    if (o->rule > MUCA_UPDATE_RECURSION) return fail(c, MUCA_ERR_BAD_ARG, "rule %u", o->rule);
    if (o->starting_M == 0) return fail(c, MUCA_ERR_BAD_ARG, "starting_M must be >= 1");
    if (o->nup_schedule > 5) return fail(c, MUCA_ERR_BAD_ARG, "nup_schedule %u (0..5)", o->nup_schedule);
    CUDA_TRY(c, cudaSetDevice(c->device));
    const auto t0 = std::chrono::steady_clock::now();
    if (o->reinit_chains) {
        if (muca_status st = muca_init_chains(c, o->init_scheme, o->jack)) return st;
    }
    const uint32_t max_iter = o->max_iter ? o->max_iter : 1000000u;
    const size_t need = cb ? 1 : cap;  // streaming keeps the latest record only
    if (need > 0 && need > c->recs_cap) {
        if (c->d_recs) cudaFree(c->d_recs);
        c->d_recs = nullptr;
        CUDA_TRY(c, dmalloc(c, &c->d_recs, need));
        c->recs_cap = need;
    }
    RunCtl &h = *c->h_ctl;
    std::memset(&h, 0, sizeof h);
    h.st.k = 0;
    h.st.nup = o->starting_M;
    h.st.width = o->width_start ? o->width_start : 10;  // muca_delta_multigpu.cu:314
    // the schedule runs at the top of every iteration (:379-382), so a run that
    // starts at full width (a later jack) grows NUPDATES before its first sweep;
    // the device applies it between iterations from then on
    if (o->nup_schedule == 4) {
        // the CPU program multiplies at the top of every iteration, the first included (muca_mag.cpp:131)
        const unsigned long long nx = (unsigned long long)((double)h.st.nup * 1.05);
        const uint32_t cap = o->nup_max ? o->nup_max : (1u << 30);
        h.st.nup = nx > cap ? (cap > h.st.nup ? cap : h.st.nup) : (uint32_t)nx;
    } else if (h.st.width == c->N && o->nup_schedule != 2) {
        // (schedule 3 knows no histogram yet: it grows like the reference's)
        unsigned long long nx = o->nup_schedule == 1   ? 2ull * h.st.nup
                                : o->nup_schedule == 5 ? (unsigned long long)((double)h.st.nup * 1.05)
                                                       : (unsigned)((h.st.nup + 1u) * 1.01);
        const uint32_t cap = o->nup_max ? o->nup_max : (o->nup_schedule == 1 || o->nup_schedule == 5 ? (1u << 30) : 0u);
        if (cap != 0 && nx > cap) nx = cap > h.st.nup ? cap : h.st.nup;
        h.st.nup = (uint32_t)nx;
    }
    h.st.total_run = (unsigned long long)h.st.nup * c->nchains;
    h.N = c->N;
    h.nchains_total = c->nchains;
    h.rule = o->rule;
    h.hold = o->hold_until_full;
    h.flat_minmean = o->flat_minmean;
    h.max_iter = max_iter;
    h.sched = o->nup_schedule;
    h.nup_max = o->nup_max;
    h.mom_thr = o->min_over_mean > 0 ? o->min_over_mean : 0.5;
    h.dkl_max = o->d_kl_max > 0 ? o->d_kl_max : 1e-4;
    h.recs = need ? c->d_recs : nullptr;
    h.rec_cap = (uint32_t)need;
    h.rec_ring = cb ? 1u : 0u;
    CUDA_TRY(c, cudaMemcpyAsync(c->d_ctl, &h, sizeof h, cudaMemcpyHostToDevice, c->stream));
    // therm_coeff * N (:315-316); the CPU program's random-site runs thermalise 0 (muca_mag.cpp:140)
    const uint64_t therm = o->therm ? o->therm : (c->algo == MUCA_ALGO_RANDOM_SITE ? 0 : c->N);
    SweepArgs a = sweep_args(c, 0, 100u, 1000u, therm, 0);  // seed SEED+1000*l (:393)
    a.dyn = &c->d_ctl->st.k;
    RandomArgs ra = random_args(c, 0, o->jack, therm, 0);  // mcs(..., WORKER, k, mm, 0, NUPDATES)
    ra.dyn = &c->d_ctl->st.k;
    cudaEvent_t e0, e1, m0, m1;
    CUDA_TRY(c, cudaEventCreate(&e0));
    CUDA_TRY(c, cudaEventCreate(&e1));
    CUDA_TRY(c, cudaEventCreate(&m0));
    CUDA_TRY(c, cudaEventCreate(&m1));
    std::vector<double> kms, mms;
    double tk = 0, tm = 0, nwidth_time = -1;
    uint32_t k_done = 0;
    muca_status rs = MUCA_OK;
    const bool graph_mode = o->graph_iters > 0 && !cb;
    if (graph_mode) {
        // K iterations (clear, sweep, update) captured once and replayed; the
        // device stops them itself, so one host round trip serves K iterations
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed);
        const bool capturing = e == cudaSuccess;
        for (uint32_t j = 0; j < o->graph_iters && e == cudaSuccess; ++j) {
            e = launch_run_clear(c->d_hist, (uint32_t)c->hist_len, c->d_ctl, c->stream);
            if (e == cudaSuccess)
                e = c->algo == MUCA_ALGO_RANDOM_SITE
                        ? launch_sweep_random(ra, c->plan.cpb, c->plan.blocks, (int)c->rounds, c->smem_optin, c->stream)
                        : launch_sweep(c->plan, a, c->stream);
            if (e == cudaSuccess) e = launch_run_update(c->d_hist, c->d_lnw, c->d_w32, c->d_pacc, c->d_ctl, c->stream,
                                                        c->N, (int)o->rule, c->d_upd, &c->rec);
        }
        if (capturing) {
            const cudaError_t ec = cudaStreamEndCapture(c->stream, &graph);
            if (e == cudaSuccess) e = ec;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        while (e == cudaSuccess) {
            e = cudaEventRecord(e0, c->stream);
            if (e == cudaSuccess) e = cudaGraphLaunch(exec, c->stream);
            if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(&h.st, &c->d_ctl->st, sizeof(IterState), cudaMemcpyDeviceToHost,
                                                      c->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
            if (e != cudaSuccess) break;
            float ks = 0;
            cudaEventElapsedTime(&ks, e0, e1);
            tk += ks;
            if (h.st.reach && nwidth_time < 0) nwidth_time = tk;
            if (h.st.stop) break;
        }
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) rs = fail(c, MUCA_ERR_CUDA, "weight run (graph): %s", cudaGetErrorString(e));
        k_done = h.st.converged ? h.st.k + 1u : h.st.k;
    }
    while (!graph_mode) {
        // one iteration per host round trip, like the reference loop; the
        // device decides the schedule and convergence
        cudaError_t e = launch_run_clear(c->d_hist, (uint32_t)c->hist_len, c->d_ctl, c->stream);
        if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
        if (e == cudaSuccess)
            e = c->algo == MUCA_ALGO_RANDOM_SITE
                    ? launch_sweep_random(ra, c->plan.cpb, c->plan.blocks, (int)c->rounds, c->smem_optin, c->stream)
                    : launch_sweep(c->plan, a, c->stream);
        if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
        if (e == cudaSuccess) e = launch_run_update(c->d_hist, c->d_lnw, c->d_w32, c->d_pacc, c->d_ctl, c->stream,
                                                        c->N, (int)o->rule, c->d_upd, &c->rec);
        if (e == cudaSuccess) e = cudaEventRecord(m0, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h.st, &c->d_ctl->st, sizeof(IterState), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaEventRecord(m1, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) { rs = fail(c, MUCA_ERR_CUDA, "weight run: %s", cudaGetErrorString(e)); break; }
        float ks = 0, ms = 0;
        cudaEventElapsedTime(&ks, e0, e1);
        cudaEventElapsedTime(&ms, m0, m1);
        kms.push_back(ks);
        mms.push_back(ms);
        tk += ks;
        tm += ms;
        if (cb) {
            // this iteration's record lies in the device record array (capacity >= 1 in stream mode)
            IterRecordDev r;
            if (cudaMemcpy(&r, c->d_recs, sizeof r, cudaMemcpyDeviceToHost) == cudaSuccess) {
                muca_iter_record ur{};
                ur.k = r.k; ur.width_temp = r.width_temp; ur.width = r.width; ur.nupdates = r.nupdates;
                ur.total_run = r.total_run; ur.d_kl = r.d_kl; ur.min_over_mean = r.min_over_mean;
                ur.kernel_ms = ks; ur.memcpy_ms = ms;
                cb(&ur, user);
            }
        }
        ++k_done;
        if (h.st.reach && nwidth_time < 0) nwidth_time = tk;
        if (h.st.stop) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(m0);
    cudaEventDestroy(m1);
    if (rs != MUCA_OK) return rs;
    if (muca_status e = check_err(c)) return e;
    if (recs && cap) {
        std::vector<IterRecordDev> r(std::min<size_t>(cap, k_done));
        CUDA_TRY(c, cudaMemcpy(r.data(), c->d_recs, r.size() * sizeof(IterRecordDev), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < r.size(); ++i) {
            recs[i].k = r[i].k;
            recs[i].width_temp = r[i].width_temp;
            recs[i].width = r[i].width;
            recs[i].nupdates = r[i].nupdates;
            recs[i].total_run = r[i].total_run;
            recs[i].d_kl = r[i].d_kl;
            recs[i].min_over_mean = r[i].min_over_mean;
            recs[i].kernel_ms = i < kms.size() ? kms[i] : 0.0;  // none per iteration in graph mode
            recs[i].memcpy_ms = i < mms.size() ? mms[i] : 0.0;
        }
    }
    if (res) {
        res->iterations = k_done;
        res->converged = h.st.converged;
        res->width_reached_iter = h.st.reach ? h.st.reach_k : 0xFFFFFFFFu;
        res->total_run = h.st.converged ? h.st.total_run : h.st.total_run;
        res->nwidth_step = h.st.nwidth_step;
        res->total_kernel_s = tk * 1e-3;
        res->total_mem_s = tm * 1e-3;
        res->nwidth_time_s = nwidth_time < 0 ? 0 : nwidth_time * 1e-3;
        res->wall_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return h.st.converged ? MUCA_OK : fail(c, MUCA_ERR_NOT_CONVERGED, "not converged after %u iterations", k_done);
}

muca_status muca_weight_run(muca_ctx *c, const muca_run_opts *o, muca_run_result *res, muca_iter_record *recs,
                            size_t cap)
{
    return run_impl(c, o, res, recs, cap, nullptr, nullptr);
}

muca_status muca_weight_run_stream(muca_ctx *c, const muca_run_opts *o, muca_run_result *res, muca_iter_callback cb,
                                   void *user)
{
    if (!cb) return fail(c, MUCA_ERR_BAD_ARG, "callback is NULL");
    return run_impl(c, o, res, nullptr, 0, cb, user);
}

muca_status muca_weight_shift(muca_ctx *c, double beta, double delta)
{
    if (!c) return fail(nullptr, MUCA_ERR_BAD_ARG, "ctx is NULL");
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, launch_weight_shift(c->d_lnw_obs, c->N, beta, delta, c->stream));
    return MUCA_OK;
}

muca_status muca_get_reweighting_weights(muca_ctx *c, double *lnw, size_t n)
{
    if (!c || !lnw) return fail(c, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n != (size_t)c->N + 1) return fail(c, MUCA_ERR_BAD_ARG, "n=%zu, expected N+1=%u", n, c->N + 1);
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaMemcpyAsync(lnw, c->d_lnw_obs, n * 8, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MUCA_OK;
}

muca_status muca_compute_observables(muca_ctx *c, double beta, double delta, muca_observables *out)
{
    if (!c || !out) return fail(c, MUCA_ERR_BAD_ARG, "NULL argument");
    if (c->mode != MUCA_MODE_PRODUCE) return fail(c, MUCA_ERR_STATE, "observables need a production-mode context");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (!c->d_obs_part) {
        CUDA_TRY(c, dmalloc(c, &c->d_obs_part, observables_partials(c->N)));
        CUDA_TRY(c, dmalloc(c, &c->d_obs_out, 4));
    }
    CUDA_TRY(c, launch_observables(c->d_hist, c->d_lnw_obs, c->N, beta, delta, c->d_obs_part, c->d_obs_out, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(c->h_obs_out, c->d_obs_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    const double s = c->h_obs_out[0], m1 = c->h_obs_out[1], m2 = c->h_obs_out[2], m4 = c->h_obs_out[3];
    out->sum = s;
    out->m1 = m1;
    out->m2 = m2;
    out->m4 = m4;
    out->m_abs = m1 / s;
    out->chi = (m2 / s - (m1 / s) * (m1 / s)) * beta / (double)c->N;
    out->u4 = 1.0 - (m4 / s) / (3.0 * (m2 / s) * (m2 / s));
    return MUCA_OK;
}

muca_status muca_jackknife(muca_ctx *c, const double *x, uint32_t n, double *avg, double *err)
{
    if (!c || !x || !avg || !err) return fail(c, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n == 0) return fail(c, MUCA_ERR_BAD_ARG, "n == 0");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (n + 2 > c->jk_cap) {
        if (c->d_jk) cudaFree(c->d_jk);
        c->d_jk = nullptr;
        CUDA_TRY(c, dmalloc(c, &c->d_jk, (size_t)n + 2));
        c->jk_cap = n + 2;
    }
    CUDA_TRY(c, cudaMemcpyAsync(c->d_jk, x, n * 8, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, launch_jackknife(c->d_jk, n, c->d_jk + n, c->stream));
    double r[2];
    CUDA_TRY(c, cudaMemcpyAsync(r, c->d_jk + n, 16, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    *avg = r[0];
    *err = r[1];
    return MUCA_OK;
}

muca_status muca_observables_noalloc(int32_t device, const uint64_t *d_hist2d, const double *d_lnw, uint32_t L,
                                    double beta, double delta, double *d_sums, void *stream)
{
    if (!d_hist2d || !d_lnw || !d_sums) return fail(nullptr, MUCA_ERR_BAD_ARG, "NULL device pointer");
    if (L < 2 || L > 128) return fail(nullptr, MUCA_ERR_BAD_ARG, "L=%u outside 2..128", L);
    const uint32_t N = L * L;
    if (observables_partials(N) > observables_static_partials())
        return fail(nullptr, MUCA_ERR_BAD_ARG, "L=%u needs %zu doubles of scratch; the static array holds %zu", L,
                    observables_partials(N), observables_static_partials());
    // the caller's current device is put back on every return path: a
    // scheduler driving several GPUs from one thread keeps its own choice
    int prev = -1;
    CUDA_TRY(nullptr, cudaGetDevice(&prev));
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess)
        e = launch_observables_static(device, reinterpret_cast<const unsigned long long *>(d_hist2d), d_lnw, N, beta,
                                      delta, d_sums, static_cast<cudaStream_t>(stream));
    const cudaError_t er = prev != device ? cudaSetDevice(prev) : cudaSuccess;
    if (e != cudaSuccess) return fail(nullptr, MUCA_ERR_CUDA, "observables_noalloc: %s", cudaGetErrorString(e));
    if (er != cudaSuccess)
        return fail(nullptr, MUCA_ERR_CUDA, "observables_noalloc: restoring device %d: %s", prev,
                    cudaGetErrorString(er));
    return MUCA_OK;
}

muca_status muca_philox_peak(int32_t device, uint32_t rounds, double *blocks_per_s)
{
    if (!blocks_per_s) return fail(nullptr, MUCA_ERR_BAD_ARG, "NULL argument");
    if (rounds != 7 && rounds != 10) return fail(nullptr, MUCA_ERR_BAD_ARG, "rounds=%u", rounds);
    CUDA_TRY(nullptr, cudaSetDevice(device));
    int sms = 0, thr = 0;
    CUDA_TRY(nullptr, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    CUDA_TRY(nullptr, cudaDeviceGetAttribute(&thr, cudaDevAttrMaxThreadsPerMultiProcessor, device));
    const uint32_t grid = (uint32_t)(sms * (thr / 256)), per = 4096;
    uint32_t *out = nullptr;
    CUDA_TRY(nullptr, cudaMalloc(&out, (size_t)grid * 256 * 4));
    cudaStream_t s;
    cudaEvent_t e0, e1;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    cudaError_t err = cudaSuccess;
    for (int rep = 0; rep < 5 && err == cudaSuccess; ++rep) {
        cudaEventRecord(e0, s);
        err = launch_philox_peak((int)rounds, grid, per, out, s);
        cudaEventRecord(e1, s);
        if (err == cudaSuccess) err = cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;  // first launch is warm-up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    cudaFree(out);
    if (err != cudaSuccess) return fail(nullptr, MUCA_ERR_CUDA, "philox peak: %s", cudaGetErrorString(err));
    *blocks_per_s = (double)grid * 256.0 * per / (best * 1e-3);
    return MUCA_OK;
}

muca_status muca_sweep_floor(int32_t device, uint32_t part, uint32_t windows, double *cycles_per_attempt)
{
    if (!cycles_per_attempt) return fail(nullptr, MUCA_ERR_BAD_ARG, "NULL argument");
    if (part > 6 || windows < 2 || windows > (1u << 20) || (windows & 1u))
        return fail(nullptr, MUCA_ERR_BAD_ARG, "part=%u windows=%u", part, windows);
    int prev = 0;
    CUDA_TRY(nullptr, cudaGetDevice(&prev));
    CUDA_TRY(nullptr, cudaSetDevice(device));
    unsigned long long *cyc = nullptr, *hd = nullptr;
    uint32_t *sink = nullptr;
    cudaError_t err = cudaMalloc(&cyc, 4 * sizeof(unsigned long long));
    if (err == cudaSuccess) err = cudaMalloc(&hd, sizeof(unsigned long long));
    if (err == cudaSuccess) err = cudaMalloc(&sink, 128 * sizeof(uint32_t));
    unsigned long long h[4] = {0, 0, 0, 0};
    // one launch to warm up, then the measured one
    for (int rep = 0; rep < 2 && err == cudaSuccess; ++rep) {
        err = launch_sweep_floor((int)part, windows, cyc, sink, hd, 0);
        if (err == cudaSuccess) err = cudaDeviceSynchronize();
    }
    if (err == cudaSuccess) err = cudaMemcpy(h, cyc, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(cyc);
    cudaFree(hd);
    cudaFree(sink);
    cudaSetDevice(prev);
    if (err != cudaSuccess) return fail(nullptr, MUCA_ERR_CUDA, "sweep floor: %s", cudaGetErrorString(err));
    unsigned long long mx = 0;
    for (int w = 0; w < 4; ++w) mx = h[w] > mx ? h[w] : mx;
    *cycles_per_attempt = (double)mx / (8.0 * windows);
    return MUCA_OK;
}

}  // extern "C"
