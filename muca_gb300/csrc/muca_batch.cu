// muca_batch.cu -- C ABI of a batch of independent weight-estimation runs.
//
// The reference runs one (L, T) weight estimation per program invocation.
// A batch runs many of them, of uneven size, through one persistent sweep
// kernel per iteration (k_batch.cu), with the iteration loop captured into a
// CUDA graph and replayed until every instance has stopped.  Instance i is
// the reference's weight loop for its L and beta with the seeds of emulated
// device `seed`: with beta = 2 its lattices, histograms and weights are those
// of a single-simulation context created with dev_offset = seed.
//
// Memory: every per-instance array lives in one arena per kind (lattice,
// chain state, weights, histograms, run state), so a batch of 256 instances
// is a handful of allocations; the BatchInst table the kernels read holds
// the per-instance pointers into the arenas.
//
// The block shape (chains per block, lattice and histogram placement, blocks
// per SM) is chosen by an autotuner at creation: every shape that fits is
// timed on this batch (one warm-up sweep and two timed sweeps of therm = N
// and nup = N attempts per chain) and the fastest is kept.
#include "../../include/muca.h"
#include "muca_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace muca;

struct muca_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sms = 0;
    size_t smem_optin = 0;
    int rounds = 7;
    std::vector<muca_instance> inst;
    uint32_t n = 0, max_N = 0, max_L = 0;
    // per-instance offsets into the arenas
    std::vector<size_t> off_w;      // N+1 arrays (weights, histograms)
    std::vector<size_t> off_chain;  // per-chain arrays
    std::vector<size_t> off_lat;    // lattice words (depends on chains per block)
    size_t total_w = 0, total_chains = 0, lat_words = 0, lat_cap = 0;
    uint32_t *d_lat = nullptr;
    int32_t *d_ej = nullptr, *d_edel = nullptr, *d_mag = nullptr;
    double *d_lnw = nullptr, *d_pacc = nullptr;
    float *d_w32 = nullptr;
    unsigned long long *d_hist = nullptr;
    RunCtl *d_ctl = nullptr;
    IterRecordDev *d_recs = nullptr;
    BatchInst *d_inst = nullptr;
    BatchItem *d_items = nullptr;
    size_t items_cap = 0;
    uint32_t n_items = 0;
    uint32_t *d_counters = nullptr;  // [0] next item, [1] running instances
    uint32_t *h_running = nullptr;
    unsigned int *d_err = nullptr;
    double log_eps = 1e30;
    // shape
    muca_batch_shape shape{};
    uint32_t grid = 0, threads = 0;
    size_t smem = 0;
    std::vector<muca_batch_shape> tried;
    // captured iteration loop
    cudaGraphExec_t graph = nullptr;
    uint32_t graph_iters = 0;
    int graph_rec = -1;
    uint64_t device_bytes = 0;
    std::string err;
};

namespace {

std::string g_batch_err;

muca_status bfail(muca_batch *b, muca_status st, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (b) b->err = buf; else g_batch_err = buf;
    return st;
}

#define BCUDA(b, x)                                                                              \
    do {                                                                                         \
        cudaError_t _e = (x);                                                                    \
        if (_e != cudaSuccess) return bfail((b), MUCA_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(_e)); \
    } while (0)

template <typename T>
cudaError_t bmalloc(muca_batch *b, T **p, size_t n)
{
    const cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e == cudaSuccess) b->device_bytes += n * sizeof(T);
    return e;
}

void free_all(muca_batch *b)
{
    if (b->graph) cudaGraphExecDestroy(b->graph);
    cudaFree(b->d_lat);
    cudaFree(b->d_ej);
    cudaFree(b->d_edel);
    cudaFree(b->d_mag);
    cudaFree(b->d_lnw);
    cudaFree(b->d_pacc);
    cudaFree(b->d_w32);
    cudaFree(b->d_hist);
    cudaFree(b->d_ctl);
    cudaFree(b->d_recs);
    cudaFree(b->d_inst);
    cudaFree(b->d_items);
    cudaFree(b->d_counters);
    cudaFree(b->d_err);
    if (b->h_running) cudaFreeHost(b->h_running);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
}

uint32_t wpr_of(uint32_t L) { return (L + 15) / 16; }

// Sweep arguments of instance i (muca_delta_multigpu.cu:740-742: keys
// {2W, 0xdecafbad}, {2W + 50000, 0x11cafead}; counter word 1 = 100 + 1000 * device).
SweepArgs inst_args(const muca_batch *b, uint32_t i)
{
    const muca_instance &m = b->inst[i];
    SweepArgs a{};
    a.lat = b->d_lat + b->off_lat[i];
    a.ej = b->d_ej + b->off_chain[i];
    a.edel = b->d_edel + b->off_chain[i];
    a.mag = b->d_mag + b->off_chain[i];
    a.w = b->d_w32 + b->off_w[i];
    a.hist = b->d_hist + b->off_w[i];
    a.L = m.L;
    a.N = m.L * m.L;
    a.WPR = wpr_of(m.L);
    a.nchains = m.nchains;
    a.chains_per_dev = m.nchains;
    a.seed_base = 100u + 1000u * m.seed;
    a.seed_dev_mul = 1000u;
    a.k1_mul = 2; a.k1_add = 0; a.k1_hi = 0xdecafbadu;
    a.k3_mul = 2; a.k3_add = 50000; a.k3_hi = 0x11cafeadu;
    a.therm = a.N;
    a.log_eps = b->log_eps;
    a.dyn = &b->d_ctl[i].st.k;
    a.err = b->d_err;
    return a;
}

// Lays the instances out for `cpb` chains per block and uploads the kernel
// tables (instances and the work list sorted by decreasing cost).
muca_status set_layout(muca_batch *b, uint32_t cpb, uint32_t rule)
{
    b->off_lat.assign(b->n, 0);
    size_t words = 0;
    std::vector<BatchItem> items;
    for (uint32_t i = 0; i < b->n; ++i) {
        const muca_instance &m = b->inst[i];
        const uint32_t blocks = (m.nchains + cpb - 1) / cpb;
        b->off_lat[i] = words;
        words += (size_t)blocks * cpb * m.L * wpr_of(m.L);
        for (uint32_t k = 0; k < blocks; ++k) items.push_back({i, k});
    }
    // largest lattices first (an item costs about N attempts per chain and
    // iteration); ties in instance and block order
    std::stable_sort(items.begin(), items.end(), [&](const BatchItem &x, const BatchItem &y) {
        return b->inst[x.inst].L > b->inst[y.inst].L;
    });
    if (words > b->lat_cap) {
        cudaFree(b->d_lat);
        b->d_lat = nullptr;
        BCUDA(b, bmalloc(b, &b->d_lat, words));
        b->lat_cap = words;
    }
    b->lat_words = words;
    if (items.size() > b->items_cap) {
        cudaFree(b->d_items);
        b->d_items = nullptr;
        BCUDA(b, bmalloc(b, &b->d_items, items.size()));
        b->items_cap = items.size();
    }
    b->n_items = (uint32_t)items.size();
    BCUDA(b, cudaMemcpyAsync(b->d_items, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice,
                             b->stream));
    std::vector<BatchInst> ti(b->n);
    for (uint32_t i = 0; i < b->n; ++i) {
        BatchInst &t = ti[i];
        std::memset(&t, 0, sizeof t);
        t.a = inst_args(b, i);
        t.ctl = b->d_ctl + i;
        t.lnw = b->d_lnw + b->off_w[i];
        t.p_acc = b->d_pacc + b->off_w[i];
        t.w32 = b->d_w32 + b->off_w[i];
        for (int d = -8; d <= 8; ++d) t.btab[d + 8] = (float)(-b->inst[i].beta * (double)d);
        t.rule = rule;
    }
    BCUDA(b, cudaMemcpyAsync(b->d_inst, ti.data(), ti.size() * sizeof(BatchInst), cudaMemcpyHostToDevice, b->stream));
    BCUDA(b, cudaStreamSynchronize(b->stream));  // `items`/`ti` are pageable locals
    return MUCA_OK;
}

// Dynamic shared memory a sweep block may use: the device's opt-in limit less
// a reserve for the kernel's static shared memory.
size_t smem_budget(const muca_batch *b) { return b->smem_optin > 1024 ? b->smem_optin - 1024 : 0; }

// Launch shared memory of a shape: the largest block over the instances, each
// with its lattice in shared memory where the shape puts it there
// (kLatWhereFits: where the block stays within the budget; the sweep kernel
// makes the same choice per instance against the launch's size), and a
// lattice left in global memory with its four-row ring where that fits the
// budget (the kernel again decides per instance against the launch's size).
size_t shape_smem(const muca_batch *b, uint32_t cpb, uint32_t lat, bool hist_smem)
{
    size_t smem = 0;
    for (const muca_instance &m : b->inst) {
        const size_t with = batch_sweep_smem(m.L, cpb, true, hist_smem);
        const size_t ring = batch_sweep_smem(m.L, cpb, false, hist_smem, true);
        const size_t without = ring <= smem_budget(b) ? ring : batch_sweep_smem(m.L, cpb, false, hist_smem);
        const bool in = lat == kLatShared || (lat == kLatWhereFits && with <= smem_budget(b));
        smem = std::max(smem, in ? with : without);
    }
    return smem;
}

muca_status apply_shape(muca_batch *b, const muca_batch_shape &s, uint32_t rule)
{
    if (muca_status st = set_layout(b, s.chains_per_block, rule)) return st;
    const size_t smem = shape_smem(b, s.chains_per_block, s.lattice_in_smem, s.hist_in_smem);
    int per_sm = 0;
    BCUDA(b, batch_sweep_occupancy(s.chains_per_block, b->rounds, s.lattice_in_smem, s.hist_in_smem, smem, &per_sm));
    if (per_sm < 1) return bfail(b, MUCA_ERR_BAD_ARG, "shape does not fit on an SM");
    b->shape = s;
    b->shape.blocks_per_sm = (uint32_t)per_sm;
    b->smem = smem;
    b->threads = (s.chains_per_block + 31u) / 32u * 32u;
    b->grid = (uint32_t)(b->sms * per_sm);
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return MUCA_OK;
}

// Reference weight-program initial spins (muca_delta_multigpu.cu:340-351)
// with emulated device index = seed, then E_J and E_Delta; graded: the same
// Philox words through graded_spin (MUCA_INIT_GRADED).
muca_status init_chains(muca_batch *b, bool graded = false)
{
    for (uint32_t i = 0; i < b->n; ++i) {
        const muca_instance &m = b->inst[i];
        InitArgs ia{};
        ia.rounds = 7;
        ia.key0_mul = 10; ia.key0_jack_mul = 2; ia.key1 = 0xdecafbadu;
        ia.ctr0[0] = 2u * m.seed; ia.ctr0[1] = 100; ia.ctr0[2] = 0xBADCAB1Eu; ia.ctr0[3] = 0xBADC0DEDu;
        ia.ctr0_dev_mul[0] = 2; ia.ctr_word = 0;
        ia.chain_offset = m.seed * m.nchains;
        ia.graded = graded ? 1u : 0u;
        const uint32_t cpb = b->shape.chains_per_block;
        uint32_t *lat = b->d_lat + b->off_lat[i];
        BCUDA(b, launch_init(lat, m.L, wpr_of(m.L), cpb, m.nchains, m.nchains, 0, ia, b->stream));
        BCUDA(b, launch_energies(lat, b->d_ej + b->off_chain[i], b->d_edel + b->off_chain[i],
                                 b->d_mag + b->off_chain[i], m.L, wpr_of(m.L), cpb, m.nchains, b->stream));
    }
    return MUCA_OK;
}

// Run state of every instance for a run with options `o` (the reference's
// loop variables, muca_delta_multigpu.cu:314,336-338).
std::vector<RunCtl> make_ctl(const muca_batch *b, const muca_batch_run_opts *o)
{
    std::vector<RunCtl> h(b->n);
    for (uint32_t i = 0; i < b->n; ++i) {
        const muca_instance &m = b->inst[i];
        RunCtl &c = h[i];
        std::memset(&c, 0, sizeof c);
        const uint32_t N = m.L * m.L;
        c.st.k = 0;
        c.st.nup = o->starting_sweeps ? o->starting_sweeps * N : o->starting_M;
        if (o->nup_schedule == 4) {
            // multiplied at the top of every iteration, the first included
            // (muca_mag.cpp:131), as the single-context run does
            const unsigned long long nx = (unsigned long long)((double)c.st.nup * 1.05);
            const uint32_t cap = o->nup_max ? o->nup_max : (1u << 30);
            c.st.nup = nx > cap ? (cap > c.st.nup ? cap : c.st.nup) : (uint32_t)nx;
        }
        c.st.width = 10;
        c.st.total_run = (unsigned long long)c.st.nup * m.nchains;
        c.N = N;
        c.nchains_total = m.nchains;
        c.rule = o->rule;
        c.hold = 0;
        c.flat_minmean = o->flat_minmean;
        c.max_iter = o->max_iter ? o->max_iter : 1000000u;
        c.sched = o->nup_schedule;
        c.nup_max = o->nup_max;
        c.mom_thr = o->min_over_mean > 0 ? o->min_over_mean : 0.5;
        c.dkl_max = o->d_kl_max > 0 ? o->d_kl_max : 1e-4;
        c.recs = b->d_recs + i;
        c.rec_cap = 1;
        c.rec_ring = 1;
    }
    return h;
}

muca_status upload_ctl(muca_batch *b, const std::vector<RunCtl> &h)
{
    BCUDA(b, cudaMemcpyAsync(b->d_ctl, h.data(), h.size() * sizeof(RunCtl), cudaMemcpyHostToDevice, b->stream));
    BCUDA(b, cudaStreamSynchronize(b->stream));  // `h` is pageable
    return MUCA_OK;
}

// Run state for timing sweeps: iteration 0, nup = N, nothing stopped.
muca_status upload_tuning_ctl(muca_batch *b)
{
    muca_batch_run_opts o{};
    o.starting_M = 1;
    std::vector<RunCtl> h = make_ctl(b, &o);
    for (uint32_t i = 0; i < b->n; ++i) h[i].st.nup = b->inst[i].L * b->inst[i].L;
    return upload_ctl(b, h);
}

muca_status sweep_once(muca_batch *b)
{
    BCUDA(b, launch_batch_prep(b->d_inst, b->n, b->d_counters, b->d_counters + 1, b->stream));
    BCUDA(b, launch_batch_sweep(b->d_inst, b->d_items, b->n_items, b->d_counters, b->shape.chains_per_block,
                                b->rounds, b->shape.lattice_in_smem, b->shape.hist_in_smem, b->grid, b->smem,
                                b->stream));
    return MUCA_OK;
}

muca_status autotune(muca_batch *b)
{
    const uint32_t cpbs[] = {32, 64, 128, 256};
    cudaEvent_t e0, e1;
    BCUDA(b, cudaEventCreate(&e0));
    BCUDA(b, cudaEventCreate(&e1));
    muca_batch_shape best{};
    best.ms = 1e30;
    b->tried.clear();
    muca_status rs = MUCA_OK;
    for (uint32_t cpb : cpbs) {
        for (uint32_t ls = kLatGlobal; ls <= kLatWhereFits && rs == MUCA_OK; ++ls) {
            for (int hs = 0; hs < 2 && rs == MUCA_OK; ++hs) {
                const size_t smem = shape_smem(b, cpb, ls, hs);
                if (smem > smem_budget(b)) continue;
                if (ls == kLatWhereFits) {
                    // only a mix differs from the all-global and all-shared shapes
                    uint32_t in = 0;
                    for (const muca_instance &m : b->inst) in += batch_sweep_smem(m.L, cpb, true, hs) <= smem_budget(b);
                    if (in == 0 || in == b->n) continue;
                }
                muca_batch_shape s{};
                s.chains_per_block = cpb;
                s.lattice_in_smem = (uint32_t)ls;
                s.hist_in_smem = (uint32_t)hs;
                if ((rs = apply_shape(b, s, 0)) != MUCA_OK) break;
                if ((rs = init_chains(b)) != MUCA_OK) break;
                if ((rs = upload_tuning_ctl(b)) != MUCA_OK) break;
                if ((rs = sweep_once(b)) != MUCA_OK) break;  // warm-up
                cudaEventRecord(e0, b->stream);
                for (int r = 0; r < 2 && rs == MUCA_OK; ++r) rs = sweep_once(b);
                cudaEventRecord(e1, b->stream);
                if (rs != MUCA_OK) break;
                const cudaError_t e = cudaEventSynchronize(e1);
                if (e != cudaSuccess) { rs = bfail(b, MUCA_ERR_CUDA, "autotune: %s", cudaGetErrorString(e)); break; }
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                s = b->shape;
                s.ms = ms * 0.5;
                b->tried.push_back(s);
                if (s.ms < best.ms) best = s;
            }
        }
        if (rs != MUCA_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rs != MUCA_OK) return rs;
    if (b->tried.empty()) return bfail(b, MUCA_ERR_BAD_ARG, "no block shape fits these instances");
    if (muca_status st = apply_shape(b, best, 0)) return st;
    b->shape.ms = best.ms;
    return MUCA_OK;
}

muca_status check_inst(muca_batch *b, uint32_t i, size_t n, size_t expect)
{
    if (i >= b->n) return bfail(b, MUCA_ERR_BAD_ARG, "instance %u of %u", i, b->n);
    if (n != expect) return bfail(b, MUCA_ERR_BAD_ARG, "n=%zu, expected %zu", n, expect);
    return MUCA_OK;
}

}  // namespace

extern "C" {

const char *muca_batch_last_error(const muca_batch *b) { return b ? b->err.c_str() : g_batch_err.c_str(); }

muca_status muca_batch_create(const muca_batch_params *p, const muca_instance *inst, uint32_t n, muca_batch **out)
{
    if (!p || !inst || !out) return bfail(nullptr, MUCA_ERR_BAD_ARG, "NULL argument");
    *out = nullptr;
    if (n == 0 || n > 65536) return bfail(nullptr, MUCA_ERR_BAD_ARG, "n=%u instances (1..65536)", n);
    const uint32_t rounds = p->rounds ? p->rounds : 7;
    if (rounds != 7 && rounds != 10) return bfail(nullptr, MUCA_ERR_BAD_ARG, "rounds=%u (7 or 10)", rounds);
    uint64_t chains = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const muca_instance &m = inst[i];
        if (m.L < 8 || m.L > 128 || m.L % 8)
            return bfail(nullptr, MUCA_ERR_BAD_ARG, "instance %u: L=%u (8..128, a multiple of 8)", i, m.L);
        if (m.nchains == 0 || m.nchains > 65536)
            return bfail(nullptr, MUCA_ERR_BAD_ARG, "instance %u: nchains=%u (1..65536)", i, m.nchains);
        if (!(m.beta > 0.0) || !std::isfinite(m.beta))
            return bfail(nullptr, MUCA_ERR_BAD_ARG, "instance %u: beta=%g (positive, finite)", i, m.beta);
        chains += m.nchains;
    }
    if (chains > (1ull << 26)) return bfail(nullptr, MUCA_ERR_BAD_ARG, "%llu chains in total (at most 2^26)",
                                            (unsigned long long)chains);
    muca_batch *b = new muca_batch();
    b->device = p->device;
    b->rounds = (int)rounds;
    b->inst.assign(inst, inst + n);
    b->n = n;
    auto bail = [&](muca_status st) {
        g_batch_err = b->err;
        free_all(b);
        delete b;
        return st;
    };
#define BTRY(x)                                                                                   \
    do {                                                                                          \
        cudaError_t _e = (x);                                                                     \
        if (_e != cudaSuccess) { bfail(b, MUCA_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(_e)); return bail(MUCA_ERR_CUDA); } \
    } while (0)
    BTRY(cudaSetDevice(b->device));
    int optin = 0;
    BTRY(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device));
    BTRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device));
    b->smem_optin = (size_t)optin;
    if (p->stream) {
        b->stream = (cudaStream_t)p->stream;
    } else {
        BTRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
        b->own_stream = true;
    }
    b->off_w.resize(n);
    b->off_chain.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t N = inst[i].L * inst[i].L;
        b->off_w[i] = b->total_w;
        b->total_w += N + 1;
        b->off_chain[i] = b->total_chains;
        b->total_chains += inst[i].nchains;
        b->max_N = std::max(b->max_N, N);
        b->max_L = std::max(b->max_L, inst[i].L);
    }
    BTRY(bmalloc(b, &b->d_ej, b->total_chains));
    BTRY(bmalloc(b, &b->d_edel, b->total_chains));
    BTRY(bmalloc(b, &b->d_mag, b->total_chains));
    BTRY(bmalloc(b, &b->d_lnw, b->total_w));
    BTRY(bmalloc(b, &b->d_pacc, b->total_w));
    BTRY(bmalloc(b, &b->d_w32, b->total_w));
    BTRY(bmalloc(b, &b->d_hist, b->total_w));
    BTRY(bmalloc(b, &b->d_ctl, n));
    BTRY(bmalloc(b, &b->d_recs, n));
    BTRY(bmalloc(b, &b->d_inst, n));
    BTRY(bmalloc(b, &b->d_counters, 2));
    BTRY(bmalloc(b, &b->d_err, 1));
    BTRY(cudaMallocHost((void **)&b->h_running, sizeof(uint32_t)));
    BTRY(cudaMemsetAsync(b->d_lnw, 0, b->total_w * 8, b->stream));
    BTRY(cudaMemsetAsync(b->d_pacc, 0, b->total_w * 8, b->stream));
    BTRY(cudaMemsetAsync(b->d_w32, 0, b->total_w * 4, b->stream));
    BTRY(cudaMemsetAsync(b->d_hist, 0, b->total_w * 8, b->stream));
    BTRY(cudaMemsetAsync(b->d_recs, 0, n * sizeof(IterRecordDev), b->stream));
    BTRY(cudaMemsetAsync(b->d_err, 0, sizeof(unsigned int), b->stream));
    BTRY(device_log_eps(b->device, b->stream, &b->log_eps));
    BTRY(prepare_batch_update(b->max_N, 1));
    muca_status st;
    if (p->shape_chains_per_block) {
        muca_batch_shape s{};
        s.chains_per_block = p->shape_chains_per_block;
        s.lattice_in_smem = p->shape_lattice_in_smem;
        s.hist_in_smem = p->shape_hist_in_smem;
        if (s.chains_per_block > 256 || s.chains_per_block % 32) {
            bfail(b, MUCA_ERR_BAD_ARG, "chains per block %u (32..256, a multiple of 32)", s.chains_per_block);
            return bail(MUCA_ERR_BAD_ARG);
        }
        if (s.lattice_in_smem > kLatWhereFits || s.hist_in_smem > 1) {
            bfail(b, MUCA_ERR_BAD_ARG, "lattice_in_smem %u (0..2), hist_in_smem %u (0..1)", s.lattice_in_smem,
                  s.hist_in_smem);
            return bail(MUCA_ERR_BAD_ARG);
        }
        const size_t smem = shape_smem(b, s.chains_per_block, s.lattice_in_smem, s.hist_in_smem);
        if (smem > smem_budget(b)) {
            bfail(b, MUCA_ERR_BAD_ARG, "shape needs %zu B of shared memory per block (device allows %zu)", smem,
                  smem_budget(b));
            return bail(MUCA_ERR_BAD_ARG);
        }
        st = apply_shape(b, s, 0);
    } else {
        st = autotune(b);
    }
    if (st == MUCA_OK) st = init_chains(b);
    if (st != MUCA_OK) return bail(st);
    BTRY(cudaStreamSynchronize(b->stream));
#undef BTRY
    *out = b;
    return MUCA_OK;
}

muca_status muca_batch_destroy(muca_batch *b)
{
    if (!b) return MUCA_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    free_all(b);
    delete b;
    return MUCA_OK;
}

muca_status muca_batch_get_info(const muca_batch *b, muca_batch_info *o)
{
    if (!b || !o) return bfail(nullptr, MUCA_ERR_BAD_ARG, "NULL argument");
    std::memset(o, 0, sizeof *o);
    o->n_instances = b->n;
    o->n_items = b->n_items;
    o->grid = b->grid;
    o->threads = b->threads;
    o->smem_bytes = (uint32_t)b->smem;
    o->shape = b->shape;
    o->n_tried = (uint32_t)std::min<size_t>(b->tried.size(), 32);
    for (uint32_t i = 0; i < o->n_tried; ++i) o->tried[i] = b->tried[i];
    o->device_bytes = b->device_bytes;
    o->log_bracket = b->log_eps;
    return MUCA_OK;
}

muca_status muca_batch_init_chains(muca_batch *b)
{
    if (!b) return bfail(nullptr, MUCA_ERR_BAD_ARG, "batch is NULL");
    BCUDA(b, cudaSetDevice(b->device));
    if (muca_status st = init_chains(b)) return st;
    BCUDA(b, cudaStreamSynchronize(b->stream));
    return MUCA_OK;
}

muca_status muca_batch_set_weights(muca_batch *b, uint32_t i, const double *lnw, size_t n)
{
    if (!b || !lnw) return bfail(b, MUCA_ERR_BAD_ARG, "NULL argument");
    if (i >= b->n) return bfail(b, MUCA_ERR_BAD_ARG, "instance %u of %u", i, b->n);
    const size_t N1 = (size_t)b->inst[i].L * b->inst[i].L + 1;
    if (muca_status st = check_inst(b, i, n, N1)) return st;
    for (size_t k = 0; k < n; ++k)
        if (!std::isfinite(lnw[k])) return bfail(b, MUCA_ERR_BAD_ARG, "weight %zu is not finite", k);
    BCUDA(b, cudaSetDevice(b->device));
    BCUDA(b, cudaMemcpyAsync(b->d_lnw + b->off_w[i], lnw, n * 8, cudaMemcpyHostToDevice, b->stream));
    BCUDA(b, launch_weights_to_f32(b->d_lnw + b->off_w[i], b->d_w32 + b->off_w[i], (uint32_t)n, b->stream));
    BCUDA(b, cudaMemsetAsync(b->d_pacc + b->off_w[i], 0, n * 8, b->stream));
    BCUDA(b, cudaStreamSynchronize(b->stream));
    return MUCA_OK;
}

muca_status muca_batch_get_weights(muca_batch *b, uint32_t i, double *lnw, size_t n)
{
    if (!b || !lnw) return bfail(b, MUCA_ERR_BAD_ARG, "NULL argument");
    if (i >= b->n) return bfail(b, MUCA_ERR_BAD_ARG, "instance %u of %u", i, b->n);
    if (muca_status st = check_inst(b, i, n, (size_t)b->inst[i].L * b->inst[i].L + 1)) return st;
    BCUDA(b, cudaSetDevice(b->device));
    BCUDA(b, cudaMemcpyAsync(lnw, b->d_lnw + b->off_w[i], n * 8, cudaMemcpyDeviceToHost, b->stream));
    BCUDA(b, cudaStreamSynchronize(b->stream));
    return MUCA_OK;
}

muca_status muca_batch_get_histogram(muca_batch *b, uint32_t i, uint64_t *h, size_t n)
{
    if (!b || !h) return bfail(b, MUCA_ERR_BAD_ARG, "NULL argument");
    if (i >= b->n) return bfail(b, MUCA_ERR_BAD_ARG, "instance %u of %u", i, b->n);
    if (muca_status st = check_inst(b, i, n, (size_t)b->inst[i].L * b->inst[i].L + 1)) return st;
    BCUDA(b, cudaSetDevice(b->device));
    BCUDA(b, cudaMemcpyAsync(h, b->d_hist + b->off_w[i], n * 8, cudaMemcpyDeviceToHost, b->stream));
    BCUDA(b, cudaStreamSynchronize(b->stream));
    return MUCA_OK;
}

muca_status muca_batch_run(muca_batch *b, const muca_batch_run_opts *o, muca_batch_result *res, double *seconds)
{
    if (!b || !o) return bfail(b, MUCA_ERR_BAD_ARG, "NULL argument");
    if (o->rule > MUCA_UPDATE_RECURSION) return bfail(b, MUCA_ERR_BAD_ARG, "rule %u", o->rule);
    if (o->starting_M == 0 && o->starting_sweeps == 0)
        return bfail(b, MUCA_ERR_BAD_ARG, "starting_M or starting_sweeps must be >= 1");
    if (o->starting_sweeps > 4096) return bfail(b, MUCA_ERR_BAD_ARG, "starting_sweeps=%u (at most 4096)", o->starting_sweeps);
    if (o->nup_schedule > 5) return bfail(b, MUCA_ERR_BAD_ARG, "nup_schedule %u (0..5)", o->nup_schedule);
    const uint32_t K = o->graph_iters ? o->graph_iters : 16u;
    if (K > 4096) return bfail(b, MUCA_ERR_BAD_ARG, "graph_iters=%u (at most 4096)", K);
    BCUDA(b, cudaSetDevice(b->device));
    if (o->graded_init > 1) return bfail(b, MUCA_ERR_BAD_ARG, "graded_init %u (0..1)", o->graded_init);
    if (o->reinit_chains) {
        if (muca_status st = init_chains(b, o->graded_init != 0)) return st;
    }
    // the instance table carries the update rule
    if (muca_status st = set_layout(b, b->shape.chains_per_block, o->rule)) return st;
    if (muca_status st = upload_ctl(b, make_ctl(b, o))) return st;
    const int rec = o->rule == MUCA_UPDATE_RECURSION ? 1 : 0;
    if (!b->graph || b->graph_iters != K || b->graph_rec != rec) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        // K iterations of the reference loop body (:374-477) for every instance
        BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        for (uint32_t k = 0; k < K && e == cudaSuccess; ++k) {
            e = launch_batch_prep(b->d_inst, b->n, b->d_counters, b->d_counters + 1, b->stream);
            if (e == cudaSuccess)
                e = launch_batch_sweep(b->d_inst, b->d_items, b->n_items, b->d_counters, b->shape.chains_per_block,
                                       b->rounds, b->shape.lattice_in_smem, b->shape.hist_in_smem, b->grid, b->smem,
                                       b->stream);
            if (e == cudaSuccess) e = launch_batch_update(b->d_inst, b->n, b->max_N, rec, b->d_counters + 1, b->stream);
        }
        cudaGraph_t g = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return bfail(b, MUCA_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        const cudaError_t e3 = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e3 != cudaSuccess) {
            b->graph = nullptr;
            return bfail(b, MUCA_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e3));
        }
        b->graph_iters = K;
        b->graph_rec = rec;
    }
    cudaEvent_t e0, e1;
    BCUDA(b, cudaEventCreate(&e0));
    BCUDA(b, cudaEventCreate(&e1));
    const uint32_t max_iter = o->max_iter ? o->max_iter : 1000000u;
    const uint64_t max_launches = (max_iter + K - 1) / K + 1;
    cudaError_t e = cudaEventRecord(e0, b->stream);
    for (uint64_t l = 0; l < max_launches && e == cudaSuccess; ++l) {
        e = cudaGraphLaunch(b->graph, b->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(b->h_running, b->d_counters + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e == cudaSuccess && *b->h_running == 0) break;
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return bfail(b, MUCA_ERR_CUDA, "batch run: %s", cudaGetErrorString(e));
    if (seconds) *seconds = ms * 1e-3;
    unsigned int err = 0;
    BCUDA(b, cudaMemcpy(&err, b->d_err, sizeof err, cudaMemcpyDeviceToHost));
    if (err) return bfail(b, MUCA_ERR_TIMEOUT, "a bounded device wait gave up (error word 0x%x)", err);
    std::vector<RunCtl> ctl(b->n);
    std::vector<IterRecordDev> recs(b->n);
    BCUDA(b, cudaMemcpy(ctl.data(), b->d_ctl, b->n * sizeof(RunCtl), cudaMemcpyDeviceToHost));
    BCUDA(b, cudaMemcpy(recs.data(), b->d_recs, b->n * sizeof(IterRecordDev), cudaMemcpyDeviceToHost));
    uint32_t not_conv = 0;
    for (uint32_t i = 0; i < b->n; ++i) {
        const IterState &s = ctl[i].st;
        if (!s.converged) ++not_conv;
        if (!res) continue;
        muca_batch_result &r = res[i];
        std::memset(&r, 0, sizeof r);
        r.iterations = s.converged ? s.k + 1 : s.k;
        r.converged = s.converged;
        r.width = s.width;
        r.reach_iter = s.reach ? s.reach_k : 0xFFFFFFFFu;
        r.total_run = s.total_run;
        r.d_kl = recs[i].d_kl;
        r.min_over_mean = recs[i].min_over_mean;
        r.nupdates = recs[i].nupdates;
    }
    if (not_conv) return bfail(b, MUCA_ERR_NOT_CONVERGED, "%u of %u instances did not converge", not_conv, b->n);
    return MUCA_OK;
}

}  // extern "C"
