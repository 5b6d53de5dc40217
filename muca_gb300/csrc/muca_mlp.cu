// muca_mlp.cu -- C ABI of the warm-start MLP (k_mlp.cu).
//
// No counterpart in the reference, whose only alternative to a zero initial
// weight is an extrapolated weight file read by the `continuing` path
// (muca_delta_multigpu.cu:223-235).  The network is trained on weights that
// converged runs of this engine produced, then predicts lnW for an unseen
// (L, T, Delta); muca_mlp_log_weights returns that prediction in the form
// muca_set_weights / muca_batch_set_weights take.
#include "../../include/muca.h"
#include "muca_internal.h"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace muca;

struct muca_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    float *d_P = nullptr, *d_G = nullptr, *d_m = nullptr, *d_v = nullptr;
    uint32_t *d_step = nullptr;  // [0] step count, [1] step count at the start of train()
    float *d_X = nullptr, *d_T = nullptr;
    uint32_t n_data = 0;
    float *d_scratch = nullptr;
    uint32_t scratch_B = 0;
    float *d_losses = nullptr;
    uint32_t losses_cap = 0;
    cudaGraphExec_t graph = nullptr;
    uint32_t graph_B = 0, graph_K = 0, graph_seed = 0;
    float graph_lr = 0;
    std::string err;
};

namespace {

std::string g_mlp_err;

muca_status mfail(muca_mlp *m, muca_status st, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (m) m->err = buf; else g_mlp_err = buf;
    return st;
}

#define MCUDA(m, x)                                                                              \
    do {                                                                                         \
        cudaError_t _e = (x);                                                                    \
        if (_e != cudaSuccess) return mfail((m), MUCA_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(_e)); \
    } while (0)

void free_all(muca_mlp *m)
{
    if (m->graph) cudaGraphExecDestroy(m->graph);
    cudaFree(m->d_P);
    cudaFree(m->d_G);
    cudaFree(m->d_m);
    cudaFree(m->d_v);
    cudaFree(m->d_step);
    cudaFree(m->d_X);
    cudaFree(m->d_T);
    cudaFree(m->d_scratch);
    cudaFree(m->d_losses);
    if (m->own_stream && m->stream) cudaStreamDestroy(m->stream);
}

// splitmix64 (Steele, Lea, Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014): the initial parameters, identical on every host.
uint64_t splitmix64(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Every weight and bias of a layer with fan_in inputs uniform in
// [-1/sqrt(fan_in), 1/sqrt(fan_in)] (the usual default of a linear layer).
std::vector<float> init_params(uint64_t seed)
{
    std::vector<float> p(mlp_param_count());
    uint64_t s = seed;
    const int fan[4] = {4, 128, 128, 128};
    const size_t size[4] = {128 * 4 + 128, 128 * 128 + 128, 128 * 128 + 128, 128 + 1};
    size_t off = 0;
    for (int l = 0; l < 4; ++l) {
        const double bound = 1.0 / std::sqrt((double)fan[l]);
        for (size_t i = 0; i < size[l]; ++i) {
            const double u = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
            p[off + i] = (float)((2.0 * u - 1.0) * bound);
        }
        off += size[l];
    }
    return p;
}

muca_status ensure_scratch(muca_mlp *m, uint32_t B)
{
    if (B <= m->scratch_B) return MUCA_OK;
    cudaFree(m->d_scratch);
    m->d_scratch = nullptr;
    MCUDA(m, cudaMalloc(&m->d_scratch, mlp_scratch_floats(B) * sizeof(float)));
    m->scratch_B = B;
    if (m->graph) {  // a captured step refers to the old scratch
        cudaGraphExecDestroy(m->graph);
        m->graph = nullptr;
    }
    return MUCA_OK;
}

muca_status ensure_losses(muca_mlp *m, uint32_t n)
{
    if (n <= m->losses_cap) return MUCA_OK;
    cudaFree(m->d_losses);
    m->d_losses = nullptr;
    MCUDA(m, cudaMalloc(&m->d_losses, (size_t)n * sizeof(float)));
    m->losses_cap = n;
    if (m->graph) {
        cudaGraphExecDestroy(m->graph);
        m->graph = nullptr;
    }
    return MUCA_OK;
}

muca_status reset_optimizer(muca_mlp *m)
{
    const size_t np = mlp_param_count();
    MCUDA(m, cudaMemsetAsync(m->d_m, 0, np * sizeof(float), m->stream));
    MCUDA(m, cudaMemsetAsync(m->d_v, 0, np * sizeof(float), m->stream));
    MCUDA(m, cudaMemsetAsync(m->d_step, 0, 2 * sizeof(uint32_t), m->stream));
    return MUCA_OK;
}

}  // namespace

extern "C" {

const char *muca_mlp_last_error(const muca_mlp *m) { return m ? m->err.c_str() : g_mlp_err.c_str(); }

size_t muca_mlp_param_count(void) { return mlp_param_count(); }

muca_status muca_mlp_create(int32_t device, uint64_t seed, void *stream, muca_mlp **out)
{
    if (!out) return mfail(nullptr, MUCA_ERR_BAD_ARG, "out is NULL");
    *out = nullptr;
    muca_mlp *m = new muca_mlp();
    m->device = device;
    auto bail = [&](muca_status st) {
        g_mlp_err = m->err;
        free_all(m);
        delete m;
        return st;
    };
#define MTRY(x)                                                                                   \
    do {                                                                                          \
        cudaError_t _e = (x);                                                                     \
        if (_e != cudaSuccess) { mfail(m, MUCA_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(_e)); return bail(MUCA_ERR_CUDA); } \
    } while (0)
    MTRY(cudaSetDevice(device));
    if (stream) {
        m->stream = (cudaStream_t)stream;
    } else {
        MTRY(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
        m->own_stream = true;
    }
    const size_t np = mlp_param_count();
    MTRY(cudaMalloc(&m->d_P, np * sizeof(float)));
    MTRY(cudaMalloc(&m->d_G, np * sizeof(float)));
    MTRY(cudaMalloc(&m->d_m, np * sizeof(float)));
    MTRY(cudaMalloc(&m->d_v, np * sizeof(float)));
    MTRY(cudaMalloc(&m->d_step, 2 * sizeof(uint32_t)));
    MTRY(mlp_prepare());
    const std::vector<float> p = init_params(seed);
    MTRY(cudaMemcpyAsync(m->d_P, p.data(), np * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MTRY(cudaMemsetAsync(m->d_G, 0, np * sizeof(float), m->stream));
    if (reset_optimizer(m) != MUCA_OK) return bail(MUCA_ERR_CUDA);
    MTRY(cudaStreamSynchronize(m->stream));
#undef MTRY
    *out = m;
    return MUCA_OK;
}

muca_status muca_mlp_destroy(muca_mlp *m)
{
    if (!m) return MUCA_OK;
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    free_all(m);
    delete m;
    return MUCA_OK;
}

muca_status muca_mlp_get_params(muca_mlp *m, float *p, size_t n)
{
    if (!m || !p) return mfail(m, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n != mlp_param_count()) return mfail(m, MUCA_ERR_BAD_ARG, "n=%zu, expected %zu", n, mlp_param_count());
    MCUDA(m, cudaSetDevice(m->device));
    MCUDA(m, cudaMemcpyAsync(p, m->d_P, n * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCUDA(m, cudaStreamSynchronize(m->stream));
    return MUCA_OK;
}

muca_status muca_mlp_set_params(muca_mlp *m, const float *p, size_t n)
{
    if (!m || !p) return mfail(m, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n != mlp_param_count()) return mfail(m, MUCA_ERR_BAD_ARG, "n=%zu, expected %zu", n, mlp_param_count());
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(p[i])) return mfail(m, MUCA_ERR_BAD_ARG, "parameter %zu is not finite", i);
    MCUDA(m, cudaSetDevice(m->device));
    MCUDA(m, cudaMemcpyAsync(m->d_P, p, n * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    if (muca_status st = reset_optimizer(m)) return st;
    MCUDA(m, cudaStreamSynchronize(m->stream));
    return MUCA_OK;
}

muca_status muca_mlp_set_data(muca_mlp *m, const float *x, const float *t, uint32_t n)
{
    if (!m || !x || !t) return mfail(m, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n == 0 || n > (1u << 28)) return mfail(m, MUCA_ERR_BAD_ARG, "n=%u points (1..2^28)", n);
    MCUDA(m, cudaSetDevice(m->device));
    cudaFree(m->d_X);
    cudaFree(m->d_T);
    m->d_X = m->d_T = nullptr;
    m->n_data = 0;
    MCUDA(m, cudaMalloc(&m->d_X, (size_t)n * 4 * sizeof(float)));
    MCUDA(m, cudaMalloc(&m->d_T, (size_t)n * sizeof(float)));
    MCUDA(m, cudaMemcpyAsync(m->d_X, x, (size_t)n * 4 * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCUDA(m, cudaMemcpyAsync(m->d_T, t, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCUDA(m, cudaStreamSynchronize(m->stream));
    m->n_data = n;
    if (m->graph) {
        cudaGraphExecDestroy(m->graph);
        m->graph = nullptr;
    }
    return MUCA_OK;
}

muca_status muca_mlp_train(muca_mlp *m, uint32_t steps, uint32_t batch, float lr, uint32_t seed, float *losses)
{
    if (!m) return mfail(nullptr, MUCA_ERR_BAD_ARG, "NULL argument");
    if (!m->n_data) return mfail(m, MUCA_ERR_STATE, "no training data (muca_mlp_set_data)");
    if (batch == 0 || batch > 65536) return mfail(m, MUCA_ERR_BAD_ARG, "batch=%u (1..65536)", batch);
    if (!(lr > 0.0f) || !std::isfinite(lr)) return mfail(m, MUCA_ERR_BAD_ARG, "lr=%g", (double)lr);
    if (steps == 0) return MUCA_OK;
    MCUDA(m, cudaSetDevice(m->device));
    if (muca_status st = ensure_scratch(m, batch)) return st;
    if (muca_status st = ensure_losses(m, steps)) return st;
    // the losses of this call are indexed from the step count at its start
    MCUDA(m, cudaMemcpyAsync(m->d_step + 1, m->d_step, sizeof(uint32_t), cudaMemcpyDeviceToDevice, m->stream));
    const uint32_t K = 32;  // steps per captured graph
    if (!m->graph || m->graph_B != batch || m->graph_seed != seed || m->graph_lr != lr || m->graph_K != K) {
        if (m->graph) {
            cudaGraphExecDestroy(m->graph);
            m->graph = nullptr;
        }
        MCUDA(m, cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        for (uint32_t k = 0; k < K && e == cudaSuccess; ++k)
            e = launch_mlp_step(m->d_P, m->d_G, m->d_m, m->d_v, m->d_X, m->d_T, m->n_data, batch, m->d_step,
                                m->d_step + 1, seed, true, lr, m->d_scratch, m->d_losses, m->losses_cap, m->stream);
        cudaGraph_t g = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(m->stream, &g);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return mfail(m, MUCA_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        const cudaError_t e3 = cudaGraphInstantiate(&m->graph, g, 0);
        cudaGraphDestroy(g);
        if (e3 != cudaSuccess) {
            m->graph = nullptr;
            return mfail(m, MUCA_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e3));
        }
        m->graph_B = batch;
        m->graph_seed = seed;
        m->graph_lr = lr;
        m->graph_K = K;
    }
    uint32_t done = 0;
    for (; done + K <= steps; done += K) MCUDA(m, cudaGraphLaunch(m->graph, m->stream));
    for (; done < steps; ++done)
        MCUDA(m, launch_mlp_step(m->d_P, m->d_G, m->d_m, m->d_v, m->d_X, m->d_T, m->n_data, batch, m->d_step,
                                 m->d_step + 1, seed, true, lr, m->d_scratch, m->d_losses, m->losses_cap, m->stream));
    if (losses)
        MCUDA(m, cudaMemcpyAsync(losses, m->d_losses, (size_t)steps * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCUDA(m, cudaStreamSynchronize(m->stream));
    return MUCA_OK;
}

muca_status muca_mlp_grad(muca_mlp *m, const float *x, const float *t, uint32_t n, float *grad, float *loss)
{
    if (!m || !x || !t || !grad) return mfail(m, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n == 0 || n > 65536) return mfail(m, MUCA_ERR_BAD_ARG, "n=%u (1..65536)", n);
    MCUDA(m, cudaSetDevice(m->device));
    if (muca_status st = ensure_scratch(m, n)) return st;
    if (muca_status st = ensure_losses(m, 1)) return st;
    float *Xb = m->d_scratch, *Tb = Xb + (size_t)n * 4;
    MCUDA(m, cudaMemcpyAsync(Xb, x, (size_t)n * 4 * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCUDA(m, cudaMemcpyAsync(Tb, t, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCUDA(m, launch_mlp_step(m->d_P, m->d_G, nullptr, nullptr, nullptr, nullptr, n, n, nullptr, nullptr, 0, false,
                             0.0f, m->d_scratch, m->d_losses, 1, m->stream));
    MCUDA(m, cudaMemcpyAsync(grad, m->d_G, mlp_param_count() * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    if (loss) MCUDA(m, cudaMemcpyAsync(loss, m->d_losses, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCUDA(m, cudaStreamSynchronize(m->stream));
    return MUCA_OK;
}

muca_status muca_mlp_predict(muca_mlp *m, const float *x, uint32_t n, float *y)
{
    if (!m || !x || !y) return mfail(m, MUCA_ERR_BAD_ARG, "NULL argument");
    if (n == 0 || n > (1u << 24)) return mfail(m, MUCA_ERR_BAD_ARG, "n=%u (1..2^24)", n);
    MCUDA(m, cudaSetDevice(m->device));
    if (muca_status st = ensure_scratch(m, n)) return st;
    float *Xb = m->d_scratch, *Y = Xb + (size_t)n * 4 + n;
    MCUDA(m, cudaMemcpyAsync(Xb, x, (size_t)n * 4 * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCUDA(m, launch_mlp_forward(m->d_P, Xb, n, nullptr, Y, m->stream));
    MCUDA(m, cudaMemcpyAsync(y, Y, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCUDA(m, cudaStreamSynchronize(m->stream));
    return MUCA_OK;
}

muca_status muca_mlp_log_weights(muca_mlp *m, uint32_t L, double T, double delta, double *lnw, size_t n)
{
    if (!m || !lnw) return mfail(m, MUCA_ERR_BAD_ARG, "NULL argument");
    if (L < 2 || L > 128) return mfail(m, MUCA_ERR_BAD_ARG, "L=%u outside 2..128", L);
    const uint32_t N = L * L;
    if (n != (size_t)N + 1) return mfail(m, MUCA_ERR_BAD_ARG, "n=%zu, expected N+1=%u", n, N + 1);
    std::vector<float> x((size_t)(N + 1) * 4), y(N + 1);
    for (uint32_t i = 0; i <= N; ++i) {
        x[(size_t)i * 4 + 0] = (float)(L / 128.0);
        x[(size_t)i * 4 + 1] = (float)T;
        x[(size_t)i * 4 + 2] = (float)delta;
        x[(size_t)i * 4 + 3] = (float)((double)i / (double)N);
    }
    if (muca_status st = muca_mlp_predict(m, x.data(), N + 1, y.data())) return st;
    // the network gives the per-site log weight; lnW[0] = 0 as the updates normalise it
    for (uint32_t i = 0; i <= N; ++i) lnw[i] = (double)N * ((double)y[i] - (double)y[0]);
    return MUCA_OK;
}

}  // extern "C"
