/*
 * refgpu.cpp -- launcher for the reference GPU kernels (test infrastructure).
 *
 * The reference kernels (muca_delta_multigpu.cu:737-829 `mcs`, :69-83
 * `computeEnergies`/`computeDeltaE`; produce2_multigpu.cu:401-496 `mcs`,
 * :66-89) are compiled unchanged from the reference sources into cubins in
 * oracle/_ref by oracle/Makefile.  This file loads such a cubin with the CUDA
 * driver API and runs one kernel launch on caller-supplied host buffers in
 * the reference's own layout (lattice int8 [site][chain], "site-major").
 * It is the bit-exact GPU oracle of the GPU tests and the "reference GPU
 * kernel" line of bench.py; the product never loads it.
 *
 * The buffers are sized with the slack the reference kernels need: the
 * production kernel's histogram reset writes one element past
 * (N+1)(N+2)/2, so one extra element is allocated.
 */
#include <cuda.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {
std::map<std::string, CUmodule> g_mods;
char g_err[512];

int fail(const char *what, CUresult r)
{
    const char *s = nullptr;
    cuGetErrorString(r, &s);
    std::snprintf(g_err, sizeof g_err, "%s: %s", what, s ? s : "?");
    return (int)r ? (int)r : -1;
}
#define CK(x) do { CUresult _r = (x); if (_r != CUDA_SUCCESS) return fail(#x, _r); } while (0)

int ensure_ctx()
{
    static bool ok = false;
    if (ok) return 0;
    CK(cuInit(0));
    CUdevice d;
    CK(cuDeviceGet(&d, 0));
    CUcontext c;
    CK(cuDevicePrimaryCtxRetain(&c, d));
    CK(cuCtxSetCurrent(c));
    ok = true;
    return 0;
}

int get_module(const char *path, CUmodule *m)
{
    auto it = g_mods.find(path);
    if (it != g_mods.end()) { *m = it->second; return 0; }
    CK(cuModuleLoad(m, path));
    g_mods[path] = *m;
    return 0;
}

int set_consts(CUmodule m, unsigned L, unsigned NW)
{
    unsigned N = L * L;
    CUdeviceptr p;
    size_t b;
    CK(cuModuleGetGlobal(&p, &b, m, "d_L"));
    CK(cuMemcpyHtoD(p, &L, 4));
    CK(cuModuleGetGlobal(&p, &b, m, "d_N"));
    CK(cuMemcpyHtoD(p, &N, 4));
    CK(cuModuleGetGlobal(&p, &b, m, "d_NUM_WORKERS"));
    CK(cuMemcpyHtoD(p, &NW, 4));
    return 0;
}

/* the host-side tables of muca_delta_multigpu.cu:157-175, as unsigned */
void tables(unsigned L, std::vector<unsigned> &naver, std::vector<unsigned> &index)
{
    unsigned N = L * L;
    naver.assign(4 * N, 0);
    index.assign(N, 0);
    for (unsigned i = 0; i < N; i++) {
        int right = (int)i + 1, left = (int)i - 1, up = (int)(i + L), down = (int)i - (int)L;
        if (right % (int)L == 0) right -= (int)L;
        if (i % L == 0) left += (int)L;
        if (up > (int)N - 1) up -= (int)N;
        if (down < 0) down += (int)N;
        naver[4 * i] = right; naver[4 * i + 1] = left; naver[4 * i + 2] = up; naver[4 * i + 3] = down;
        index[i] = ((unsigned)(0 == ((i / (N / 2)) % 2)) * (2 * i)) % N
                 + ((unsigned)(1 == ((i / (N / 2)) % 2)) * (2 * i + 1)) % N;
    }
}

struct DevBuf {
    CUdeviceptr p = 0;
    ~DevBuf() { if (p) cuMemFree(p); }
};
}  // namespace

extern "C" {

const char *refgpu_last_error(void) { return g_err; }

/* One launch of the reference weight kernel.  lat: int8 [N][NW]; hist: u32
 * [N+1] (output of this launch only); w: float [N+1]; energy/deltaE: [NW]
 * in/out.  If compute_energies, the reference init kernels fill
 * energy/deltaE first.  NW must be a multiple of 256 (the reference launch
 * shape NUM_WORKERS/256 blocks of 256).  ms (optional) gets the kernel time. */
int refgpu_weight_mcs(const char *cubin, unsigned L, unsigned NW, int8_t *lat, unsigned *hist, const float *w,
                      int *energy, int *deltaE, unsigned iter, unsigned seed, unsigned therm, unsigned nup,
                      int compute_energies, float *ms)
{
    if (NW == 0 || NW % 256 != 0 || L < 2) { std::snprintf(g_err, sizeof g_err, "bad NW/L"); return -1; }
    if (int e = ensure_ctx()) return e;
    CUmodule m;
    if (int e = get_module(cubin, &m)) return e;
    if (int e = set_consts(m, L, NW)) return e;
    CUfunction fm, fe, fd;
    CK(cuModuleGetFunction(&fm, m, "_Z3mcsPaPjPfS0_S0_PiS2_jjjj"));
    CK(cuModuleGetFunction(&fe, m, "_Z15computeEnergiesPaPi"));
    CK(cuModuleGetFunction(&fd, m, "_Z13computeDeltaEPaPi"));
    unsigned N = L * L;
    std::vector<unsigned> naver, index;
    tables(L, naver, index);
    DevBuf dl, dh, dw, dn, di, de, dd;
    CK(cuMemAlloc(&dl.p, (size_t)N * NW));
    CK(cuMemAlloc(&dh.p, (size_t)(N + 1) * 4));
    CK(cuMemAlloc(&dw.p, (size_t)(N + 1) * 4));
    CK(cuMemAlloc(&dn.p, (size_t)4 * N * 4));
    CK(cuMemAlloc(&di.p, (size_t)N * 4));
    CK(cuMemAlloc(&de.p, (size_t)NW * 4));
    CK(cuMemAlloc(&dd.p, (size_t)NW * 4));
    CK(cuMemcpyHtoD(dl.p, lat, (size_t)N * NW));
    CK(cuMemsetD32(dh.p, 0, N + 1));
    CK(cuMemcpyHtoD(dw.p, w, (size_t)(N + 1) * 4));
    CK(cuMemcpyHtoD(dn.p, naver.data(), (size_t)4 * N * 4));
    CK(cuMemcpyHtoD(di.p, index.data(), (size_t)N * 4));
    unsigned blocks = NW / 256;
    if (compute_energies) {
        void *a1[] = {&dl.p, &de.p};
        CK(cuLaunchKernel(fe, blocks, 1, 1, 256, 1, 1, 0, 0, a1, 0));
        void *a2[] = {&dl.p, &dd.p};
        CK(cuLaunchKernel(fd, blocks, 1, 1, 256, 1, 1, 0, 0, a2, 0));
    } else {
        CK(cuMemcpyHtoD(de.p, energy, (size_t)NW * 4));
        CK(cuMemcpyHtoD(dd.p, deltaE, (size_t)NW * 4));
    }
    CK(cuCtxSynchronize());
    CUevent e0, e1;
    CK(cuEventCreate(&e0, 0));
    CK(cuEventCreate(&e1, 0));
    void *a[] = {&dl.p, &dh.p, &dw.p, &di.p, &dn.p, &de.p, &dd.p, &iter, &seed, &therm, &nup};
    CK(cuEventRecord(e0, 0));
    CK(cuLaunchKernel(fm, blocks, 1, 1, 256, 1, 1, 0, 0, a, 0));
    CK(cuEventRecord(e1, 0));
    CK(cuEventSynchronize(e1));
    float t = 0;
    CK(cuEventElapsedTime(&t, e0, e1));
    if (ms) *ms = t;
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    CK(cuMemcpyDtoH(lat, dl.p, (size_t)N * NW));
    CK(cuMemcpyDtoH(hist, dh.p, (size_t)(N + 1) * 4));
    CK(cuMemcpyDtoH(energy, de.p, (size_t)NW * 4));
    CK(cuMemcpyDtoH(deltaE, dd.p, (size_t)NW * 4));
    return 0;
}

/* One launch of the reference production kernel (FP64 weights, 2D
 * histogram u64 [(N+1)(N+2)/2], output of this launch only). */
int refgpu_produce_mcs(const char *cubin, unsigned L, unsigned NW, int8_t *lat, unsigned long long *hist2d,
                       const double *w, int *energy, int *deltaE, int *mag, unsigned iter, unsigned seed,
                       unsigned long long therm, unsigned long long nup, int compute_energies, float *ms)
{
    if (NW == 0 || NW % 256 != 0 || L < 2) { std::snprintf(g_err, sizeof g_err, "bad NW/L"); return -1; }
    if (int e = ensure_ctx()) return e;
    CUmodule m;
    if (int e = get_module(cubin, &m)) return e;
    if (int e = set_consts(m, L, NW)) return e;
    CUfunction fm, fe, fd, fM;
    CK(cuModuleGetFunction(&fm, m, "_Z3mcsPaPyPjS1_PdddPiS3_S3_jjyy"));
    CK(cuModuleGetFunction(&fe, m, "_Z13computeEnergyPaPi"));
    CK(cuModuleGetFunction(&fd, m, "_Z13computeDeltaEPaPi"));
    CK(cuModuleGetFunction(&fM, m, "_Z8computeMPaPi"));
    unsigned N = L * L;
    size_t hs = (size_t)(N + 1) * (N + 2) / 2;
    std::vector<unsigned> naver, index;
    tables(L, naver, index);
    DevBuf dl, dh, dw, dn, di, de, dd, dm;
    CK(cuMemAlloc(&dl.p, (size_t)N * NW));
    CK(cuMemAlloc(&dh.p, (hs + 1) * 8));
    CK(cuMemAlloc(&dw.p, (size_t)(N + 1) * 8));
    CK(cuMemAlloc(&dn.p, (size_t)4 * N * 4));
    CK(cuMemAlloc(&di.p, (size_t)N * 4));
    CK(cuMemAlloc(&de.p, (size_t)NW * 4));
    CK(cuMemAlloc(&dd.p, (size_t)NW * 4));
    CK(cuMemAlloc(&dm.p, (size_t)NW * 4));
    CK(cuMemcpyHtoD(dl.p, lat, (size_t)N * NW));
    CK(cuMemsetD32(dh.p, 0, (unsigned)((hs + 1) * 2)));
    CK(cuMemcpyHtoD(dw.p, w, (size_t)(N + 1) * 8));
    CK(cuMemcpyHtoD(dn.p, naver.data(), (size_t)4 * N * 4));
    CK(cuMemcpyHtoD(di.p, index.data(), (size_t)N * 4));
    unsigned blocks = NW / 256;
    if (compute_energies) {
        void *a1[] = {&dl.p, &de.p};
        CK(cuLaunchKernel(fe, blocks, 1, 1, 256, 1, 1, 0, 0, a1, 0));
        void *a2[] = {&dl.p, &dd.p};
        CK(cuLaunchKernel(fd, blocks, 1, 1, 256, 1, 1, 0, 0, a2, 0));
        void *a3[] = {&dl.p, &dm.p};
        CK(cuLaunchKernel(fM, blocks, 1, 1, 256, 1, 1, 0, 0, a3, 0));
    } else {
        CK(cuMemcpyHtoD(de.p, energy, (size_t)NW * 4));
        CK(cuMemcpyHtoD(dd.p, deltaE, (size_t)NW * 4));
        CK(cuMemcpyHtoD(dm.p, mag, (size_t)NW * 4));
    }
    CK(cuCtxSynchronize());
    double beta = 2.0, delta = 0.0;
    CUevent e0, e1;
    CK(cuEventCreate(&e0, 0));
    CK(cuEventCreate(&e1, 0));
    void *a[] = {&dl.p, &dh.p, &di.p, &dn.p, &dw.p, &beta, &delta, &de.p, &dd.p, &dm.p, &iter, &seed, &therm, &nup};
    CK(cuEventRecord(e0, 0));
    CK(cuLaunchKernel(fm, blocks, 1, 1, 256, 1, 1, 0, 0, a, 0));
    CK(cuEventRecord(e1, 0));
    CK(cuEventSynchronize(e1));
    float t = 0;
    CK(cuEventElapsedTime(&t, e0, e1));
    if (ms) *ms = t;
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    CK(cuMemcpyDtoH(lat, dl.p, (size_t)N * NW));
    CK(cuMemcpyDtoH(hist2d, dh.p, hs * 8));
    CK(cuMemcpyDtoH(energy, de.p, (size_t)NW * 4));
    CK(cuMemcpyDtoH(deltaE, dd.p, (size_t)NW * 4));
    CK(cuMemcpyDtoH(mag, dm.p, (size_t)NW * 4));
    return 0;
}
}
