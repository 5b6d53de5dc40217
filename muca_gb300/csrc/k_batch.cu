// k_batch.cu -- kernels of a batch of independent weight-estimation runs.
//
// Many (L, beta) instances of uneven size advance one weight iteration
// together: a prep kernel clears the histograms of the instances still
// running, one persistent sweep kernel works through the list of chain
// blocks of all instances, and one update block per instance applies the
// statistics, the schedule and the weight update (k_weights.cu).  The three
// launches of an iteration are captured into a CUDA graph by the host
// (muca_batch.cu) and replayed.
//
// The sweep of a chain block is the single-simulation windowed sweep
// (sweep_core.cuh) with two differences: the Metropolis term -beta*dE comes
// from the instance's table (exactly -2 dE for the reference's beta = 2), and
// the histogram may go straight to the u64 device histogram, which frees the
// shared memory of the u32 bins for more blocks per SM.  Work is fetched by
// an atomic counter over items sorted by decreasing cost, so the large
// lattices start first and the small ones fill the tail.
#include "sweep_core.cuh"

namespace muca {

__global__ void k_batch_prep(const BatchInst *__restrict__ insts, uint32_t *__restrict__ next_item,
                             uint32_t *__restrict__ running)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *next_item = 0u;
        *running = 0u;
    }
    const BatchInst &I = insts[blockIdx.x];
    if (I.ctl->st.stop) return;
    const uint32_t n = I.a.N + 1;
    unsigned long long *h = I.a.hist;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) h[i] = 0ull;
}

template <int R, int LAT, bool HS>
__global__ void __launch_bounds__(256, 1) k_batch_sweep(const BatchInst *__restrict__ insts,
                                                         const BatchItem *__restrict__ items, uint32_t n_items,
                                                         uint32_t *__restrict__ next_item, uint32_t cpb,
                                                         uint32_t smem_bytes)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t s_item;
    __shared__ float s_btab[17];
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(next_item, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if (it >= n_items) return;  // uniform: every thread read the same item
        const BatchItem item = items[it];
        const BatchInst *I = insts + item.inst;
        const SweepArgs a = I->a;
        uint32_t iter;
        unsigned long long nup;
        if (launch_params(a, iter, nup)) {  // the instance is still running
            if (threadIdx.x < 17) s_btab[threadIdx.x] = I->btab[threadIdx.x];
            // s_btab is read only after the block barrier inside the sweep's prologue
            if (LAT == kLatShared) {
                win_sweep_block<kModeWeight, R, true, HS, true>(a, smem, cpb, item.blk, iter, nup, s_btab);
            } else {
                // uniform per item: the lattice joins the weights (and bins) in
                // shared memory when all fit in the launch's allocation
                // (kLatWhereFits); otherwise it stays in global memory, behind
                // a four-row ring per lane where that fits
                const size_t base = smem_weights_bytes(kModeWeight, a.N) + (HS ? smem_hist_bytes(kModeWeight, a.N) : 0);
                if (LAT == kLatWhereFits && base + (size_t)a.L * a.WPR * 4u * cpb <= smem_bytes)
                    win_sweep_block<kModeWeight, R, true, HS, true>(a, smem, cpb, item.blk, iter, nup, s_btab);
                else if (a.L % 4 == 0 && a.WPR <= 8 && base + ring_bytes(a.L, cpb) <= smem_bytes)
                    win_sweep_block<kModeWeight, R, false, HS, true, true>(a, smem, cpb, item.blk, iter, nup, s_btab);
                else
                    win_sweep_block<kModeWeight, R, false, HS, true>(a, smem, cpb, item.blk, iter, nup, s_btab);
            }
        }
        __syncthreads();
    }
}

cudaError_t launch_batch_prep(const BatchInst *insts, uint32_t n_inst, uint32_t *next_item, uint32_t *running,
                              cudaStream_t s)
{
    k_batch_prep<<<n_inst, 256, 0, s>>>(insts, next_item, running);
    return cudaGetLastError();
}

size_t batch_sweep_smem(uint32_t L, uint32_t cpb, bool lat_smem, bool hist_smem, bool row_ring)
{
    const uint32_t N = L * L, WPR = (L + 15) / 16;
    return smem_weights_bytes(kModeWeight, N) + (hist_smem ? smem_hist_bytes(kModeWeight, N) : 0) +
           (lat_smem ? (size_t)L * WPR * 4 * cpb : (row_ring ? ring_bytes(L, cpb) : 0));
}

using BatchKernel = void (*)(const BatchInst *, const BatchItem *, uint32_t, uint32_t *, uint32_t, uint32_t);

template <int R, int LAT>
static BatchKernel batch_kernel_lat(bool hist_smem)
{
    return hist_smem ? k_batch_sweep<R, LAT, true> : k_batch_sweep<R, LAT, false>;
}

template <int R>
static BatchKernel batch_kernel_r(uint32_t lat, bool hist_smem)
{
    return lat == kLatWhereFits ? batch_kernel_lat<R, kLatWhereFits>(hist_smem)
         : lat == kLatShared    ? batch_kernel_lat<R, kLatShared>(hist_smem)
                                : batch_kernel_lat<R, kLatGlobal>(hist_smem);
}

static BatchKernel batch_kernel(int rounds, uint32_t lat, bool hist_smem)
{
    return rounds == 10 ? batch_kernel_r<10>(lat, hist_smem) : batch_kernel_r<7>(lat, hist_smem);
}

cudaError_t batch_sweep_occupancy(uint32_t cpb, int rounds, uint32_t lat, bool hist_smem, size_t smem, int *blocks)
{
    if (lat > kLatWhereFits) return cudaErrorInvalidValue;
    const BatchKernel k = batch_kernel(rounds, lat, hist_smem);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k, (int)((cpb + 31u) / 32u * 32u), smem);
}

cudaError_t launch_batch_sweep(const BatchInst *insts, const BatchItem *items, uint32_t n_items, uint32_t *next_item,
                               uint32_t cpb, int rounds, uint32_t lat, bool hist_smem, uint32_t grid, size_t smem,
                               cudaStream_t s)
{
    // the shared-memory attribute was set by batch_sweep_occupancy for this shape
    if (cpb == 0 || cpb > 256 || lat > kLatWhereFits) return cudaErrorInvalidValue;
    const BatchKernel k = batch_kernel(rounds, lat, hist_smem);
    k<<<grid, (cpb + 31u) / 32u * 32u, smem, s>>>(insts, items, n_items, next_item, cpb, (uint32_t)smem);
    return cudaGetLastError();
}

}  // namespace muca
