// Batched persistent launch: many independent simulations (uneven grid sizes) advanced by one
// kernel launch (no reference counterpart; the reference runs one domain per process).
//
// Each instance is owned, for all of its steps, by one thread-block cluster. Clusters take
// instances from a queue (longest first; an atomic counter, nothing waits on it) and run the
// two-pass schedule on them: the E update of every node, a hardware cluster barrier, the H update
// of every node, a cluster barrier, and so on. Instances never depend on each other, so there is
// no grid-wide synchronisation; the cluster barrier is the only wait, and the CTAs of a cluster
// are co-scheduled by construction. The per-node updates are those of the two-pass schedule
// (node_global.cuh), so every instance produces the bits it would produce alone. Inside an
// instance, warp w of the cluster takes x-rows w, w + W, ... of the (ny * nz) rows and its lanes
// cover a row 32 nodes at a time (coalesced).
#include <cooperative_groups.h>

#include "batch.h"
#include "node_global.cuh"

namespace cg = cooperative_groups;

namespace fdtd {

template <int THREADS, int MIN_BLOCKS>
__global__ void __launch_bounds__(THREADS, MIN_BLOCKS)
k_batch(BatchInstance* __restrict__ inst, const int* __restrict__ order, int n_inst, int* __restrict__ queue,
        long long steps) {
    cg::cluster_group cluster = cg::this_cluster();
    __shared__ int s_next;
    // The instance's descriptor in shared memory: the node updates read it constantly, and shared
    // memory cannot alias the global field stores, so the compiler need not reload it after them.
    __shared__ __align__(16) BatchInstance s_inst;
    const int rank = (int)cluster.block_rank();
    const int nblk = (int)cluster.num_blocks();
    constexpr int warps_per_cta = THREADS / 32;
    const int warp = rank * warps_per_cta + (int)threadIdx.x / 32, lane = threadIdx.x % 32;
    const int n_warps = nblk * warps_per_cta;
    for (;;) {
        if (rank == 0 && threadIdx.x == 0) s_next = atomicAdd(queue, 1);
        cluster.sync();
        const int q = *cluster.map_shared_rank(&s_next, 0);
        cluster.sync();  // every CTA has read the slot before rank 0 writes the next one
        if (q >= n_inst) return;
        BatchInstance* gI = inst + order[q];
        {
            const int4* src = reinterpret_cast<const int4*>(gI);
            int4* dst = reinterpret_cast<int4*>(&s_inst);
            for (int w = threadIdx.x; w < (int)(sizeof(BatchInstance) / sizeof(int4)); w += THREADS) dst[w] = src[w];
        }
        __syncthreads();
        const BatchInstance& I = s_inst;
        const StepParams& p = I.p;
        const int nx = p.g.nx, ny = p.g.ny, rows = p.g.ny * p.g.nz;
        const long long m0 = I.step;
        for (long long s = 0; s < steps; ++s) {
            const long long m = m0 + s;
            for (int r = warp; r < rows; r += n_warps) {
                const int j = r % ny, k = r / ny;
                for (int i = lane; i < nx; i += 32) e_node_global<false, true>(p, I.f, I.f, I.ps, I.ps, i, j, k, m);
            }
            cluster.sync();
            for (int r = warp; r < rows; r += n_warps) {
                const int j = r % ny, k = r / ny;
                for (int i = lane; i < nx; i += 32) h_node_global<true>(p, I.f, I.f, I.f, I.ps, I.ps, i, j, k, m);
            }
            cluster.sync();
        }
        if (rank == 0 && threadIdx.x == 0) gI->step = m0 + steps;
    }
}

// Flat form: per step one E kernel and one H kernel over the tiles of every instance (item
// {instance, x0, y0, k}: a 32 x 8 block of plane k), then the step counters advance. Every CTA
// copies its instance's descriptor to shared memory first. The GPU is filled by all instances
// at once with one node per thread, as in the two-pass schedule, instead of a cluster marching
// through one instance; the per-node updates are the same, so the bits are too.
// 6 CTAs of 256 per SM (40 registers), as the two-pass kernels
#ifndef FDTD_BATCH_FLAT_MIN_BLOCKS
#define FDTD_BATCH_FLAT_MIN_BLOCKS 6
#endif
__global__ void __launch_bounds__(256, FDTD_BATCH_FLAT_MIN_BLOCKS) k_batch_flat_e(const BatchInstance* __restrict__ inst,
                                                      const int4* __restrict__ items) {
    __shared__ __align__(16) BatchInstance s;
    const int4 it = items[blockIdx.x];
    {
        const int4* src = reinterpret_cast<const int4*>(inst + it.x);
        int4* dst = reinterpret_cast<int4*>(&s);
        const int t = threadIdx.y * 32 + threadIdx.x;
        for (int w = t; w < (int)(sizeof(BatchInstance) / sizeof(int4)); w += 256) dst[w] = src[w];
    }
    __syncthreads();
    const int i = it.y + (int)threadIdx.x, j = it.z + (int)threadIdx.y;
    // instances are small enough for 32-bit node offsets (checked when the batch is created)
    if (i < s.p.g.nx && j < s.p.g.ny) e_node_global<false, false, false, uint32_t>(s.p, s.f, s.f, s.ps, s.ps, i, j, it.w, s.step);
}

__global__ void __launch_bounds__(256, FDTD_BATCH_FLAT_MIN_BLOCKS) k_batch_flat_h(const BatchInstance* __restrict__ inst,
                                                      const int4* __restrict__ items) {
    __shared__ __align__(16) BatchInstance s;
    const int4 it = items[blockIdx.x];
    {
        const int4* src = reinterpret_cast<const int4*>(inst + it.x);
        int4* dst = reinterpret_cast<int4*>(&s);
        const int t = threadIdx.y * 32 + threadIdx.x;
        for (int w = t; w < (int)(sizeof(BatchInstance) / sizeof(int4)); w += 256) dst[w] = src[w];
    }
    __syncthreads();
    const int i = it.y + (int)threadIdx.x, j = it.z + (int)threadIdx.y;
    if (i < s.p.g.nx && j < s.p.g.ny) h_node_global<false, uint32_t>(s.p, s.f, s.f, s.f, s.ps, s.ps, i, j, it.w, s.step);
}

__global__ void k_batch_advance(BatchInstance* inst, int n, int by) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) inst[q].step += by;
}

cudaError_t launch_batch_advance(BatchInstance* inst, int n_inst, int by, cudaStream_t st) {
    k_batch_advance<<<(n_inst + 127) / 128, 128, 0, st>>>(inst, n_inst, by);
    return cudaGetLastError();
}

cudaError_t launch_batch_flat(BatchInstance* inst, int n_inst, const int4* items, int n_items, long long steps,
                              cudaStream_t st) {
    for (long long s = 0; s < steps; ++s) {
        k_batch_flat_e<<<n_items, dim3(32, 8, 1), 0, st>>>(inst, items);
        k_batch_flat_h<<<n_items, dim3(32, 8, 1), 0, st>>>(inst, items);
        k_batch_advance<<<(n_inst + 127) / 128, 128, 0, st>>>(inst, n_inst, 1);
    }
    return cudaGetLastError();
}

// CTA sizes the autotuner may pick, with register budgets that keep several CTAs per SM.
using BatchKernel = void (*)(BatchInstance*, const int*, int, int*, long long);
static BatchKernel kernel_for(int threads) {
    if (threads == 128) return k_batch<128, 6>;
    if (threads == 256) return k_batch<256, 3>;
    return k_batch<512, 1>;
}

bool batch_threads_supported(int threads) { return threads == 128 || threads == 256 || threads == 512; }

static cudaLaunchConfig_t batch_config(int cluster, int threads, int n_clusters, cudaStream_t st,
                                       cudaLaunchAttribute* attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cluster * n_clusters, 1, 1);
    cfg.blockDim = dim3(threads, 1, 1);
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

cudaError_t batch_max_clusters(int cluster, int threads, int* out) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = batch_config(cluster, threads, 1, nullptr, attr);
    return cudaOccupancyMaxActiveClusters(out, kernel_for(threads), &cfg);
}

cudaError_t launch_batch(BatchInstance* inst, const int* order, int n_inst, int* queue, long long steps, int cluster,
                         int threads, int n_clusters, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = batch_config(cluster, threads, n_clusters, st, attr);
    return cudaLaunchKernelEx(&cfg, kernel_for(threads), inst, order, n_inst, queue, steps);
}

}  // namespace fdtd
