// Launch interface of the batched persistent kernel (batch.cu).
#pragma once

#include "fdtd_device.cuh"
#include "yee_kernels.h"

namespace fdtd {

// One instance of a batch: its step parameters, field and CPML pointers (the handle's in-place
// two-pass buffers) and its current step, which the kernel advances.
struct __align__(16) BatchInstance {
    StepParams p;
    FieldPtrs f;
    PsiSet ps;
    long long step;
};
static_assert(sizeof(BatchInstance) % 16 == 0, "copied to shared memory in 16-byte words");

// CTA sizes with a kernel instantiation (128, 256, 512 threads).
bool batch_threads_supported(int threads);
// Clusters of `cluster` CTAs of `threads` threads that fit on the device at once.
cudaError_t batch_max_clusters(int cluster, int threads, int* out);
// Advance every instance by `steps` steps: the queue is reset, then one launch of n_clusters
// clusters takes the instances in `order` (indices into inst, longest first).
cudaError_t launch_batch(BatchInstance* inst, const int* order, int n_inst, int* queue, long long steps, int cluster,
                         int threads, int n_clusters, cudaStream_t st);

// Flat form: `steps` times an E kernel and an H kernel over `items` ({instance, x0, y0, k}, 32 x 8
// nodes of plane k of an instance), then the step counters of the instances advance by one.
cudaError_t launch_batch_flat(BatchInstance* inst, int n_inst, const int4* items, int n_items, long long steps,
                              cudaStream_t st);

// Add `by` to the step counter of every instance.
cudaError_t launch_batch_advance(BatchInstance* inst, int n_inst, int by, cudaStream_t st);

}  // namespace fdtd
