// Launch interface of the adjoint kernels (adjoint.cu).
#pragma once

#include "fdtd_device.cuh"
#include "yee_kernels.h"

namespace fdtd {

// Adjoint fields (same layout as the fields) and the curl contributions exchanged between the two
// kernels of a reverse step: l = {Ex, Ey, Ez, Hx, Hy, Hz}; ge = G_E slots {Ex->Hz, Ex->Hy, Ey->Hx,
// Ey->Hz, Ez->Hy, Ez->Hx}; gh = G_H slots {Hx->Ey, Hx->Ez, Hy->Ez, Hy->Ex, Hz->Ex, Hz->Ey}.
struct AdjState {
    float* l[6];
    float* ge[6];
    float* gh[6];
};

// Per reverse step: the FoM source at the probe node and the design-gradient inputs (edge
// accumulators and the design-region E before / after the step; acc = NULL skips the gradient).
struct AdjStep {
    long long probe;
    float source;
    double* acc;
    const float* e_old;
    const float* e_new;
};

// One reverse step (k_adj_h then k_adj_e).
cudaError_t launch_adj_step(const StepParams& p, const AdjState& a, const PsiSet& psa, const AdjStep& st, cudaStream_t s);
// FoM sample of a forward step (Ez at node `probe` into *sample) and, if snap != NULL, the E
// components over the design edge box into snap (3 x box volume).
cudaError_t launch_after_step(const float* ex, const float* ey, const float* ez, const DeviceGrid& g, long long probe,
                              float* sample, const int dbox[6], float* snap, cudaStream_t s);
// The six field components over node box b (inside the grid) saved to / restored from buf
// (6 x box volume floats).
cudaError_t launch_box_state(const FieldPtrs& f, const DeviceGrid& g, const NodeBox& b, float* buf, bool save,
                             cudaStream_t s);
// grad (design cells, FP64) from the edge accumulators.
cudaError_t launch_grad_finalize(const double* acc, const int dbox[6], double* grad, cudaStream_t s);

}  // namespace fdtd
