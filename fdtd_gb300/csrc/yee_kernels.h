// Launch interface of the update kernels (host-visible declarations).
#pragma once

#include "fdtd_device.cuh"

namespace fdtd {

struct FieldPtrs {
    float *ex, *ey, *ez, *hx, *hy, *hz;
};

// Six CPML faces in the order x_n, x_p, y_n, y_p, z_n, z_p.
struct PsiSet {
    PsiFace f[6];
};

// One time step m with the two-pass schedule (E pass then H pass, in place).
cudaError_t launch_two_pass(const StepParams& p, const FieldPtrs& f, const PsiSet& ps, long long m,
                            cudaStream_t st);

// Setup kernels (setup_kernels.cu).
cudaError_t launch_cpml_profiles(const DeviceGrid& g, float pi, float* const prof[18], cudaStream_t st);
cudaError_t launch_material_tables(const DeviceGrid& g, const MatProps* props, int n, MatCoef* coef,
                                   cudaStream_t st);
cudaError_t launch_lumped_coefs(const DeviceGrid& g, const uint8_t* mat, const MatProps* props,
                                LumpedEdge* edges, const int* boxes, const float* resist, const int* owner,
                                int n_edges, cudaStream_t st);
cudaError_t launch_fill(float* p, long long n, float v, cudaStream_t st);
cudaError_t launch_paint(uint8_t* mat, const DeviceGrid& g, const int box[6], uint8_t value, cudaStream_t st);

}  // namespace fdtd
