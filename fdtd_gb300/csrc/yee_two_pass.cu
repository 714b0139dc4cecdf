// Two-pass schedule: an E pass then an H pass per time step, both in place, one thread per node.
//
// This is the reference's own order of work (calc_e then calc_h, solver fdtdrav.h:3222-3333)
// expressed over the compact data layout. It runs at any grid size and is the schedule the fused
// sweep is checked against bit for bit; both call the same e_update / h_update.
#include "yee_common.cuh"
#include "yee_kernels.h"

namespace fdtd {

__global__ void __launch_bounds__(256) k_update_e(const __grid_constant__ StepParams p, FieldPtrs f,
                                                  const __grid_constant__ PsiSet ps, long long m) {
    const DeviceGrid& g = p.g;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.nx || j >= g.ny) return;
    const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
    const long long P = g.plane, R = g.pitch;
    const uint8_t* mat = p.mat;
    ENbr nb;
    nb.ex = f.ex[n]; nb.ey = f.ey[n]; nb.ez = f.ez[n];
    nb.hx = f.hx[n]; nb.hy = f.hy[n]; nb.hz = f.hz[n];
    nb.hx_jm = j > 0 ? f.hx[n - R] : 0.f;
    nb.hx_km = k > 0 ? f.hx[n - P] : 0.f;
    nb.hy_im = i > 0 ? f.hy[n - 1] : 0.f;
    nb.hy_km = k > 0 ? f.hy[n - P] : 0.f;
    nb.hz_im = i > 0 ? f.hz[n - 1] : 0.f;
    nb.hz_jm = j > 0 ? f.hz[n - R] : 0.f;
    nb.m0 = mat[n];
    nb.mi = i > 0 ? mat[n - 1] : 0;
    nb.mj = j > 0 ? mat[n - R] : 0;
    nb.mk = k > 0 ? mat[n - P] : 0;
    nb.mij = (i > 0 && j > 0) ? mat[n - 1 - R] : 0;
    nb.mik = (i > 0 && k > 0) ? mat[n - 1 - P] : 0;
    nb.mjk = (j > 0 && k > 0) ? mat[n - R - P] : 0;
    float out[3], pre[3];
    const PsiIO io{ps.f, ps.f, true};
    const bool plane_lumped = p.lumped_k[k] < p.lumped_k[k + 1];
    if (!plane_lumped && interior(i, g.nx, g.pxn, g.pxp) && interior(j, g.ny, g.pyn, g.pyp) &&
        interior(k, g.nz, g.pzn, g.pzp) && e_uniform(nb)) {
        e_update_interior(p, nb, out);
        pre[0] = out[0]; pre[1] = out[1]; pre[2] = out[2];
    } else {
        e_update(p, nb, i, j, k, m, plane_lumped, io, out, pre);
    }
    f.ex[n] = out[0]; f.ey[n] = out[1]; f.ez[n] = out[2];
    if (p.probe_k[k] < p.probe_k[k + 1]) {
        const long long row = m % p.ring_cap;
        for (int c = 0; c < 3; ++c) sample(p, row, c, i, j, k, pre[c]);
    }
}

__global__ void __launch_bounds__(256) k_update_h(const __grid_constant__ StepParams p, FieldPtrs f,
                                                  const __grid_constant__ PsiSet ps, long long m) {
    const DeviceGrid& g = p.g;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.nx || j >= g.ny) return;
    const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
    const long long P = g.plane, R = g.pitch;
    const uint8_t* mat = p.mat;
    HNbr nb;
    nb.hx = f.hx[n]; nb.hy = f.hy[n]; nb.hz = f.hz[n];
    nb.ex = f.ex[n]; nb.ey = f.ey[n]; nb.ez = f.ez[n];
    nb.ey_kp = k < g.nz - 1 ? f.ey[n + P] : 0.f;
    nb.ez_jp = j < g.ny - 1 ? f.ez[n + R] : 0.f;
    nb.ez_ip = i < g.nx - 1 ? f.ez[n + 1] : 0.f;
    nb.ex_kp = k < g.nz - 1 ? f.ex[n + P] : 0.f;
    nb.ex_jp = j < g.ny - 1 ? f.ex[n + R] : 0.f;
    nb.ey_ip = i < g.nx - 1 ? f.ey[n + 1] : 0.f;
    nb.m0 = mat[n];
    nb.mi = i > 0 ? mat[n - 1] : 0;
    nb.mj = j > 0 ? mat[n - R] : 0;
    nb.mk = k > 0 ? mat[n - P] : 0;
    float out[3], pre[3];
    const PsiIO io{ps.f, ps.f, true};
    if (interior(i, g.nx, g.pxn, g.pxp) && interior(j, g.ny, g.pyn, g.pyp) && interior(k, g.nz, g.pzn, g.pzp) &&
        h_uniform(nb)) {
        h_update_interior(p, nb, out);
        pre[0] = out[0]; pre[1] = out[1]; pre[2] = out[2];
    } else {
        h_update(p, nb, i, j, k, io, out, pre);
    }
    f.hx[n] = out[0]; f.hy[n] = out[1]; f.hz[n] = out[2];
    if (p.probe_k[k] < p.probe_k[k + 1]) {
        const long long row = m % p.ring_cap;
        for (int c = 0; c < 3; ++c) sample(p, row, 3 + c, i, j, k, pre[c]);
    }
}

cudaError_t launch_two_pass(const StepParams& p, const FieldPtrs& f, const PsiSet& ps, long long m,
                            cudaStream_t st) {
    dim3 block(32, 8, 1);
    dim3 grid((p.g.nx + 31) / 32, (p.g.ny + 7) / 8, p.g.nz);
    k_update_e<<<grid, block, 0, st>>>(p, f, ps, m);
    k_update_h<<<grid, block, 0, st>>>(p, f, ps, m);
    return cudaGetLastError();
}

}  // namespace fdtd
