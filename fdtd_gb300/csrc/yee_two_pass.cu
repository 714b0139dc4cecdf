// Two-pass schedule: an E pass then an H pass per time step, both in place, one thread per node.
//
// This is the reference's own order of work (calc_e then calc_h, solver fdtdrav.h:3222-3333)
// expressed over the compact data layout. It runs at any grid size and is the schedule the fused
// sweep is checked against bit for bit; both call the same e_update / h_update.
#include "yee_common.cuh"
#include "yee_kernels.h"

namespace fdtd {

// One node's E (or H) update reading the fields `fi` and CPML memory `pin`, writing `fo` / `pout`
// (the same buffers for the in-place two-pass schedule). Every node loads its twelve field values
// and its class byte together (one round of memory latency); fast-path nodes (class != kGeneral)
// then update from the material table, the rest also gather the seven cell materials and take
// e_update / h_update. kDesign (k_design_e only): skip the class test and average the per-cell
// eps_r of design cells.
template <bool kDesign = false>
__device__ __forceinline__ void e_node_global(const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo,
                                              const PsiSet& pin, const PsiSet& pout, int i, int j, int k, long long m) {
    const DeviceGrid& g = p.g;
    const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
    const long long P = g.plane, R = g.pitch;
    ENbr nb;
    nb.ex = fi.ex[n]; nb.ey = fi.ey[n]; nb.ez = fi.ez[n];
    nb.hx = fi.hx[n]; nb.hy = fi.hy[n]; nb.hz = fi.hz[n];
    nb.hx_jm = j > 0 ? fi.hx[n - R] : 0.f;
    nb.hx_km = k > 0 ? fi.hx[n - P] : 0.f;
    nb.hy_im = i > 0 ? fi.hy[n - 1] : 0.f;
    nb.hy_km = k > 0 ? fi.hy[n - P] : 0.f;
    nb.hz_im = i > 0 ? fi.hz[n - 1] : 0.f;
    nb.hz_jm = j > 0 ? fi.hz[n - R] : 0.f;
    const int c = kDesign ? kGeneral : p.cls[n];
    float out[3], pre[3];
    if (c < kDesignNode) {
        e_update_interior(p, c, nb.ex, nb.ey, nb.ez, __fsub_rn(nb.hz, nb.hz_jm), __fsub_rn(nb.hy, nb.hy_km),
                          __fsub_rn(nb.hx, nb.hx_km), __fsub_rn(nb.hz, nb.hz_im), __fsub_rn(nb.hy, nb.hy_im),
                          __fsub_rn(nb.hx, nb.hx_jm), out);
        pre[0] = out[0]; pre[1] = out[1]; pre[2] = out[2];
    } else {
        const uint8_t* mat = p.mat;
        nb.m0 = mat[n];
        nb.mi = i > 0 ? mat[n - 1] : 0;
        nb.mj = j > 0 ? mat[n - R] : 0;
        nb.mk = k > 0 ? mat[n - P] : 0;
        nb.mij = (i > 0 && j > 0) ? mat[n - 1 - R] : 0;
        nb.mik = (i > 0 && k > 0) ? mat[n - 1 - P] : 0;
        nb.mjk = (j > 0 && k > 0) ? mat[n - R - P] : 0;
        const PsiIO io{pin.f, pout.f, true};
        const bool plane_lumped = p.lumped_k[k] < p.lumped_k[k + 1];
        e_update<kDesign>(p, nb, i, j, k, m, plane_lumped, io, out, pre);
    }
    if (!kDesign && c == kDesignNode) return;  // k_design_e writes the design region's E
    fo.ex[n] = out[0]; fo.ey[n] = out[1]; fo.ez[n] = out[2];
    if (p.probe_k[k] < p.probe_k[k + 1]) {
        const long long row = m % p.ring_cap;
        for (int q = 0; q < 3; ++q) sample(p, row, q, i, j, k, pre[q]);
    }
}

// H reads the old H from `fi` and the new E from `fe`.
__device__ __forceinline__ void h_node_global(const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fe,
                                              const FieldPtrs& fo, const PsiSet& pin, const PsiSet& pout, int i, int j,
                                              int k, long long m) {
    const DeviceGrid& g = p.g;
    const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
    const long long P = g.plane, R = g.pitch;
    HNbr nb;
    nb.hx = fi.hx[n]; nb.hy = fi.hy[n]; nb.hz = fi.hz[n];
    nb.ex = fe.ex[n]; nb.ey = fe.ey[n]; nb.ez = fe.ez[n];
    nb.ey_kp = k < g.nz - 1 ? fe.ey[n + P] : 0.f;
    nb.ez_jp = j < g.ny - 1 ? fe.ez[n + R] : 0.f;
    nb.ez_ip = i < g.nx - 1 ? fe.ez[n + 1] : 0.f;
    nb.ex_kp = k < g.nz - 1 ? fe.ex[n + P] : 0.f;
    nb.ex_jp = j < g.ny - 1 ? fe.ex[n + R] : 0.f;
    nb.ey_ip = i < g.nx - 1 ? fe.ey[n + 1] : 0.f;
    const int c = p.cls[n];
    float out[3], pre[3];
    if (c < kDesignNode) {
        h_update_interior(p, c, nb.hx, nb.hy, nb.hz, __fsub_rn(nb.ey_kp, nb.ey), __fsub_rn(nb.ez_jp, nb.ez),
                          __fsub_rn(nb.ez_ip, nb.ez), __fsub_rn(nb.ex_kp, nb.ex), __fsub_rn(nb.ex_jp, nb.ex),
                          __fsub_rn(nb.ey_ip, nb.ey), out);
        pre[0] = out[0]; pre[1] = out[1]; pre[2] = out[2];
    } else {
        const uint8_t* mat = p.mat;
        nb.m0 = mat[n];
        nb.mi = i > 0 ? mat[n - 1] : 0;
        nb.mj = j > 0 ? mat[n - R] : 0;
        nb.mk = k > 0 ? mat[n - P] : 0;
        const PsiIO io{pin.f, pout.f, true};
        h_update(p, nb, i, j, k, io, out, pre);
    }
    fo.hx[n] = out[0]; fo.hy[n] = out[1]; fo.hz[n] = out[2];
    if (p.probe_k[k] < p.probe_k[k + 1]) {
        const long long row = m % p.ring_cap;
        for (int q = 0; q < 3; ++q) sample(p, row, 3 + q, i, j, k, pre[q]);
    }
}

__global__ void __launch_bounds__(256) k_update_e(const __grid_constant__ StepParams p, FieldPtrs f,
                                                  const __grid_constant__ PsiSet ps, long long m) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    if (i >= p.g.nx || j >= p.g.ny) return;
    e_node_global(p, f, f, ps, ps, i, j, blockIdx.z, m);
}

__global__ void __launch_bounds__(256) k_update_h(const __grid_constant__ StepParams p, FieldPtrs f,
                                                  const __grid_constant__ PsiSet ps, long long m) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    if (i >= p.g.nx || j >= p.g.ny) return;
    h_node_global(p, f, f, f, ps, ps, i, j, blockIdx.z, m);
}

// Shell passes of the fused schedule: the nodes of the general items (int4 {x0, y0, k0, k1}, a
// 32 x tile_h tile and a plane range; x0, y0 may be negative) read buffer A (`fi`, `pin`) and
// write buffer B (`fo`, `pout`). The E pass runs before the interior sweep, the H pass after it,
// since H reads new E at interior nodes next to the shell.
__global__ void __launch_bounds__(256) k_shell_e(const __grid_constant__ StepParams p, FieldPtrs fi, FieldPtrs fo,
                                                 const __grid_constant__ PsiSet pin, const __grid_constant__ PsiSet pout,
                                                 const int4* __restrict__ items, int tile_h, long long m) {
    const int4 it = items[blockIdx.x];
    const int i = it.x + (int)threadIdx.x;
    if (i < 0 || i >= p.g.nx) return;
    for (int r = threadIdx.y; r < tile_h; r += 8) {
        const int j = it.y + r;
        if (j < 0 || j >= p.g.ny) continue;
        for (int k = it.z; k < it.w; ++k) e_node_global(p, fi, fo, pin, pout, i, j, k, m);
    }
}

__global__ void __launch_bounds__(256) k_shell_h(const __grid_constant__ StepParams p, FieldPtrs fi, FieldPtrs fo,
                                                 const __grid_constant__ PsiSet pin, const __grid_constant__ PsiSet pout,
                                                 const int4* __restrict__ items, int tile_h, long long m) {
    const int4 it = items[blockIdx.x];
    const int i = it.x + (int)threadIdx.x;
    if (i < 0 || i >= p.g.nx) return;
    for (int r = threadIdx.y; r < tile_h; r += 8) {
        const int j = it.y + r;
        if (j < 0 || j >= p.g.ny) continue;
        for (int k = it.z; k < it.w; ++k) h_node_global(p, fi, fo, fo, pin, pout, i, j, k, m);
    }
}

cudaError_t launch_shell(bool e_pass, const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo, const PsiSet& pin,
                         const PsiSet& pout, const int4* items, int n_items, int tile_h, long long m, cudaStream_t st) {
    if (n_items <= 0) return cudaSuccess;
    if (e_pass) k_shell_e<<<n_items, dim3(32, 8, 1), 0, st>>>(p, fi, fo, pin, pout, items, tile_h, m);
    else k_shell_h<<<n_items, dim3(32, 8, 1), 0, st>>>(p, fi, fo, pin, pout, items, tile_h, m);
    return cudaGetLastError();
}

// E of the nodes of the design region's edge box [d0, d3] x [d1, d4] x [d2, d5] (node class
// kDesignNode, which the other E kernels do not store), with the per-cell eps_r of the design
// cells. Design nodes are interior: no CPML memory, no lumped edge.
__global__ void __launch_bounds__(256) k_design_e(const __grid_constant__ StepParams p, FieldPtrs fi, FieldPtrs fo,
                                                  const __grid_constant__ PsiSet pin,
                                                  const __grid_constant__ PsiSet pout, long long m) {
    const int* d = p.dbox;
    const int i = d[0] + blockIdx.x * 32 + threadIdx.x;
    const int j = d[1] + blockIdx.y * 8 + threadIdx.y;
    const int k = d[2] + blockIdx.z;
    if (i > d[3] || j > d[4]) return;
    e_node_global<true>(p, fi, fo, pin, pout, i, j, k, m);
}

cudaError_t launch_design_e(const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo, const PsiSet& pin,
                            const PsiSet& pout, long long m, cudaStream_t st) {
    if (!p.deps) return cudaSuccess;
    const int* d = p.dbox;
    const dim3 grid((d[3] - d[0] + 32) / 32, (d[4] - d[1] + 8) / 8, d[5] - d[2] + 1);
    k_design_e<<<grid, dim3(32, 8, 1), 0, st>>>(p, fi, fo, pin, pout, m);
    return cudaGetLastError();
}

cudaError_t launch_two_pass(const StepParams& p, const FieldPtrs& f, const PsiSet& ps, long long m,
                            cudaStream_t st) {
    dim3 block(32, 8, 1);
    dim3 grid((p.g.nx + 31) / 32, (p.g.ny + 7) / 8, p.g.nz);
    k_update_e<<<grid, block, 0, st>>>(p, f, ps, m);
    cudaError_t e = launch_design_e(p, f, f, ps, ps, m, st);
    if (e != cudaSuccess) return e;
    k_update_h<<<grid, block, 0, st>>>(p, f, ps, m);
    return cudaGetLastError();
}

}  // namespace fdtd
