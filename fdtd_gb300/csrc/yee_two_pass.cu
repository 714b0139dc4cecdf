// Two-pass schedule: an E pass then an H pass per time step, both in place, one thread per node.
//
// This is the reference's own order of work (calc_e then calc_h, solver fdtdrav.h:3222-3333)
// expressed over the compact data layout. It runs at any grid size and is the schedule the fused
// sweep is checked against bit for bit; both call the same e_update / h_update.
#include "node_global.cuh"

namespace fdtd {

// CTAs of 256 per SM the one-node-per-thread kernels are compiled for: 6 caps them at 40 registers
// (48 warps resident; the general path spills a few words), which measured 4-7 % faster at 512^3
// than the compiler's own choice of 48 registers (5 CTAs).
#ifndef FDTD_TWO_PASS_MIN_BLOCKS
#define FDTD_TWO_PASS_MIN_BLOCKS 6
#endif
#ifndef FDTD_SHELL_MIN_BLOCKS
#define FDTD_SHELL_MIN_BLOCKS 6
#endif
// The shell E pass loads a CPML node's old psi together with its fields (e_node_global's kEarly):
// measured at 512^3, the fused step 2.2 % faster (256^3: 3.3 %). The shell H pass gains nothing
// from it, and the two-pass kernels, whose spills it raises, lose 7-9 % at 64^3 and 128^3.
#ifndef FDTD_SHELL_EARLY_E
#define FDTD_SHELL_EARLY_E 1
#endif
#ifndef FDTD_SHELL_EARLY_H
#define FDTD_SHELL_EARLY_H 0
#endif
template <typename Idx>
__global__ void __launch_bounds__(256, FDTD_TWO_PASS_MIN_BLOCKS) k_update_e(const __grid_constant__ StepParams p, FieldPtrs f,
                                                  const __grid_constant__ PsiSet ps, long long m) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    if (i >= p.g.nx || j >= p.g.ny) return;
    e_node_global<false, false, false, Idx>(p, f, f, ps, ps, i, j, blockIdx.z, m);
}

template <typename Idx>
__global__ void __launch_bounds__(256, FDTD_TWO_PASS_MIN_BLOCKS) k_update_h(const __grid_constant__ StepParams p, FieldPtrs f,
                                                  const __grid_constant__ PsiSet ps, long long m) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    if (i >= p.g.nx || j >= p.g.ny) return;
    h_node_global<false, Idx>(p, f, f, f, ps, ps, i, j, blockIdx.z, m);
}

// Shell passes of the fused schedule: the nodes of the shell items (int4 {x0, y0, k, code}: a
// block of shape s = code & 15 (widths 32, 16, 64, 128, 256, 8, 4, 2, 1; 256 nodes) of which the
// first (code >> 4) & 511 columns and (code >> 13) & 511 rows are the item's, in planes k ..
// k + ((code >> 22) & 15)) read buffer A (`fi`,
// `pin`) and write buffer B (`fo`, `pout`), one node per thread as in the two-pass kernels. The E
// pass runs before the interior sweep, the H pass after it, since H reads new E at interior nodes
// next to the shell.
__device__ __forceinline__ bool shell_node(const int4& it, const DeviceGrid& g, int& i, int& j) {
    const int s = it.w & 15;
    const int lw = s == 0 ? 5 : s == 1 ? 4 : s <= 4 ? s + 4 : 8 - s;  // log2 of the block width
    const int t = (int)(threadIdx.y * 32 + threadIdx.x);
    const int tx = t & ((1 << lw) - 1), ty = t >> lw;
    i = it.x + tx;
    j = it.y + ty;
    return tx < ((it.w >> 4) & 511) && ty < ((it.w >> 13) & 511) && i < g.nx && j < g.ny;
}

// One launch per pass covers the four shell lists (yee_kernels.h), which lie one after the other
// in device memory: a block takes the instantiation of its list, kSlabs = the CPML slabs (bit 0 x,
// 1 y, 2 z) its nodes may lie in, so the other slab tests compile out of that list's code. One
// launch, not one per list, since small grids are bound by the chain of launches.
template <typename Idx, int kSlabs>
__device__ __forceinline__ void shell_e_item(const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo,
                                             const PsiSet& pin, const PsiSet& pout, const int4& it, long long m) {
    int i, j;
    if (!shell_node(it, p.g, i, j)) return;
    for (int k = it.z, k1 = it.z + ((it.w >> 22) & 15); k <= k1; ++k)
        e_node_global<false, false, false, Idx, kSlabs, FDTD_SHELL_EARLY_E != 0>(p, fi, fo, pin, pout, i, j, k, m);
}
template <typename Idx, int kSlabs>
__device__ __forceinline__ void shell_h_item(const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo,
                                             const PsiSet& pin, const PsiSet& pout, const int4& it, long long m) {
    int i, j;
    if (!shell_node(it, p.g, i, j)) return;
    for (int k = it.z, k1 = it.z + ((it.w >> 22) & 15); k <= k1; ++k)
        h_node_global<false, Idx, kSlabs, FDTD_SHELL_EARLY_H != 0>(p, fi, fo, fo, pin, pout, i, j, k, m);
}

// e1, e2, e3: the ends of the first three lists in the launch (blocks from e3 on take the fourth).
template <typename Idx>
__global__ void __launch_bounds__(256, FDTD_SHELL_MIN_BLOCKS) k_shell_e(const __grid_constant__ StepParams p, FieldPtrs fi, FieldPtrs fo,
                                                 const __grid_constant__ PsiSet pin, const __grid_constant__ PsiSet pout,
                                                 const int4* __restrict__ items, int e1, int e2, int e3, long long m) {
    const int b = blockIdx.x;
    const int4 it = items[b];
    if (b < e1) shell_e_item<Idx, 4>(p, fi, fo, pin, pout, it, m);
    else if (b < e2) shell_e_item<Idx, 6>(p, fi, fo, pin, pout, it, m);
    else if (b < e3) shell_e_item<Idx, 1>(p, fi, fo, pin, pout, it, m);
    else shell_e_item<Idx, 7>(p, fi, fo, pin, pout, it, m);
}

template <typename Idx>
__global__ void __launch_bounds__(256, FDTD_SHELL_MIN_BLOCKS) k_shell_h(const __grid_constant__ StepParams p, FieldPtrs fi, FieldPtrs fo,
                                                 const __grid_constant__ PsiSet pin, const __grid_constant__ PsiSet pout,
                                                 const int4* __restrict__ items, int e1, int e2, int e3, long long m) {
    const int b = blockIdx.x;
    const int4 it = items[b];
    if (b < e1) shell_h_item<Idx, 4>(p, fi, fo, pin, pout, it, m);
    else if (b < e2) shell_h_item<Idx, 6>(p, fi, fo, pin, pout, it, m);
    else if (b < e3) shell_h_item<Idx, 1>(p, fi, fo, pin, pout, it, m);
    else shell_h_item<Idx, 7>(p, fi, fo, pin, pout, it, m);
}

cudaError_t launch_shell(bool e_pass, const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo, const PsiSet& pin,
                         const PsiSet& pout, const ShellWork& w, long long m, cudaStream_t st) {
    int n = 0;
    for (int q = 0; q < kShellLists; ++q) {
        if (q > 0 && w.items[q] != w.items[q - 1] + w.n[q - 1]) return cudaErrorInvalidValue;  // the lists must be contiguous
        n += w.n[q];
    }
    if (n <= 0) return cudaSuccess;
    const dim3 b(32, 8, 1);
    const int e1 = w.n[kShellZ], e2 = e1 + w.n[kShellYZ], e3 = e2 + w.n[kShellX];
    const int4* items = w.items[kShellZ];
    if (p.g.plane * (long long)(p.g.nz + 1) < (1LL << 31)) {
        if (e_pass) k_shell_e<uint32_t><<<n, b, 0, st>>>(p, fi, fo, pin, pout, items, e1, e2, e3, m);
        else k_shell_h<uint32_t><<<n, b, 0, st>>>(p, fi, fo, pin, pout, items, e1, e2, e3, m);
    } else {
        if (e_pass) k_shell_e<long long><<<n, b, 0, st>>>(p, fi, fo, pin, pout, items, e1, e2, e3, m);
        else k_shell_h<long long><<<n, b, 0, st>>>(p, fi, fo, pin, pout, items, e1, e2, e3, m);
    }
    return cudaGetLastError();
}

// E of the nodes of the design region's edge box [d0, d3] x [d1, d4] x [d2, d5] (node class
// kDesignNode, which the other E kernels do not store), with the per-cell eps_r of the design
// cells. Design nodes are interior: no CPML memory, no lumped edge.
__global__ void __launch_bounds__(256) k_design_e(const __grid_constant__ StepParams p, FieldPtrs fi, FieldPtrs fo,
                                                  const __grid_constant__ PsiSet pin,
                                                  const __grid_constant__ PsiSet pout, long long m) {
    const int* d = p.dbox;
    // an FoM probe outside the design region: its E is final once the other E kernels are done
    if (p.fom_sample && p.fom_read >= 0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 &&
        threadIdx.y == 0)
        *p.fom_sample = fi.ez[p.fom_read];
    const int i = d[0] + blockIdx.x * 32 + threadIdx.x;
    const int j = d[1] + blockIdx.y * 8 + threadIdx.y;
    const int k = d[2] + blockIdx.z;
    if (i > d[3] || j > d[4]) return;
    e_node_global<true>(p, fi, fo, pin, pout, i, j, k, m);
}

// E of the nodes with a plate-covered edge (node class kPlateNode, which the other E kernels leave
// alone): one thread per listed node, plate-aware coefficients.
__global__ void __launch_bounds__(128) k_plate_e(const __grid_constant__ StepParams p, FieldPtrs fi, FieldPtrs fo,
                                                 const __grid_constant__ PsiSet pin,
                                                 const __grid_constant__ PsiSet pout, long long m) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= p.n_plate_nodes) return;
    const int4 v = p.plate_nodes[q];
    e_node_global<false, false, true>(p, fi, fo, pin, pout, v.x, v.y, v.z, m);
}

cudaError_t launch_plate_e(const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo, const PsiSet& pin,
                           const PsiSet& pout, long long m, cudaStream_t st) {
    if (p.n_plate_nodes <= 0) return cudaSuccess;
    k_plate_e<<<(p.n_plate_nodes + 127) / 128, 128, 0, st>>>(p, fi, fo, pin, pout, m);
    return cudaGetLastError();
}

cudaError_t launch_design_e(const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo, const PsiSet& pin,
                            const PsiSet& pout, long long m, cudaStream_t st) {
    if (!p.deps) return cudaSuccess;
    const int* d = p.dbox;
    const dim3 grid((d[3] - d[0] + 32) / 32, (d[4] - d[1] + 8) / 8, d[5] - d[2] + 1);
    k_design_e<<<grid, dim3(32, 8, 1), 0, st>>>(p, fi, fo, pin, pout, m);
    return cudaGetLastError();
}

// Two-pass kernels whose step index is *base + s: a CUDA graph captured once replays them while
// a counter on the device advances (the batched chain form).
template <typename Idx>
__global__ void __launch_bounds__(256, FDTD_TWO_PASS_MIN_BLOCKS) k_update_e_rel(const __grid_constant__ StepParams p,
                                                                                 FieldPtrs f,
                                                                                 const __grid_constant__ PsiSet ps,
                                                                                 const long long* __restrict__ base, int s) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    if (i >= p.g.nx || j >= p.g.ny) return;
    e_node_global<false, false, false, Idx>(p, f, f, ps, ps, i, j, blockIdx.z, *base + s);
}
template <typename Idx>
__global__ void __launch_bounds__(256, FDTD_TWO_PASS_MIN_BLOCKS) k_update_h_rel(const __grid_constant__ StepParams p,
                                                                                 FieldPtrs f,
                                                                                 const __grid_constant__ PsiSet ps,
                                                                                 const long long* __restrict__ base, int s) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    if (i >= p.g.nx || j >= p.g.ny) return;
    h_node_global<false, Idx>(p, f, f, f, ps, ps, i, j, blockIdx.z, *base + s);
}

cudaError_t launch_two_pass_rel(const StepParams& p, const FieldPtrs& f, const PsiSet& ps, const long long* base, int s,
                                cudaStream_t st) {
    if (p.deps || p.n_plate_nodes > 0) return cudaErrorInvalidValue;  // no design region, no plates
    dim3 block(32, 8, 1);
    dim3 grid((p.g.nx + 31) / 32, (p.g.ny + 7) / 8, p.g.nz);
    const bool idx32 = p.g.plane * (long long)(p.g.nz + 1) < (1LL << 31);
    if (idx32) k_update_e_rel<uint32_t><<<grid, block, 0, st>>>(p, f, ps, base, s);
    else k_update_e_rel<long long><<<grid, block, 0, st>>>(p, f, ps, base, s);
    if (idx32) k_update_h_rel<uint32_t><<<grid, block, 0, st>>>(p, f, ps, base, s);
    else k_update_h_rel<long long><<<grid, block, 0, st>>>(p, f, ps, base, s);
    return cudaGetLastError();
}

// Two-pass kernels over the nodes [b.x0, b.x1) x [b.y0, b.y1) x [b.z0, b.z1) only (the adjoint's
// segment recompute, whose nodes outside a shrinking box around the design region are never read
// again). Same per-node code, so the nodes inside give the same bits as a whole-grid step.
template <typename Idx>
__global__ void __launch_bounds__(256, FDTD_TWO_PASS_MIN_BLOCKS) k_update_e_box(const __grid_constant__ StepParams p,
                                                                                 FieldPtrs f,
                                                                                 const __grid_constant__ PsiSet ps,
                                                                                 NodeBox b, long long m) {
    const int i = b.x0 + blockIdx.x * 32 + threadIdx.x;
    const int j = b.y0 + blockIdx.y * 8 + threadIdx.y;
    if (i >= b.x1 || j >= b.y1) return;
    e_node_global<false, false, false, Idx>(p, f, f, ps, ps, i, j, b.z0 + blockIdx.z, m);
}
template <typename Idx>
__global__ void __launch_bounds__(256, FDTD_TWO_PASS_MIN_BLOCKS) k_update_h_box(const __grid_constant__ StepParams p,
                                                                                 FieldPtrs f,
                                                                                 const __grid_constant__ PsiSet ps,
                                                                                 NodeBox b, long long m) {
    const int i = b.x0 + blockIdx.x * 32 + threadIdx.x;
    const int j = b.y0 + blockIdx.y * 8 + threadIdx.y;
    if (i >= b.x1 || j >= b.y1) return;
    h_node_global<false, Idx>(p, f, f, f, ps, ps, i, j, b.z0 + blockIdx.z, m);
}

cudaError_t launch_two_pass_box(const StepParams& p, const FieldPtrs& f, const PsiSet& ps, const NodeBox& b, long long m,
                                cudaStream_t st) {
    const DeviceGrid& g = p.g;
    if (b.x0 < 0 || b.y0 < 0 || b.z0 < 0 || b.x1 > g.nx || b.y1 > g.ny || b.z1 > g.nz) return cudaErrorInvalidValue;
    if (b.x1 <= b.x0 || b.y1 <= b.y0 || b.z1 <= b.z0) return cudaSuccess;
    const dim3 block(32, 8, 1);
    const dim3 grid((b.x1 - b.x0 + 31) / 32, (b.y1 - b.y0 + 7) / 8, b.z1 - b.z0);
    const bool idx32 = g.plane * (long long)(g.nz + 1) < (1LL << 31);
    if (idx32) k_update_e_box<uint32_t><<<grid, block, 0, st>>>(p, f, ps, b, m);
    else k_update_e_box<long long><<<grid, block, 0, st>>>(p, f, ps, b, m);
    cudaError_t e = launch_design_e(p, f, f, ps, ps, m, st);
    if (e == cudaSuccess) e = launch_plate_e(p, f, f, ps, ps, m, st);
    if (e != cudaSuccess) return e;
    if (idx32) k_update_h_box<uint32_t><<<grid, block, 0, st>>>(p, f, ps, b, m);
    else k_update_h_box<long long><<<grid, block, 0, st>>>(p, f, ps, b, m);
    return cudaGetLastError();
}

cudaError_t launch_two_pass(const StepParams& p, const FieldPtrs& f, const PsiSet& ps, long long m,
                            cudaStream_t st) {
    dim3 block(32, 8, 1);
    dim3 grid((p.g.nx + 31) / 32, (p.g.ny + 7) / 8, p.g.nz);
    // 32-bit node offsets when every offset (plus one plane of lookahead) fits
    const bool idx32 = p.g.plane * (long long)(p.g.nz + 1) < (1LL << 31);
    if (idx32) k_update_e<uint32_t><<<grid, block, 0, st>>>(p, f, ps, m);
    else k_update_e<long long><<<grid, block, 0, st>>>(p, f, ps, m);
    cudaError_t e = launch_design_e(p, f, f, ps, ps, m, st);
    if (e == cudaSuccess) e = launch_plate_e(p, f, f, ps, ps, m, st);
    if (e != cudaSuccess) return e;
    if (idx32) k_update_h<uint32_t><<<grid, block, 0, st>>>(p, f, ps, m);
    else k_update_h<long long><<<grid, block, 0, st>>>(p, f, ps, m);
    return cudaGetLastError();
}

}  // namespace fdtd
