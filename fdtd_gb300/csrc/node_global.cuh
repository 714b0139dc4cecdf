// Per-node E and H updates reading the fields from global memory: the two-pass schedule, the
// shell passes of the fused schedule, the design-region kernel and the batched launch share them.
#pragma once

#include "yee_common.cuh"
#include "yee_kernels.h"

namespace fdtd {

// One node's E (or H) update reading the fields `fi` and CPML memory `pin`, writing `fo` / `pout`
// (the same buffers for the in-place two-pass schedule). Every node loads its twelve field values
// and its class byte together (one round of memory latency); fast-path nodes (class below
// kUniformGeneral) then update from the material table, interface nodes from their row of the
// coefficient table, the rest also gather the seven cell materials and take
// e_update / h_update. kDesign (k_design_e only): skip the class test and average the per-cell
// eps_r of design cells. kPlate (k_plate_e only): plate-covered edges take the plate's sigma_e;
// the other kernels leave plate nodes (class kPlateNode) alone, CPML memory included.
// Idx: the integer type of node offsets; uint32_t when the field arrays hold fewer than 2^31
// elements, which saves the 64-bit address arithmetic of every load and store. kSlabs: the CPML
// slabs (bit 0 x, 1 y, 2 z) the caller's nodes may lie in; the other slab tests compile out.
// kEarly: a CPML node's old psi is loaded together with its fields (the addresses depend only on
// the node's position) instead of after its class has chosen the path; one round of memory latency
// less, a few more registers live across the loads.
template <bool kDesign = false, bool kCoherent = false, bool kPlate = false, typename Idx = long long, int kSlabs = 7,
          bool kEarly = false>
__device__ __forceinline__ void e_node_global(const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo,
                                              const PsiSet& pin, const PsiSet& pout, int i, int j, int k, long long m) {
    const DeviceGrid& g = p.g;
    const Idx n = (Idx)k * (Idx)g.plane + (Idx)j * (Idx)g.pitch + (Idx)i;
    const Idx P = (Idx)g.plane, R = (Idx)g.pitch;
    ENbr nb;
    nb.ex = fi.ex[n]; nb.ey = fi.ey[n]; nb.ez = fi.ez[n];
    nb.hx = fi.hx[n]; nb.hy = fi.hy[n]; nb.hz = fi.hz[n];
    nb.hx_jm = j > 0 ? fi.hx[n - R] : 0.f;
    nb.hx_km = k > 0 ? fi.hx[n - P] : 0.f;
    nb.hy_im = i > 0 ? fi.hy[n - 1] : 0.f;
    nb.hy_km = k > 0 ? fi.hy[n - P] : 0.f;
    nb.hz_im = i > 0 ? fi.hz[n - 1] : 0.f;
    nb.hz_jm = j > 0 ? fi.hz[n - R] : 0.f;
    PsiOld po;
    if (kEarly && !kDesign) psi_preload<true, kCoherent, kSlabs>(g, pin.f, i, j, k, po);
    const PsiOld* pop = (kEarly && !kDesign) ? &po : nullptr;
    const int c = kDesign ? kGeneral : p.cls[n];
    float out[3], pre[3];
    if (c < kUniformGeneral || c == kInterfaceNode) {
        // an interface node's coefficient row is one more load, taken only by such nodes
        const int row = c == kInterfaceNode ? (int)p.rec[n] : c;
        e_update_interior(p, row, nb.ex, nb.ey, nb.ez, __fsub_rn(nb.hz, nb.hz_jm), __fsub_rn(nb.hy, nb.hy_km),
                          __fsub_rn(nb.hx, nb.hx_km), __fsub_rn(nb.hz, nb.hz_im), __fsub_rn(nb.hy, nb.hy_im),
                          __fsub_rn(nb.hx, nb.hx_jm), out);
        pre[0] = out[0]; pre[1] = out[1]; pre[2] = out[2];
    } else {
        if (c >= kUniformGeneral && c < kInterfaceNode) {  // seven cells of one material: no loads
            nb.m0 = nb.mi = nb.mj = nb.mk = nb.mij = nb.mik = nb.mjk = c - kUniformGeneral;
        } else {
            const uint8_t* mat = p.mat;
            nb.m0 = mat[n];
            nb.mi = i > 0 ? mat[n - 1] : 0;
            nb.mj = j > 0 ? mat[n - R] : 0;
            nb.mk = k > 0 ? mat[n - P] : 0;
            nb.mij = (i > 0 && j > 0) ? mat[n - 1 - R] : 0;
            nb.mik = (i > 0 && k > 0) ? mat[n - 1 - P] : 0;
            nb.mjk = (j > 0 && k > 0) ? mat[n - R - P] : 0;
        }
        // plate nodes are k_plate_e's, CPML memory included: the other kernels store nothing of them
        const PsiIO io{pin.f, pout.f, kPlate || c != kPlateNode};
        if (!kDesign && !kPlate && c == kUniformGeneral + p.bg.mat) {  // CPML / boundary background node
            e_update<false, kCoherent, false, true, kSlabs>(p, nb, i, j, k, m, false, io, out, pre, pop);
        } else {
            const bool plane_lumped = p.lumped_k[k] < p.lumped_k[k + 1];
            e_update<kDesign, kCoherent, kPlate, false, kSlabs>(p, nb, i, j, k, m, plane_lumped, io, out, pre, pop);
        }
    }
    // k_design_e writes the design region's E, k_plate_e the plate nodes' E
    if (!kDesign && !kPlate && (c == kDesignNode || c == kPlateNode)) return;
    fo.ex[n] = out[0]; fo.ey[n] = out[1]; fo.ez[n] = out[2];
    if (kDesign && p.design_snap) {  // adjoint records (k_design_e covers the design edge box)
        const int* d = p.dbox;
        const long long bx = d[3] - d[0] + 1, by = d[4] - d[1] + 1, ne = bx * by * (d[5] - d[2] + 1);
        const long long q = ((long long)(k - d[2]) * by + (j - d[1])) * bx + (i - d[0]);
        p.design_snap[q] = out[0]; p.design_snap[ne + q] = out[1]; p.design_snap[2 * ne + q] = out[2];
    }
    if (kDesign && p.fom_sample && (long long)n == p.fom_node) *p.fom_sample = out[2];
    if (p.probe_k[k] < p.probe_k[k + 1]) {
        const long long row = m % p.ring_cap;
        for (int q = 0; q < 3; ++q) sample(p, row, q, i, j, k, pre[q]);
    }
}

// H reads the old H from `fi` and the new E from `fe`.
template <bool kCoherent = false, typename Idx = long long, int kSlabs = 7, bool kEarly = false>
__device__ __forceinline__ void h_node_global(const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fe,
                                              const FieldPtrs& fo, const PsiSet& pin, const PsiSet& pout, int i, int j,
                                              int k, long long m) {
    const DeviceGrid& g = p.g;
    const Idx n = (Idx)k * (Idx)g.plane + (Idx)j * (Idx)g.pitch + (Idx)i;
    const Idx P = (Idx)g.plane, R = (Idx)g.pitch;
    HNbr nb;
    nb.hx = fi.hx[n]; nb.hy = fi.hy[n]; nb.hz = fi.hz[n];
    nb.ex = fe.ex[n]; nb.ey = fe.ey[n]; nb.ez = fe.ez[n];
    nb.ey_kp = k < g.nz - 1 ? fe.ey[n + P] : 0.f;
    nb.ez_jp = j < g.ny - 1 ? fe.ez[n + R] : 0.f;
    nb.ez_ip = i < g.nx - 1 ? fe.ez[n + 1] : 0.f;
    nb.ex_kp = k < g.nz - 1 ? fe.ex[n + P] : 0.f;
    nb.ex_jp = j < g.ny - 1 ? fe.ex[n + R] : 0.f;
    nb.ey_ip = i < g.nx - 1 ? fe.ey[n + 1] : 0.f;
    PsiOld po;
    if (kEarly) psi_preload<false, kCoherent, kSlabs>(g, pin.f, i, j, k, po);
    const PsiOld* pop = kEarly ? &po : nullptr;
    const int c = p.cls[n];
    float out[3], pre[3];
    if (c < kUniformGeneral || c == kInterfaceNode) {
        const int row = c == kInterfaceNode ? (int)p.rec[n] : c;
        h_update_interior(p, row, nb.hx, nb.hy, nb.hz, __fsub_rn(nb.ey_kp, nb.ey), __fsub_rn(nb.ez_jp, nb.ez),
                          __fsub_rn(nb.ez_ip, nb.ez), __fsub_rn(nb.ex_kp, nb.ex), __fsub_rn(nb.ex_jp, nb.ex),
                          __fsub_rn(nb.ey_ip, nb.ey), out);
        pre[0] = out[0]; pre[1] = out[1]; pre[2] = out[2];
    } else {
        if (c >= kUniformGeneral && c < kInterfaceNode) {
            nb.m0 = nb.mi = nb.mj = nb.mk = c - kUniformGeneral;
        } else {
            const uint8_t* mat = p.mat;
            nb.m0 = mat[n];
            nb.mi = i > 0 ? mat[n - 1] : 0;
            nb.mj = j > 0 ? mat[n - R] : 0;
            nb.mk = k > 0 ? mat[n - P] : 0;
        }
        const PsiIO io{pin.f, pout.f, true};
        if (c == kUniformGeneral + p.bg.mat) h_update<kCoherent, true, kSlabs>(p, nb, i, j, k, io, out, pre, pop);  // background node
        else h_update<kCoherent, false, kSlabs>(p, nb, i, j, k, io, out, pre, pop);
    }
    fo.hx[n] = out[0]; fo.hy[n] = out[1]; fo.hz[n] = out[2];
    if (p.probe_k[k] < p.probe_k[k + 1]) {
        const long long row = m % p.ring_cap;
        for (int q = 0; q < 3; ++q) sample(p, row, 3 + q, i, j, k, pre[q]);
    }
}

}  // namespace fdtd
