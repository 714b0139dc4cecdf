// Per-node pieces of the Yee update shared by the two-pass and the fused schedules: coefficient
// reconstruction from the material index (with CPML kappa and cpsi), the component updates with
// their CPML corrections, lumped-edge overrides and probe sampling.
#pragma once

#include "fdtd_device.cuh"

namespace fdtd {

// True when node coordinate q lies in the CPML slabs of an axis with n nodes (setABCPML regions,
// fdtdrav.h:1860, 1912, 1960, 1993, 2059, 2107).
__device__ __forceinline__ bool in_slab(int q, int n, int pn, int pp) { return q < pn || q >= n - pp; }

// Slab index of psi for node (i,j,k) on the x / y / z faces. Returns the face (0 = n side,
// 1 = p side) through `side`.
__device__ __forceinline__ long long psi_index_x(const DeviceGrid& g, int i, int j, int k, int& side) {
    if (i < g.pxn) { side = 0; return ((long long)k * g.ny + j) * g.pxn + i; }
    side = 1;
    return ((long long)k * g.ny + j) * g.pxp + (i - (g.nx - g.pxp));
}
__device__ __forceinline__ long long psi_index_y(const DeviceGrid& g, int i, int j, int k, int& side) {
    if (j < g.pyn) { side = 0; return ((long long)k * g.pyn + j) * g.pitch + i; }
    side = 1;
    return ((long long)k * g.pyp + (j - (g.ny - g.pyp))) * g.pitch + i;
}
__device__ __forceinline__ long long psi_index_z(const DeviceGrid& g, int i, int j, int k, int& side) {
    if (k < g.pzn) { side = 0; return ((long long)k * g.ny + j) * g.pitch + i; }
    side = 1;
    return ((long long)(k - (g.nz - g.pzp)) * g.ny + j) * g.pitch + i;
}

// E-edge coefficients from the four cells around the edge (a: the node's own cell, then the
// reference's order of setSigmaEpsSigmaMu). comp: 0 = Ex, 1 = Ey, 2 = Ez.
__device__ __forceinline__ Coef3 e_coef(const StepParams& p, int comp, int m0, int m1, int m2, int m3) {
    if (m0 == m1 && m0 == m2 && m0 == m3) {
        const float* c = p.coef[m0].e[comp];
        return Coef3{c[0], c[1], c[2]};
    }
    const MatProps a = p.props[m0], b = p.props[m1], c = p.props[m2], d = p.props[m3];
    const float eps = avg4(a.eps, b.eps, c.eps, d.eps);
    const float sig = avg4(a.sig, b.sig, c.sig, d.sig);
    const DeviceGrid& g = p.g;
    // (Cb_plus, Cb_minus) cell sizes: Ex (dy, dz), Ey (dz, dx), Ez (dx, dy) (fdtdrav.h:1280-1303)
    const float dp = comp == 0 ? g.dy : comp == 1 ? g.dz : g.dx;
    const float dm = comp == 0 ? g.dz : comp == 1 ? g.dx : g.dy;
    return coef3(eps, sig, g.dt, g.eps0, dp, dm);
}

// H-face coefficients from the two cells sharing the face (harmonic means). `edge` is true on the
// low face of the axis (i = 0 for Hx, ...), where the reference keeps its initial mu = 1,
// sigma_m = 1.2e-38 (setSigmaEpsSigmaMu masks, fdtdrav.h:1181-1213).
__device__ __forceinline__ Coef3 h_coef(const StepParams& p, int comp, bool edge, int m0, int m1) {
    if (edge) {
        const float* c = p.coef[kDefaultEntry].h[comp];
        return Coef3{c[0], c[1], c[2]};
    }
    if (m0 == m1) {
        const float* c = p.coef[m0].h[comp];
        return Coef3{c[0], c[1], c[2]};
    }
    const MatProps a = p.props[m0], b = p.props[m1];
    const float mu = harm2(a.mu, b.mu);
    const float sm = harm2(a.sigm, b.sigm);
    const DeviceGrid& g = p.g;
    // Hx (dz, dy), Hy (dx, dz), Hz (dy, dx) (fdtdrav.h:1250-1272)
    const float dp = comp == 0 ? g.dz : comp == 1 ? g.dx : g.dy;
    const float dm = comp == 0 ? g.dy : comp == 1 ? g.dz : g.dx;
    return coef3(mu, sm, g.dt, g.mu0, dp, dm);
}

// Look up a lumped-edge override for node (i,j) among the edges bucketed in plane k.
__device__ __forceinline__ const LumpedEdge* find_lumped(const StepParams& p, int i, int j, int k) {
    const int b = p.lumped_k[k], e = p.lumped_k[k + 1];
    for (int q = b; q < e; ++q) {
        const LumpedEdge& L = p.lumped[q];
        if (L.i == i && L.j == j) return &L;
    }
    return nullptr;
}

__device__ __forceinline__ void sample(const StepParams& p, long long row, int comp, int i, int j, int k, float v) {
    const int b = p.probe_k[k], e = p.probe_k[k + 1];
    for (int q = b; q < e; ++q) {
        const Probe& pr = p.probes[q];
        if (pr.comp == comp && pr.i == i && pr.j == j)
            p.probe_ring[row * p.n_probes + p.probe_ids[q]] = v;
    }
}

}  // namespace fdtd
