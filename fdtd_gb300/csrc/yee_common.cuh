// Per-node Yee update shared by every schedule.
//
// e_update / h_update compute one node's three E (or H) components from a neighbourhood struct
// that the caller fills, from global memory (two-pass schedule) or from shared-memory plane tiles
// (fused sweep). Coefficient reconstruction, masks, the lumped-element override, the CPML
// recurrences and every rounding step live here only, so all schedules produce identical bits.
//
// The function is written so that the common case costs little and the special cases diverge per
// component only: an edge whose surrounding cells hold one material takes its coefficients from
// the material table (the reference's averaging formula, with its divisions, runs only at material
// interfaces); in CPML slabs filled with the background material the kappa-divided coefficient
// comes from a per-axis table; components a boundary mask excludes keep their old value.
#pragma once

#include "fdtd_device.cuh"

namespace fdtd {

// True when node coordinate q lies in the CPML slabs of an axis with n nodes (setABCPML regions,
// fdtdrav.h:1860, 1912, 1960, 1993, 2059, 2107).
__device__ __forceinline__ bool in_slab(int q, int n, int pn, int pp) { return q < pn || q >= n - pp; }

// Offset of psi for node (i,j,k) in the x / y / z face slabs; `side` = 0 on the n face, 1 on the p face.
__device__ __forceinline__ int psi_off_x(const DeviceGrid& g, int i, int j, int k, int& side) {
    if (i < g.pxn) { side = 0; return (k * g.ny + j) * g.pxn + i; }
    side = 1;
    return (k * g.ny + j) * g.pxp + (i - (g.nx - g.pxp));
}
__device__ __forceinline__ int psi_off_y(const DeviceGrid& g, int i, int j, int k, int& side) {
    if (j < g.pyn) { side = 0; return (k * g.pyn + j) * g.pitch + i; }
    side = 1;
    return (k * g.pyp + (j - (g.ny - g.pyp))) * g.pitch + i;
}
__device__ __forceinline__ int psi_off_z(const DeviceGrid& g, int i, int j, int k, int& side) {
    if (k < g.pzn) { side = 0; return (k * g.ny + j) * g.pitch + i; }
    side = 1;
    return ((k - (g.nz - g.pzp)) * g.ny + j) * g.pitch + i;
}

// Coefficients of an edge between different materials: the edge averages of setSigmaEpsSigmaMu
// (fdtdrav.h:1135, 1153, 1170, reference summation order) and setCoefficients' expressions. Out of
// line with scalar arguments: it runs only at material interfaces and keeps its divisions out of
// the hot loop's instruction footprint.
// axis: the component's axis, whose cell values are averaged.
static __device__ __noinline__ Coef3 e_coef_mixed(const MatProps* props, int axis, int m0, int m1, int m2, int m3,
                                                  float dt, float eps0, float dp, float dm) {
    const MatAxis a = props[m0].a[axis], b = props[m1].a[axis], c = props[m2].a[axis], d = props[m3].a[axis];
    return coef3(avg4(a.eps, b.eps, c.eps, d.eps), avg4(a.sig, b.sig, c.sig, d.sig), dt, eps0, dp, dm);
}
// Harmonic means of two cells for an H face (fdtdrav.h:1183-1213).
static __device__ __noinline__ Coef3 h_coef_mixed(const MatProps* props, int axis, int m0, int m1, float dt, float mu0,
                                                  float dp, float dm) {
    const MatAxis a = props[m0].a[axis], b = props[m1].a[axis];
    return coef3(harm2(a.mu, b.mu), harm2(a.sigm, b.sigm), dt, mu0, dp, dm);
}
// A curl coefficient divided by the CPML kappa (setABCPML, fdtdrav.h:1903-1906 and mirrors).
static __device__ __noinline__ float kappa_div(float c, float kappa) { return __fdiv_rn(c, kappa); }

// eps_r of axis `axis` of cell (ci, cj, ck) holding material m: the design array for design
// cells (isotropic).
__device__ __forceinline__ float cell_eps(const StepParams& p, int m, int axis, int ci, int cj, int ck) {
    if (m == kDesign && p.deps) {
        const int* d = p.dbox;
        return p.deps[((long long)(ck - d[2]) * (d[4] - d[1]) + (cj - d[1])) * (d[3] - d[0]) + (ci - d[0])];
    }
    return p.props[m].a[axis].eps;
}
// The averaged eps_r and sigma_e of E edge `comp` at node (i, j, k) over its four cells in the
// reference's summation order: Ex (i,j,k) (i,j-1,k) (i,j,k-1) (i,j-1,k-1); Ey (i,j,k) (i-1,j,k)
// (i,j,k-1) (i-1,j,k-1); Ez (i,j,k) (i-1,j,k) (i,j-1,k) (i-1,j-1,k). m0..m3 are those cells' materials.
__device__ __forceinline__ void edge_material(const StepParams& p, int comp, int i, int j, int k, int m0, int m1, int m2,
                                              int m3, float& eps, float& sig) {
    int c1i = i, c1j = j, c1k = k, c2i = i, c2j = j, c2k = k - 1, c3i = i, c3j = j, c3k = k - 1;
    if (comp == 0) { c1j = j - 1; c3j = j - 1; }
    else if (comp == 1) { c1i = i - 1; c3i = i - 1; }
    else { c1i = i - 1; c2k = k; c2j = j - 1; c3i = i - 1; c3j = j - 1; c3k = k; }
    eps = avg4(cell_eps(p, m0, comp, i, j, k), cell_eps(p, m1, comp, c1i, c1j, c1k),
               cell_eps(p, m2, comp, c2i, c2j, c2k), cell_eps(p, m3, comp, c3i, c3j, c3k));
    sig = avg4(p.props[m0].a[comp].sig, p.props[m1].a[comp].sig, p.props[m2].a[comp].sig, p.props[m3].a[comp].sig);
}
// Coefficients of an E edge with a design cell among its four cells (setCoefficients on the
// averages, fdtdrav.h:1280-1303). Out of line: design edges are a small region.
static __device__ __noinline__ Coef3 e_coef_design(const StepParams* pp, int comp, int i, int j, int k, int m0, int m1,
                                                   int m2, int m3) {
    const StepParams& p = *pp;
    float eps, sig;
    edge_material(p, comp, i, j, k, m0, m1, m2, m3, eps, sig);
    const DeviceGrid& g = p.g;
    const float dp = comp == 0 ? g.dy : comp == 1 ? g.dz : g.dx;
    const float dm = comp == 0 ? g.dz : comp == 1 ? g.dx : g.dy;
    return coef3(eps, sig, g.dt, g.eps0, dp, dm);
}
__device__ __forceinline__ bool has_design(const StepParams& p, int m0, int m1, int m2, int m3) {
    return p.deps && (m0 == kDesign || m1 == kDesign || m2 == kDesign || m3 == kDesign);
}

// Zero-thickness plates (definePlateX / Y / Z, fdtdrav.h:1574-1679, applied after the edge averages
// and before setCoefficients): for each E component of node (i, j, k) that a plate covers, the
// coefficients from the edge's averaged eps_r and the plate's sigma_e (the last plate listed
// wins, as the reference writes them in order). Returns a bit per overridden component and
// writes its coefficients to c[comp]. Out of line: it runs only in planes holding a plate.
static __device__ __noinline__ int e_plate(const StepParams* pp, int i, int j, int k, int m0, int mi, int mj, int mk,
                                           int mij, int mik, int mjk, Coef3* c) {
    const StepParams& p = *pp;
    const int b = p.plate_k[k], e = p.plate_k[k + 1];
    float sig[3];
    int hit = 0;
    for (int q = b; q < e; ++q) {
        const PlateEdges& P = p.plates[q];
        if (i >= P.i0 && i <= P.i1 && j >= P.j0 && j <= P.j1) {
            sig[P.comp] = P.sigma;
            hit |= 1 << P.comp;
        }
    }
    const DeviceGrid& g = p.g;
    for (int comp = 0; comp < 3; ++comp) {
        if (!(hit & (1 << comp))) continue;
        float eps, s_avg;
        if (comp == 0) edge_material(p, 0, i, j, k, m0, mj, mk, mjk, eps, s_avg);
        else if (comp == 1) edge_material(p, 1, i, j, k, m0, mi, mk, mik, eps, s_avg);
        else edge_material(p, 2, i, j, k, m0, mi, mj, mij, eps, s_avg);
        const float dp = comp == 0 ? g.dy : comp == 1 ? g.dz : g.dx;
        const float dm = comp == 0 ? g.dz : comp == 1 ? g.dx : g.dy;
        c[comp] = coef3(eps, sig[comp], g.dt, g.eps0, dp, dm);
    }
    return hit;
}
__device__ __forceinline__ bool plane_has_plate(const StepParams& p, int k) {
    return p.plate_k && p.plate_k[k] < p.plate_k[k + 1];
}

// E-edge coefficients (setCoefficients, fdtdrav.h:1280-1303). `uni`: the four cells around the
// edge hold material m0, so the table entry applies. comp: 0 = Ex, 1 = Ey, 2 = Ez; the Cb cell
// sizes are Ex (dy, dz), Ey (dz, dx), Ez (dx, dy). kDesignAware: edges touching the design region
// average the per-cell eps_r. The update kernels compile without it (their registers, and with
// them their occupancy, would grow); the design region's E is then redone by k_design_e.
template <bool kDesignAware = false>
__device__ __forceinline__ Coef3 e_coef(const StepParams& p, int comp, bool uni, int m0, int m1, int m2, int m3, int i,
                                        int j, int k) {
    if (kDesignAware && has_design(p, m0, m1, m2, m3)) return e_coef_design(&p, comp, i, j, k, m0, m1, m2, m3);
    if (uni) {
        const float4 c = __ldg(&p.coef[m0].e[comp]);
        return Coef3{c.x, c.y, c.z};
    }
    const DeviceGrid& g = p.g;
    const float dp = comp == 0 ? g.dy : comp == 1 ? g.dz : g.dx;
    const float dm = comp == 0 ? g.dz : comp == 1 ? g.dx : g.dy;
    return e_coef_mixed(p.props, comp, m0, m1, m2, m3, g.dt, g.eps0, dp, dm);
}

// H-face coefficients (fdtdrav.h:1250-1272). `edge`: the low face of the axis (i = 0 for Hx, ...),
// where the reference keeps its initial mu = 1, sigma_m = 1.2e-38 (setSigmaEpsSigmaMu masks,
// fdtdrav.h:1181-1213); `uni`: both cells hold m0. Cb cell sizes: Hx (dz, dy), Hy (dx, dz), Hz (dy, dx).
__device__ __forceinline__ Coef3 h_coef(const StepParams& p, int comp, bool edge, bool uni, int m0, int m1) {
    if (edge || uni) {
        const float4 c = __ldg(&p.coef[edge ? kDefaultEntry : m0].h[comp]);
        return Coef3{c.x, c.y, c.z};
    }
    const DeviceGrid& g = p.g;
    const float dp = comp == 0 ? g.dz : comp == 1 ? g.dx : g.dy;
    const float dm = comp == 0 ? g.dy : comp == 1 ? g.dz : g.dx;
    return h_coef_mixed(p.props, comp, m0, m1, g.dt, g.mu0, dp, dm);
}

// Curl coefficient divided by the CPML kappa of its derivative axis. `bg_ok`: the coefficient is
// the table entry of the background material, whose divided values are tabulated per node (same
// division); otherwise divide here.
__device__ __forceinline__ float kdiv(float c, bool bg_ok, const float* bg_table, const float* kappa, int q) {
    return bg_ok ? __ldg(bg_table + q) : kappa_div(c, __ldg(kappa + q));
}

// Interior range of an axis: nodes that are neither on the two boundary planes nor in a CPML slab.
__device__ __forceinline__ bool interior(int q, int n, int pn, int pp) {
    return q >= (pn > 1 ? pn : 1) && q <= (n - 1 - pp < n - 2 ? n - 1 - pp : n - 2);
}

// Interior fast path: a node with every component updated, outside every CPML slab and lumped
// edge, whose surrounding cells all hold one material: table coefficients, no corrections.
// Same bits as e_update / h_update for such nodes.
__device__ __forceinline__ void e_update_interior(const StepParams& p, int m0, float ex, float ey, float ez,
                                                  float dHz_j, float dHy_k, float dHx_k, float dHz_i, float dHy_i,
                                                  float dHx_j, float out[3]) {
    const MatCoef* mc = p.coef + m0;
    const float4 a = __ldg(&mc->e[0]), b = __ldg(&mc->e[1]), c = __ldg(&mc->e[2]);
    out[0] = upd3(a.x, ex, a.y, dHz_j, a.z, dHy_k);
    out[1] = upd3(b.x, ey, b.y, dHx_k, b.z, dHz_i);
    out[2] = upd3(c.x, ez, c.y, dHy_i, c.z, dHx_j);
}
__device__ __forceinline__ void h_update_interior(const StepParams& p, int m0, float hx, float hy, float hz,
                                                  float dEy_k, float dEz_j, float dEz_i, float dEx_k, float dEx_j,
                                                  float dEy_i, float out[3]) {
    const MatCoef* mc = p.coef + m0;
    const float4 a = __ldg(&mc->h[0]), b = __ldg(&mc->h[1]), c = __ldg(&mc->h[2]);
    out[0] = upd3_hx(a.x, hx, a.y, dEy_k, a.z, dEz_j);
    out[1] = upd3(b.x, hy, b.y, dEz_i, b.z, dEx_k);
    out[2] = upd3(c.x, hz, c.y, dEx_j, c.z, dEy_i);
}

// Lumped-edge override of component comp (0 Ex, 2 Ez) for node (i,j) among the edges bucketed
// in plane k.
__device__ __forceinline__ const LumpedEdge* find_lumped(const StepParams& p, int i, int j, int k, int comp) {
    const int b = p.lumped_k[k], e = p.lumped_k[k + 1];
    for (int q = b; q < e; ++q) {
        const LumpedEdge& L = p.lumped[q];
        if (L.i == i && L.j == j && L.comp == comp) return &L;
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

// Neighbourhood of E(i,j,k): old E, H at the node and its lower neighbours, and the materials of the
// seven cells the three edge averages touch. Entries whose neighbour lies outside the grid are never
// used (the masks exclude those edges).
struct ENbr {
    float ex, ey, ez;
    float hx, hy, hz;
    float hx_jm, hx_km;  // Hx(i,j-1,k), Hx(i,j,k-1)
    float hy_im, hy_km;  // Hy(i-1,j,k), Hy(i,j,k-1)
    float hz_im, hz_jm;  // Hz(i-1,j,k), Hz(i,j-1,k)
    int m0, mi, mj, mk, mij, mik, mjk;  // cells (i,j,k) (i-1,j,k) (i,j-1,k) (i,j,k-1) (i-1,j-1,k) (i-1,j,k-1) (i,j-1,k-1)
};

// Neighbourhood of H(i,j,k): old H, new E at the node and its upper neighbours, cell materials.
struct HNbr {
    float hx, hy, hz;
    float ex, ey, ez;
    float ey_kp, ez_jp;  // Ey(i,j,k+1), Ez(i,j+1,k)   (Hx)
    float ez_ip, ex_kp;  // Ez(i+1,j,k), Ex(i,j,k+1)   (Hy)
    float ex_jp, ey_ip;  // Ex(i,j+1,k), Ey(i+1,j,k)   (Hz)
    int m0, mi, mj, mk;  // cells (i,j,k) (i-1,j,k) (i,j-1,k) (i,j,k-1)
};

__device__ __forceinline__ bool e_uniform(const ENbr& n) {
    return n.m0 == n.mi && n.m0 == n.mj && n.m0 == n.mk && n.m0 == n.mij && n.m0 == n.mik && n.m0 == n.mjk;
}
__device__ __forceinline__ bool h_uniform(const HNbr& n) { return n.m0 == n.mi && n.m0 == n.mj && n.m0 == n.mk; }

// The interior fast paths applied to a filled neighbourhood.
__device__ __forceinline__ void e_update_interior(const StepParams& p, const ENbr& n, float out[3]) {
    e_update_interior(p, n.m0, n.ex, n.ey, n.ez, __fsub_rn(n.hz, n.hz_jm), __fsub_rn(n.hy, n.hy_km),
                      __fsub_rn(n.hx, n.hx_km), __fsub_rn(n.hz, n.hz_im), __fsub_rn(n.hy, n.hy_im),
                      __fsub_rn(n.hx, n.hx_jm), out);
}
__device__ __forceinline__ void h_update_interior(const StepParams& p, const HNbr& n, float out[3]) {
    h_update_interior(p, n.m0, n.hx, n.hy, n.hz, __fsub_rn(n.ey_kp, n.ey), __fsub_rn(n.ez_jp, n.ez),
                      __fsub_rn(n.ez_ip, n.ez), __fsub_rn(n.ex_kp, n.ex), __fsub_rn(n.ex_jp, n.ex),
                      __fsub_rn(n.ey_ip, n.ey), out);
}

// CPML memory of one time level: read from `in`, written to `out` (the same set for in-place
// schedules). write = false computes with the old psi without storing (halo recomputation).
struct PsiIO {
    const PsiFace* in;
    const PsiFace* out;
    bool write;
};


// Old CPML memory of one node loaded ahead (the per-node kernels issue these loads with the field
// loads, since the addresses depend only on the node's position): for E (H) the two arrays of the
// x face, then the y face, then the z face, in e_update's (h_update's) order; entries of slabs the
// node is not in are unused.
struct PsiOld {
    float v[6];
};

// The old CPML memory of one slot. kCoherent: through L2 (ld.global.cg) instead of the read-only
// path; the batched persistent launch needs it, since it rewrites psi in one step and reads it
// again in the next within the same kernel. The other kernels read each psi once per launch.
template <bool kCoherent = false>
__device__ __forceinline__ float psi_load(const float* in, int q) {
    return kCoherent ? __ldcg(in + q) : __ldg(in + q);
}
// The old CPML memory of node (i, j, k) for e_update (kE) or h_update, for each slab of kSlabs the
// node lies in (entries of the others are left unset).
template <bool kE, bool kCoherent, int kSlabs>
__device__ __forceinline__ void psi_preload(const DeviceGrid& g, const PsiFace* in, int i, int j, int k, PsiOld& o) {
    int side;
    if ((kSlabs & 1) && in_slab(i, g.nx, g.pxn, g.pxp)) {
        const int q = psi_off_x(g, i, j, k, side);
        const PsiFace& f = in[side];
        o.v[0] = psi_load<kCoherent>(kE ? f.e[0] : f.h[0], q);
        o.v[1] = psi_load<kCoherent>(kE ? f.e[1] : f.h[1], q);
    }
    if ((kSlabs & 2) && in_slab(j, g.ny, g.pyn, g.pyp)) {
        const int q = psi_off_y(g, i, j, k, side);
        const PsiFace& f = in[2 + side];
        o.v[2] = psi_load<kCoherent>(kE ? f.e[0] : f.h[0], q);
        o.v[3] = psi_load<kCoherent>(kE ? f.e[1] : f.h[1], q);
    }
    if ((kSlabs & 4) && in_slab(k, g.nz, g.pzn, g.pzp)) {
        const int q = psi_off_z(g, i, j, k, side);
        const PsiFace& f = in[4 + side];
        o.v[4] = psi_load<kCoherent>(kE ? f.e[0] : f.h[0], q);
        o.v[5] = psi_load<kCoherent>(kE ? f.e[1] : f.h[1], q);
    }
}

// One CPML recurrence from the old memory value `old`.
template <bool kHyz = false>
__device__ __forceinline__ float psi_apply(float old, float* out, int q, bool write, float b, float a, float d, float f,
                                           float cpsi) {
    const float s = kHyz ? psi_upd_hyz(b, old, a, d) : psi_upd(b, old, a, d);
    if (write) out[q] = s;
    return psi_add(f, cpsi, s);
}

// Component masks of calc_e (fdtdrav.h:665, 696, 720) and calc_h (fdtdrav.h:328, 357, 382).
__device__ __forceinline__ void e_masks(const DeviceGrid& g, int i, int j, int k, bool& ex_m, bool& ey_m, bool& ez_m) {
    const bool in_x = i > 0 && i < g.nx - 1, in_y = j > 0 && j < g.ny - 1, in_z = k > 0 && k < g.nz - 1;
    ex_m = i < g.nx - 1 && in_y && in_z;
    ey_m = in_x && j < g.ny - 1 && in_z;
    ez_m = in_x && in_y && k < g.nz - 1;
}
__device__ __forceinline__ void h_masks(const DeviceGrid& g, int i, int j, int k, bool& hx_m, bool& hy_m, bool& hz_m) {
    hx_m = j < g.ny - 1 && k < g.nz - 1;
    hy_m = i < g.nx - 1 && k < g.nz - 1;
    hz_m = i < g.nx - 1 && j < g.ny - 1;
}

// One E node (calc_e fdtdrav.h:577-915): main updates with their masks and the lumped override,
// then the CPML corrections in the reference's order (x, y, z). pre[] receives the values between
// the main update and the CPML corrections (the sampleField values, fdtdrav.h:740).
// plane_lumped: some lumped edge lies in plane k (uniform across a CTA).
// kPlate: plate-covered edges take the plate's sigma_e (only k_plate_e, which updates the nodes of
// node class kPlateNode, instantiates it). kBg: a node whose seven cells all hold the background
// material and that carries no lumped edge (node class kUniformGeneral + background): the same
// arithmetic with the uniformity, background and lumped tests decided at compile time.
// kSlabs: the CPML slabs (bit 0 x, 1 y, 2 z) the node may lie in; the other slab tests compile out.
template <bool kDesignAware = false, bool kCoherent = false, bool kPlate = false, bool kBg = false, int kSlabs = 7>
__device__ __forceinline__ void e_update(const StepParams& p, const ENbr& n, int i, int j, int k, long long m,
                                         bool plane_lumped, const PsiIO& ps, float out[3], float pre[3],
                                         const PsiOld* old = nullptr) {
    const DeviceGrid& g = p.g;
    bool ex_m, ey_m, ez_m;  // fdtdrav.h:665, 696, 720
    e_masks(g, i, j, k, ex_m, ey_m, ez_m);
    const bool xs = (kSlabs & 1) && in_slab(i, g.nx, g.pxn, g.pxp);
    const bool ys = (kSlabs & 2) && in_slab(j, g.ny, g.pyn, g.pyp);
    const bool zs = (kSlabs & 4) && in_slab(k, g.nz, g.pzn, g.pzp);
    const int bg = p.bg.mat;
    const int m0 = kBg ? bg : n.m0;
    const bool ux = kBg || (n.m0 == n.mj && n.m0 == n.mk && n.m0 == n.mjk);
    const bool uy = kBg || (n.m0 == n.mi && n.m0 == n.mk && n.m0 == n.mik);
    const bool uz = kBg || (n.m0 == n.mi && n.m0 == n.mj && n.m0 == n.mij);
    const bool on_bg = kBg || n.m0 == bg;
    Coef3 cx = e_coef<kDesignAware>(p, 0, ux, m0, n.mj, n.mk, n.mjk, i, j, k);
    Coef3 cy = e_coef<kDesignAware>(p, 1, uy, m0, n.mi, n.mk, n.mik, i, j, k);
    Coef3 cz = e_coef<kDesignAware>(p, 2, uz, m0, n.mi, n.mj, n.mij, i, j, k);
    // plate-covered components (kPlate only): plate coefficients, and the background's tabulated
    // kappa-divided values (which belong to its table coefficients) no longer apply
    int pm = 0;
    if constexpr (kPlate) {
        if (plane_has_plate(p, k)) {
            Coef3 pc[3];
            pm = e_plate(&p, i, j, k, n.m0, n.mi, n.mj, n.mk, n.mij, n.mik, n.mjk, pc);
            if (pm & 1) cx = pc[0];
            if (pm & 2) cy = pc[1];
            if (pm & 4) cz = pc[2];
        }
    }
    const float dHz_j = __fsub_rn(n.hz, n.hz_jm), dHy_k = __fsub_rn(n.hy, n.hy_km);
    const float dHx_k = __fsub_rn(n.hx, n.hx_km), dHz_i = __fsub_rn(n.hz, n.hz_im);
    const float dHy_i = __fsub_rn(n.hy, n.hy_im), dHx_j = __fsub_rn(n.hx, n.hx_jm);
    const BgCurl& B = p.bg;
    // Ex (fdtdrav.h:665-676), with defineSourceX's coefficients on its edges (fdtdrav.h:1311-1365)
    const LumpedEdge* Lx = (!kBg && plane_lumped) ? find_lumped(p, i, j, k, 0) : nullptr;
    float vx = Lx ? upd3(Lx->ceze, n.ex, Lx->cezhy, dHz_j, Lx->cezhx, dHy_k)
                  : upd3(cx.a, n.ex, ys ? kdiv(cx.bp, ux && on_bg && !(pm & 1), B.e[1][0], p.key, j) : cx.bp, dHz_j,
                         zs ? kdiv(cx.bm, ux && on_bg && !(pm & 1), B.e[2][0], p.kez, k) : cx.bm, dHy_k);
    // Ey (fdtdrav.h:696-707)
    float vy = upd3(cy.a, n.ey, zs ? kdiv(cy.bp, uy && on_bg && !(pm & 2), B.e[2][1], p.kez, k) : cy.bp, dHx_k,
                    xs ? kdiv(cy.bm, uy && on_bg && !(pm & 2), B.e[0][0], p.kex, i) : cy.bm, dHz_i);
    // Ez with lumped elements (fdtdrav.h:720-741)
    float vz;
    const LumpedEdge* L = (!kBg && plane_lumped) ? find_lumped(p, i, j, k, 2) : nullptr;
    if (L) {
        if (L->source >= 0) {
            const float s = m < p.wave_len[L->source] ? p.waves[L->source][m] : 0.f;
            vz = upd4(L->ceze, n.ez, L->cezhy, dHy_i, L->cezhx, dHx_j, L->cezj, s);
        } else {
            vz = upd3(L->ceze, n.ez, L->cezhy, dHy_i, L->cezhx, dHx_j);
        }
    } else {
        vz = upd3(cz.a, n.ez, xs ? kdiv(cz.bp, uz && on_bg && !(pm & 4), B.e[0][1], p.kex, i) : cz.bp, dHy_i,
                  ys ? kdiv(cz.bm, uz && on_bg && !(pm & 4), B.e[1][1], p.key, j) : cz.bm, dHx_j);
    }
    pre[0] = ex_m ? vx : n.ex;
    pre[1] = ey_m ? vy : n.ey;
    pre[2] = ez_m ? vz : n.ez;
    int side;
    // CPML, per component in the reference's block order: x (fdtdrav.h:752-785), y (790-827),
    // z (829-911). The psi regions of the reference equal the component masks restricted to the
    // slabs, so psi is updated exactly where a correction is applied.
    if (xs && (ey_m || ez_m)) {
        const int q = psi_off_x(g, i, j, k, side);
        const float bb = __ldg(p.bex + i), aa = __ldg(p.aex + i);
        if (ey_m) vy = psi_apply(old ? old->v[0] : psi_load<kCoherent>(ps.in[side].e[0], q), ps.out[side].e[0], q, ps.write, bb, aa, dHz_i, vy, __fmul_rn(cy.bm, g.dx));
        if (ez_m) vz = psi_apply(old ? old->v[1] : psi_load<kCoherent>(ps.in[side].e[1], q), ps.out[side].e[1], q, ps.write, bb, aa, dHy_i, vz, __fmul_rn(cz.bp, g.dx));
    }
    if (ys && (ex_m || ez_m)) {
        const int q = psi_off_y(g, i, j, k, side);
        const float bb = __ldg(p.bey + j), aa = __ldg(p.aey + j);
        if (ex_m) vx = psi_apply(old ? old->v[2] : psi_load<kCoherent>(ps.in[2 + side].e[0], q), ps.out[2 + side].e[0], q, ps.write, bb, aa, dHz_j, vx, __fmul_rn(cx.bp, g.dy));
        if (ez_m) vz = psi_apply(old ? old->v[3] : psi_load<kCoherent>(ps.in[2 + side].e[1], q), ps.out[2 + side].e[1], q, ps.write, bb, aa, dHx_j, vz, __fmul_rn(cz.bm, g.dy));
    }
    if (zs && (ex_m || ey_m)) {
        const int q = psi_off_z(g, i, j, k, side);
        const float bb = __ldg(p.bez + k), aa = __ldg(p.aez + k);
        if (ex_m) vx = psi_apply(old ? old->v[4] : psi_load<kCoherent>(ps.in[4 + side].e[0], q), ps.out[4 + side].e[0], q, ps.write, bb, aa, dHy_k, vx, __fmul_rn(cx.bm, g.dz));
        if (ey_m) vy = psi_apply(old ? old->v[5] : psi_load<kCoherent>(ps.in[4 + side].e[1], q), ps.out[4 + side].e[1], q, ps.write, bb, aa, dHx_k, vy, __fmul_rn(cy.bp, g.dz));
    }
    out[0] = ex_m ? vx : n.ex;
    out[1] = ey_m ? vy : n.ey;
    out[2] = ez_m ? vz : n.ez;
}

// One H node (calc_h fdtdrav.h:249-573).
// kSlabs as for e_update.
template <bool kCoherent = false, bool kBg = false, int kSlabs = 7>
__device__ __forceinline__ void h_update(const StepParams& p, const HNbr& n, int i, int j, int k,
                                         const PsiIO& ps, float out[3], float pre[3], const PsiOld* old = nullptr) {
    const DeviceGrid& g = p.g;
    bool hx_m, hy_m, hz_m;  // fdtdrav.h:328, 357, 382
    h_masks(g, i, j, k, hx_m, hy_m, hz_m);
    const bool xs = (kSlabs & 1) && in_slab(i, g.nx, g.pxn, g.pxp);
    const bool ys = (kSlabs & 2) && in_slab(j, g.ny, g.pyn, g.pyp);
    const bool zs = (kSlabs & 4) && in_slab(k, g.nz, g.pzn, g.pzp);
    const int bg = p.bg.mat;
    const int m0 = kBg ? bg : n.m0;
    const bool ux = kBg || n.m0 == n.mi, uy = kBg || n.m0 == n.mj, uz = kBg || n.m0 == n.mk;
    const bool on_bg = kBg || n.m0 == bg;
    const Coef3 cx = h_coef(p, 0, i == 0, ux, m0, n.mi);
    const Coef3 cy = h_coef(p, 1, j == 0, uy, m0, n.mj);
    const Coef3 cz = h_coef(p, 2, k == 0, uz, m0, n.mk);
    // the tabulated kappa-divided values belong to the background material's table entry
    const bool bx = i != 0 && ux && on_bg, by = j != 0 && uy && on_bg, bz = k != 0 && uz && on_bg;
    const float dEy_k = __fsub_rn(n.ey_kp, n.ey), dEz_j = __fsub_rn(n.ez_jp, n.ez);
    const float dEz_i = __fsub_rn(n.ez_ip, n.ez), dEx_k = __fsub_rn(n.ex_kp, n.ex);
    const float dEx_j = __fsub_rn(n.ex_jp, n.ex), dEy_i = __fsub_rn(n.ey_ip, n.ey);
    const BgCurl& B = p.bg;
    // Hx (fdtdrav.h:331-338)
    float vx = upd3_hx(cx.a, n.hx, zs ? kdiv(cx.bp, bx, B.h[2][0], p.kmz, k) : cx.bp, dEy_k,
                       ys ? kdiv(cx.bm, bx, B.h[1][0], p.kmy, j) : cx.bm, dEz_j);
    // Hy (fdtdrav.h:360-366)
    float vy = upd3(cy.a, n.hy, xs ? kdiv(cy.bp, by, B.h[0][0], p.kmx, i) : cy.bp, dEz_i,
                    zs ? kdiv(cy.bm, by, B.h[2][1], p.kmz, k) : cy.bm, dEx_k);
    // Hz (fdtdrav.h:385)
    float vz = upd3(cz.a, n.hz, ys ? kdiv(cz.bp, bz, B.h[1][1], p.kmy, j) : cz.bp, dEx_j,
                    xs ? kdiv(cz.bm, bz, B.h[0][1], p.kmx, i) : cz.bm, dEy_i);
    pre[0] = hx_m ? vx : n.hx;
    pre[1] = hy_m ? vy : n.hy;
    pre[2] = hz_m ? vz : n.hz;
    int side;
    // CPML x (fdtdrav.h:401-442), y (445-486), z (489-562)
    if (xs && (hy_m || hz_m)) {
        const int q = psi_off_x(g, i, j, k, side);
        const float bb = __ldg(p.bmx + i), aa = __ldg(p.amx + i);
        if (hy_m) vy = psi_apply(old ? old->v[0] : psi_load<kCoherent>(ps.in[side].h[0], q), ps.out[side].h[0], q, ps.write, bb, aa, dEz_i, vy, __fmul_rn(cy.bp, g.dx));
        if (hz_m) vz = psi_apply(old ? old->v[1] : psi_load<kCoherent>(ps.in[side].h[1], q), ps.out[side].h[1], q, ps.write, bb, aa, dEy_i, vz, __fmul_rn(cz.bm, g.dx));
    }
    if (ys && (hx_m || hz_m)) {
        const int q = psi_off_y(g, i, j, k, side);
        const float bb = __ldg(p.bmy + j), aa = __ldg(p.amy + j);
        if (hx_m) vx = psi_apply(old ? old->v[2] : psi_load<kCoherent>(ps.in[2 + side].h[0], q), ps.out[2 + side].h[0], q, ps.write, bb, aa, dEz_j, vx, __fmul_rn(cx.bm, g.dy));
        if (hz_m) vz = psi_apply(old ? old->v[3] : psi_load<kCoherent>(ps.in[2 + side].h[1], q), ps.out[2 + side].h[1], q, ps.write, bb, aa, dEx_j, vz, __fmul_rn(cz.bp, g.dy));
    }
    if (zs && (hx_m || hy_m)) {
        const int q = psi_off_z(g, i, j, k, side);
        const float bb = __ldg(p.bmz + k), aa = __ldg(p.amz + k);
        if (hx_m) vx = psi_apply(old ? old->v[4] : psi_load<kCoherent>(ps.in[4 + side].h[0], q), ps.out[4 + side].h[0], q, ps.write, bb, aa, dEy_k, vx, __fmul_rn(cx.bp, g.dz));
        if (hy_m) vy = psi_apply<true>(old ? old->v[5] : psi_load<kCoherent>(ps.in[4 + side].h[1], q), ps.out[4 + side].h[1], q, ps.write, bb, aa, dEx_k, vy, __fmul_rn(cy.bm, g.dz));
    }
    out[0] = hx_m ? vx : n.hx;
    out[1] = hy_m ? vy : n.hy;
    out[2] = hz_m ? vz : n.hz;
}

}  // namespace fdtd
