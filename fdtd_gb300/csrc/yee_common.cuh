// Per-node Yee update shared by every schedule.
//
// e_update / h_update compute one node's three E (or H) components from a neighbourhood struct
// that the caller fills, from global memory (two-pass schedule) or from shared-memory plane tiles
// (fused sweep). The coefficient reconstruction, the masks, the lumped-element override, the CPML
// recurrences and every rounding step live here only, so all schedules produce identical bits.
#pragma once

#include "fdtd_device.cuh"

namespace fdtd {

// True when node coordinate q lies in the CPML slabs of an axis with n nodes (setABCPML regions,
// fdtdrav.h:1860, 1912, 1960, 1993, 2059, 2107).
__device__ __forceinline__ bool in_slab(int q, int n, int pn, int pp) { return q < pn || q >= n - pp; }

// Slab index of psi for node (i,j,k) on the x / y / z faces; `side` = 0 on the n face, 1 on the p face.
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

// E-edge coefficients from the four cells around the edge, in the reference's summation order
// (setSigmaEpsSigmaMu fdtdrav.h:1135, 1153, 1170). comp: 0 = Ex, 1 = Ey, 2 = Ez.
__device__ __forceinline__ Coef3 e_coef(const StepParams& p, int comp, int m0, int m1, int m2, int m3) {
    if (m0 == m1 && m0 == m2 && m0 == m3) {
        const float* c = p.coef[m0].e[comp];
        return Coef3{__ldg(c), __ldg(c + 1), __ldg(c + 2)};
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

// H-face coefficients from the two cells sharing the face (harmonic means, fdtdrav.h:1183-1213).
// `edge` is true on the low face of the axis (i = 0 for Hx, ...), where the reference keeps its
// initial mu = 1, sigma_m = 1.2e-38.
__device__ __forceinline__ Coef3 h_coef(const StepParams& p, int comp, bool edge, int m0, int m1) {
    const int e = edge ? kDefaultEntry : m0;
    if (edge || m0 == m1) {
        const float* c = p.coef[e].h[comp];
        return Coef3{__ldg(c), __ldg(c + 1), __ldg(c + 2)};
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

// Lumped-edge override for node (i,j) among the edges bucketed in plane k.
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

// CPML memory of one time level: read from `in`, written to `out` (the same set for in-place
// schedules). write = false computes with the old psi without storing (halo recomputation).
struct PsiIO {
    const PsiFace* in;
    const PsiFace* out;
    bool write;
};

template <bool kHyz = false>
__device__ __forceinline__ float psi_step(const float* in, float* out, long long q, bool write,
                                          float b, float a, float d, float f, float cpsi) {
    const float s = kHyz ? psi_upd_hyz(b, in[q], a, d) : psi_upd(b, in[q], a, d);
    if (write) out[q] = s;
    return psi_add(f, cpsi, s);
}

// Fast path for an E node strictly inside the grid, outside every CPML slab and lumped element,
// whose seven surrounding cells hold one material m: every coefficient is the table entry of m and
// no correction follows the main update. Gives the same bits as e_update for such a node.
__device__ __forceinline__ bool e_fast_ok(const ENbr& n) {
    return n.m0 == n.mi && n.m0 == n.mj && n.m0 == n.mk && n.m0 == n.mij && n.m0 == n.mik && n.m0 == n.mjk;
}
__device__ __forceinline__ void e_update_fast(const StepParams& p, const ENbr& n, float out[3]) {
    const float* c = p.coef[n.m0].e[0];
    out[0] = upd3(__ldg(c + 0), n.ex, __ldg(c + 1), __fsub_rn(n.hz, n.hz_jm), __ldg(c + 2), __fsub_rn(n.hy, n.hy_km));
    out[1] = upd3(__ldg(c + 3), n.ey, __ldg(c + 4), __fsub_rn(n.hx, n.hx_km), __ldg(c + 5), __fsub_rn(n.hz, n.hz_im));
    out[2] = upd3(__ldg(c + 6), n.ez, __ldg(c + 7), __fsub_rn(n.hy, n.hy_im), __ldg(c + 8), __fsub_rn(n.hx, n.hx_jm));
}
// Same for an H node with i, j, k >= 1 (no reference-default faces) and four equal cells.
__device__ __forceinline__ bool h_fast_ok(const HNbr& n) { return n.m0 == n.mi && n.m0 == n.mj && n.m0 == n.mk; }
__device__ __forceinline__ void h_update_fast(const StepParams& p, const HNbr& n, float out[3]) {
    const float* c = p.coef[n.m0].h[0];
    out[0] = upd3_hx(__ldg(c + 0), n.hx, __ldg(c + 1), __fsub_rn(n.ey_kp, n.ey), __ldg(c + 2), __fsub_rn(n.ez_jp, n.ez));
    out[1] = upd3(__ldg(c + 3), n.hy, __ldg(c + 4), __fsub_rn(n.ez_ip, n.ez), __ldg(c + 5), __fsub_rn(n.ex_kp, n.ex));
    out[2] = upd3(__ldg(c + 6), n.hz, __ldg(c + 7), __fsub_rn(n.ex_jp, n.ex), __ldg(c + 8), __fsub_rn(n.ey_ip, n.ey));
}

// One E node (calc_e fdtdrav.h:577-915): main updates with masks and the lumped override, then the
// CPML corrections in the reference's order (x, y, z per component). pre[] receives the values
// between the main update and the CPML corrections (the sampleField values).
__device__ __forceinline__ void e_update(const StepParams& p, const ENbr& n, int i, int j, int k, long long m,
                                         const PsiIO& ps, float out[3], float pre[3]) {
    const DeviceGrid& g = p.g;
    out[0] = n.ex; out[1] = n.ey; out[2] = n.ez;
    pre[0] = n.ex; pre[1] = n.ey; pre[2] = n.ez;
    const bool in_x = i > 0 && i < g.nx - 1, in_y = j > 0 && j < g.ny - 1, in_z = k > 0 && k < g.nz - 1;
    const bool ex_m = i < g.nx - 1 && in_y && in_z;
    const bool ey_m = in_x && j < g.ny - 1 && in_z;
    const bool ez_m = in_x && in_y && k < g.nz - 1;
    if (!(ex_m || ey_m || ez_m)) return;
    const bool xs = in_slab(i, g.nx, g.pxn, g.pxp);
    const bool ys = in_slab(j, g.ny, g.pyn, g.pyp);
    const bool zs = in_slab(k, g.nz, g.pzn, g.pzp);
    int side;
    if (ex_m) {  // Ex (fdtdrav.h:665-676); CPML y (790-808) then z (829-850)
        const Coef3 c = e_coef(p, 0, n.m0, n.mj, n.mk, n.mjk);
        float cy = c.bp, cz = c.bm;
        if (ys) cy = __fdiv_rn(c.bp, p.key[j]);
        if (zs) cz = __fdiv_rn(c.bm, p.kez[k]);
        const float dHz = __fsub_rn(n.hz, n.hz_jm);
        const float dHy = __fsub_rn(n.hy, n.hy_km);
        float v = upd3(c.a, n.ex, cy, dHz, cz, dHy);
        pre[0] = v;
        if (ys) {
            const long long q = psi_index_y(g, i, j, k, side);
            v = psi_step(ps.in[2 + side].e[0], ps.out[2 + side].e[0], q, ps.write, p.bey[j], p.aey[j], dHz, v,
                         __fmul_rn(c.bp, g.dy));
        }
        if (zs) {
            const long long q = psi_index_z(g, i, j, k, side);
            v = psi_step(ps.in[4 + side].e[0], ps.out[4 + side].e[0], q, ps.write, p.bez[k], p.aez[k], dHy, v,
                         __fmul_rn(c.bm, g.dz));
        }
        out[0] = v;
    }
    if (ey_m) {  // Ey (fdtdrav.h:696-707); CPML x then z
        const Coef3 c = e_coef(p, 1, n.m0, n.mi, n.mk, n.mik);
        float cz = c.bp, cx = c.bm;
        if (zs) cz = __fdiv_rn(c.bp, p.kez[k]);
        if (xs) cx = __fdiv_rn(c.bm, p.kex[i]);
        const float dHx = __fsub_rn(n.hx, n.hx_km);
        const float dHz = __fsub_rn(n.hz, n.hz_im);
        float v = upd3(c.a, n.ey, cz, dHx, cx, dHz);
        pre[1] = v;
        if (xs) {
            const long long q = psi_index_x(g, i, j, k, side);
            v = psi_step(ps.in[side].e[0], ps.out[side].e[0], q, ps.write, p.bex[i], p.aex[i], dHz, v,
                         __fmul_rn(c.bm, g.dx));
        }
        if (zs) {
            const long long q = psi_index_z(g, i, j, k, side);
            v = psi_step(ps.in[4 + side].e[1], ps.out[4 + side].e[1], q, ps.write, p.bez[k], p.aez[k], dHx, v,
                         __fmul_rn(c.bp, g.dz));
        }
        out[1] = v;
    }
    if (ez_m) {  // Ez with lumped elements (fdtdrav.h:720-741); CPML x then y
        const Coef3 c = e_coef(p, 2, n.m0, n.mi, n.mj, n.mij);
        float cx = c.bp, cy = c.bm;
        if (xs) cx = __fdiv_rn(c.bp, p.kex[i]);
        if (ys) cy = __fdiv_rn(c.bm, p.key[j]);
        const float dHy = __fsub_rn(n.hy, n.hy_im);
        const float dHx = __fsub_rn(n.hx, n.hx_jm);
        float v;
        const LumpedEdge* L = (p.lumped_k[k] < p.lumped_k[k + 1]) ? find_lumped(p, i, j, k) : nullptr;
        if (L) {
            if (L->source >= 0) {
                const float s = m < p.wave_len[L->source] ? p.waves[L->source][m] : 0.f;
                v = upd4(L->ceze, n.ez, L->cezhy, dHy, L->cezhx, dHx, L->cezj, s);
            } else {
                v = upd3(L->ceze, n.ez, L->cezhy, dHy, L->cezhx, dHx);
            }
        } else {
            v = upd3(c.a, n.ez, cx, dHy, cy, dHx);
        }
        pre[2] = v;
        if (xs) {
            const long long q = psi_index_x(g, i, j, k, side);
            v = psi_step(ps.in[side].e[1], ps.out[side].e[1], q, ps.write, p.bex[i], p.aex[i], dHy, v,
                         __fmul_rn(c.bp, g.dx));
        }
        if (ys) {
            const long long q = psi_index_y(g, i, j, k, side);
            v = psi_step(ps.in[2 + side].e[1], ps.out[2 + side].e[1], q, ps.write, p.bey[j], p.aey[j], dHx, v,
                         __fmul_rn(c.bm, g.dy));
        }
        out[2] = v;
    }
}

// One H node (calc_h fdtdrav.h:249-573).
__device__ __forceinline__ void h_update(const StepParams& p, const HNbr& n, int i, int j, int k,
                                         const PsiIO& ps, float out[3], float pre[3]) {
    const DeviceGrid& g = p.g;
    out[0] = n.hx; out[1] = n.hy; out[2] = n.hz;
    pre[0] = n.hx; pre[1] = n.hy; pre[2] = n.hz;
    const bool hx_m = j < g.ny - 1 && k < g.nz - 1;
    const bool hy_m = i < g.nx - 1 && k < g.nz - 1;
    const bool hz_m = i < g.nx - 1 && j < g.ny - 1;
    const bool xs = in_slab(i, g.nx, g.pxn, g.pxp);
    const bool ys = in_slab(j, g.ny, g.pyn, g.pyp);
    const bool zs = in_slab(k, g.nz, g.pzn, g.pzp);
    int side;
    if (hx_m) {  // Hx (fdtdrav.h:328-348); CPML y (445-486) then z (489-528)
        const Coef3 c = h_coef(p, 0, i == 0, n.m0, n.mi);
        float cz = c.bp, cy = c.bm;
        if (zs) cz = __fdiv_rn(c.bp, p.kmz[k]);
        if (ys) cy = __fdiv_rn(c.bm, p.kmy[j]);
        const float dEy = __fsub_rn(n.ey_kp, n.ey);
        const float dEz = __fsub_rn(n.ez_jp, n.ez);
        float v = upd3_hx(c.a, n.hx, cz, dEy, cy, dEz);
        pre[0] = v;
        if (ys) {
            const long long q = psi_index_y(g, i, j, k, side);
            v = psi_step(ps.in[2 + side].h[0], ps.out[2 + side].h[0], q, ps.write, p.bmy[j], p.amy[j], dEz, v,
                         __fmul_rn(c.bm, g.dy));
        }
        if (zs) {
            const long long q = psi_index_z(g, i, j, k, side);
            v = psi_step(ps.in[4 + side].h[0], ps.out[4 + side].h[0], q, ps.write, p.bmz[k], p.amz[k], dEy, v,
                         __fmul_rn(c.bp, g.dz));
        }
        out[0] = v;
    }
    if (hy_m) {  // Hy (fdtdrav.h:357-373); CPML x then z
        const Coef3 c = h_coef(p, 1, j == 0, n.m0, n.mj);
        float cx = c.bp, cz = c.bm;
        if (xs) cx = __fdiv_rn(c.bp, p.kmx[i]);
        if (zs) cz = __fdiv_rn(c.bm, p.kmz[k]);
        const float dEz = __fsub_rn(n.ez_ip, n.ez);
        const float dEx = __fsub_rn(n.ex_kp, n.ex);
        float v = upd3(c.a, n.hy, cx, dEz, cz, dEx);
        pre[1] = v;
        if (xs) {
            const long long q = psi_index_x(g, i, j, k, side);
            v = psi_step(ps.in[side].h[0], ps.out[side].h[0], q, ps.write, p.bmx[i], p.amx[i], dEz, v,
                         __fmul_rn(c.bp, g.dx));
        }
        if (zs) {
            const long long q = psi_index_z(g, i, j, k, side);
            v = psi_step<true>(ps.in[4 + side].h[1], ps.out[4 + side].h[1], q, ps.write, p.bmz[k], p.amz[k], dEx, v,
                               __fmul_rn(c.bm, g.dz));
        }
        out[1] = v;
    }
    if (hz_m) {  // Hz (fdtdrav.h:382-392); CPML x then y
        const Coef3 c = h_coef(p, 2, k == 0, n.m0, n.mk);
        float cy = c.bp, cx = c.bm;
        if (ys) cy = __fdiv_rn(c.bp, p.kmy[j]);
        if (xs) cx = __fdiv_rn(c.bm, p.kmx[i]);
        const float dEx = __fsub_rn(n.ex_jp, n.ex);
        const float dEy = __fsub_rn(n.ey_ip, n.ey);
        float v = upd3(c.a, n.hz, cy, dEx, cx, dEy);
        pre[2] = v;
        if (xs) {
            const long long q = psi_index_x(g, i, j, k, side);
            v = psi_step(ps.in[side].h[1], ps.out[side].h[1], q, ps.write, p.bmx[i], p.amx[i], dEy, v,
                         __fmul_rn(c.bm, g.dx));
        }
        if (ys) {
            const long long q = psi_index_y(g, i, j, k, side);
            v = psi_step(ps.in[2 + side].h[1], ps.out[2 + side].h[1], q, ps.write, p.bmy[j], p.amy[j], dEx, v,
                         __fmul_rn(c.bp, g.dy));
        }
        out[2] = v;
    }
}

}  // namespace fdtd
