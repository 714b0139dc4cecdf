// Discrete adjoint of the Yee step (no reference counterpart; the reference has no gradient).
//
// The forward step is linear in the state (E, H, CPML memory psi): calc_e maps (E, H, psi_E) to
// (E', psi_E'), then calc_h maps (H, E', psi_H) to (H', psi_H'). The adjoint state lambda holds
// dJ/d(state); one reverse step applies the transposes in reverse order:
//   k_adj_h  (transpose of calc_h) and then
//   k_adj_e  (transpose of calc_e, plus the figure-of-merit source and the design gradient).
// The curl operators are transposed in gather form: each kernel writes, per node and component,
// the two contributions its derivative terms send to the other field (arrays G_H and G_E, zero for
// components the update masks keep fixed), and the next kernel gathers them from the neighbours.
// No atomics; each node owns its lambda and its CPML adjoint memory. The coefficients are rebuilt
// exactly as e_update / h_update build them (material table, edge averages, design cells, CPML
// kappa division, lumped overrides), so the adjoint is the transpose of the FP32 update.
//
// Figure of merit J = sum_m dt * Ez(p)^2 with Ez sampled after step m's E update: its derivative
// 2 dt Ez_p(m) enters lambda_Ez(p) at reverse step m. The gradient with respect to the eps_r of a
// design cell collects, over the steps and the twelve E edges around the cell, lambda_e *
// dE_e'/d(eps_avg) / 4, where for an edge update E' = a E + c1 d1 + c2 d2 with
// den = 2 eps_avg eps0 + dt sigma_avg:
//   da/deps = 4 eps0 dt sigma / den^2,  d(c1, c2)/deps = -(2 eps0 / den) (c1, c2),
// so dE'/deps = da/deps * E - (2 eps0 / den) * (E' - a E), from the saved design-region E of the
// step (edges of the design region carry no CPML term and no lumped element).
#include "yee_common.cuh"
#include "adjoint.h"

namespace fdtd {

namespace {

// One CPML term of an adjoint component: memory slot, profile values and psi coefficient.
struct PsiTerm {
    float* mem;  // adjoint psi entry, NULL when the node is outside the slab
    float b, a, cpsi;
    float old;   // its value before this step
};
// The term of adjoint psi entry `mem`, its old value read here: where the term is built, not
// where it is applied (3-4 % off the reverse step at 128^3).
__device__ __forceinline__ PsiTerm psi_term(float* mem, float b, float a, float cpsi) {
    return PsiTerm{mem, b, a, cpsi, *mem};
}

// Transpose of one component update v' = a v + c1 d1 + c2 d2 (+ psi terms t1 on d1, t2 on d2):
// returns the new lambda of the component and the contributions g1, g2 to the fields of d1, d2.
__device__ __forceinline__ float adj_comp(float L, float a, float c1, float c2, const PsiTerm& t1, const PsiTerm& t2,
                                          float& g1, float& g2) {
    g1 = c1 * L;
    g2 = c2 * L;
    if (t1.mem) {
        const float mm = __fmaf_rn(t1.cpsi, L, t1.old);
        *t1.mem = t1.b * mm;
        g1 = __fmaf_rn(t1.a, mm, g1);
    }
    if (t2.mem) {
        const float mm = __fmaf_rn(t2.cpsi, L, t2.old);
        *t2.mem = t2.b * mm;
        g2 = __fmaf_rn(t2.a, mm, g2);
    }
    return a * L;
}

__device__ __forceinline__ long long node(const DeviceGrid& g, int i, int j, int k) {
    return (long long)k * g.plane + (long long)j * g.pitch + i;
}

}  // namespace

// ---- transpose of calc_h (h_update) -------------------------------------------------------
// G_E slots (written by k_adj_e): 0 Ex->Hz, 1 Ex->Hy, 2 Ey->Hx, 3 Ey->Hz, 4 Ez->Hy, 5 Ez->Hx.
// G_H slots (written here):        0 Hx->Ey, 1 Hx->Ez, 2 Hy->Ez, 3 Hy->Ex, 4 Hz->Ex, 5 Hz->Ey.
// 5 CTAs of 256 per SM (48 registers; k_adj_e spills a few words): measured 14 % faster for the
// reverse sweep at 128^3 than the compiler's own 80 registers (3 CTAs).
#ifndef FDTD_ADJ_MIN_BLOCKS
#define FDTD_ADJ_MIN_BLOCKS 5
#endif
// General path of k_adj_h. kBg: a node of class kUniformGeneral + background (CPML slabs and
// boundary planes in the usual layouts): uniform cells and background tables decided at compile
// time, as in the forward's specialisation.
template <bool kBg>
__device__ __forceinline__ void adj_h_general(const StepParams& p, const AdjState& a, const PsiSet& psa, int i, int j,
                                              int k, long long n, int c, float lx, float ly, float lz) {
    const DeviceGrid& g = p.g;
    const long long P = g.plane, R = g.pitch;
    const bool kp = k < g.nz - 1, jp = j < g.ny - 1, ip = i < g.nx - 1;
    const uint8_t* mat = p.mat;
    const bool one = kBg || c < kInterfaceNode;  // seven cells of one material, given by the class
    const int m0 = kBg ? p.bg.mat : one ? c - kUniformGeneral : mat[n];
    const int mi = one ? m0 : i > 0 ? mat[n - 1] : 0, mj = one ? m0 : j > 0 ? mat[n - R] : 0;
    const int mk = one ? m0 : k > 0 ? mat[n - P] : 0;
    const bool hx_m = jp && kp, hy_m = ip && kp, hz_m = ip && jp;
    const bool xs = in_slab(i, g.nx, g.pxn, g.pxp), ys = in_slab(j, g.ny, g.pyn, g.pyp), zs = in_slab(k, g.nz, g.pzn, g.pzp);
    const int bg = p.bg.mat;
    const bool ux = kBg || m0 == mi, uy = kBg || m0 == mj, uz = kBg || m0 == mk;
    const bool on_bg = kBg || m0 == bg;
    const Coef3 cx = h_coef(p, 0, i == 0, ux, m0, mi);
    const Coef3 cy = h_coef(p, 1, j == 0, uy, m0, mj);
    const Coef3 cz = h_coef(p, 2, k == 0, uz, m0, mk);
    const bool bx = i != 0 && ux && on_bg, by = j != 0 && uy && on_bg, bz = k != 0 && uz && on_bg;
    const BgCurl& B = p.bg;
    int side;
    float g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f, g4 = 0.f, g5 = 0.f;
    if (hx_m) {  // Hx: c1 on dEy_k (z CPML), c2 on dEz_j (y CPML)
        PsiTerm t1{nullptr, 0, 0, 0, 0}, t2{nullptr, 0, 0, 0, 0};
        if (zs) { const int q = psi_off_z(g, i, j, k, side); t1 = psi_term(psa.f[4 + side].h[0] + q, p.bmz[k], p.amz[k], __fmul_rn(cx.bp, g.dz)); }
        if (ys) { const int q = psi_off_y(g, i, j, k, side); t2 = psi_term(psa.f[2 + side].h[0] + q, p.bmy[j], p.amy[j], __fmul_rn(cx.bm, g.dy)); }
        const float c1 = zs ? kdiv(cx.bp, bx, B.h[2][0], p.kmz, k) : cx.bp;
        const float c2 = ys ? kdiv(cx.bm, bx, B.h[1][0], p.kmy, j) : cx.bm;
        lx = adj_comp(lx, cx.a, c1, c2, t1, t2, g0, g1);
    }
    if (hy_m) {  // Hy: c1 on dEz_i (x CPML), c2 on dEx_k (z CPML)
        PsiTerm t1{nullptr, 0, 0, 0, 0}, t2{nullptr, 0, 0, 0, 0};
        if (xs) { const int q = psi_off_x(g, i, j, k, side); t1 = psi_term(psa.f[side].h[0] + q, p.bmx[i], p.amx[i], __fmul_rn(cy.bp, g.dx)); }
        if (zs) { const int q = psi_off_z(g, i, j, k, side); t2 = psi_term(psa.f[4 + side].h[1] + q, p.bmz[k], p.amz[k], __fmul_rn(cy.bm, g.dz)); }
        const float c1 = xs ? kdiv(cy.bp, by, B.h[0][0], p.kmx, i) : cy.bp;
        const float c2 = zs ? kdiv(cy.bm, by, B.h[2][1], p.kmz, k) : cy.bm;
        ly = adj_comp(ly, cy.a, c1, c2, t1, t2, g2, g3);
    }
    if (hz_m) {  // Hz: c1 on dEx_j (y CPML), c2 on dEy_i (x CPML)
        PsiTerm t1{nullptr, 0, 0, 0, 0}, t2{nullptr, 0, 0, 0, 0};
        if (ys) { const int q = psi_off_y(g, i, j, k, side); t1 = psi_term(psa.f[2 + side].h[1] + q, p.bmy[j], p.amy[j], __fmul_rn(cz.bp, g.dy)); }
        if (xs) { const int q = psi_off_x(g, i, j, k, side); t2 = psi_term(psa.f[side].h[1] + q, p.bmx[i], p.amx[i], __fmul_rn(cz.bm, g.dx)); }
        const float c1 = ys ? kdiv(cz.bp, bz, B.h[1][1], p.kmy, j) : cz.bp;
        const float c2 = xs ? kdiv(cz.bm, bz, B.h[0][1], p.kmx, i) : cz.bm;
        lz = adj_comp(lz, cz.a, c1, c2, t1, t2, g4, g5);
    }
    a.l[3][n] = lx; a.l[4][n] = ly; a.l[5][n] = lz;
    a.gh[0][n] = g0; a.gh[1][n] = g1; a.gh[2][n] = g2; a.gh[3][n] = g3; a.gh[4][n] = g4; a.gh[5][n] = g5;
}

__global__ void __launch_bounds__(256, FDTD_ADJ_MIN_BLOCKS) k_adj_h(const __grid_constant__ StepParams p, AdjState a,
                                               const __grid_constant__ PsiSet psa) {
    const DeviceGrid& g = p.g;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.nx || j >= g.ny) return;
    const long long n = node(g, i, j, k);
    const long long P = g.plane, R = g.pitch;
    const bool kp = k < g.nz - 1, jp = j < g.ny - 1, ip = i < g.nx - 1;
    // finish the transpose of the previous reverse step's calc_e: gather G_E
    float lx = a.l[3][n] + a.ge[2][n] - (kp ? a.ge[2][n + P] : 0.f) + a.ge[5][n] - (jp ? a.ge[5][n + R] : 0.f);
    float ly = a.l[4][n] + a.ge[1][n] - (kp ? a.ge[1][n + P] : 0.f) + a.ge[4][n] - (ip ? a.ge[4][n + 1] : 0.f);
    float lz = a.l[5][n] + a.ge[0][n] - (jp ? a.ge[0][n + R] : 0.f) + a.ge[3][n] - (ip ? a.ge[3][n + 1] : 0.f);

    const int c = p.cls[n];
    if (c < kUniformGeneral) {  // fast-path node: table coefficients, every component, no CPML
        const MatCoef* mc = p.coef + c;
        const float4 x = __ldg(&mc->h[0]), y = __ldg(&mc->h[1]), z = __ldg(&mc->h[2]);
        a.l[3][n] = x.x * lx; a.l[4][n] = y.x * ly; a.l[5][n] = z.x * lz;
        a.gh[0][n] = x.y * lx; a.gh[1][n] = x.z * lx; a.gh[2][n] = y.y * ly;
        a.gh[3][n] = y.z * ly; a.gh[4][n] = z.y * lz; a.gh[5][n] = z.z * lz;
        return;
    }
    if (c == kUniformGeneral + p.bg.mat) adj_h_general<true>(p, a, psa, i, j, k, n, c, lx, ly, lz);
    else adj_h_general<false>(p, a, psa, i, j, k, n, c, lx, ly, lz);
}

// ---- transpose of calc_e (e_update), FoM source and design gradient ------------------------
// General path of k_adj_e, specialised like adj_h_general (background nodes carry no lumped edge
// and lie outside the design edge box).
template <bool kBg>
__device__ __forceinline__ void adj_e_general(const StepParams& p, const AdjState& a, const PsiSet& psa,
                                              const AdjStep& st, int i, int j, int k, long long n, int c, float lx,
                                              float ly, float lz) {
    const DeviceGrid& g = p.g;
    const long long P = g.plane, R = g.pitch;
    const uint8_t* mat = p.mat;
    const bool one = kBg || c < kInterfaceNode;  // seven cells of one material, given by the class
    const int m0 = kBg ? p.bg.mat : one ? c - kUniformGeneral : mat[n];
    const int mi = one ? m0 : i > 0 ? mat[n - 1] : 0, mj = one ? m0 : j > 0 ? mat[n - R] : 0;
    const int mk = one ? m0 : k > 0 ? mat[n - P] : 0;
    const int mij = one ? m0 : (i > 0 && j > 0) ? mat[n - 1 - R] : 0;
    const int mik = one ? m0 : (i > 0 && k > 0) ? mat[n - 1 - P] : 0;
    const int mjk = one ? m0 : (j > 0 && k > 0) ? mat[n - R - P] : 0;
    const bool in_x = i > 0 && i < g.nx - 1, in_y = j > 0 && j < g.ny - 1, in_z = k > 0 && k < g.nz - 1;
    const bool ex_m = i < g.nx - 1 && in_y && in_z, ey_m = in_x && j < g.ny - 1 && in_z, ez_m = in_x && in_y && k < g.nz - 1;
    const bool xs = in_slab(i, g.nx, g.pxn, g.pxp), ys = in_slab(j, g.ny, g.pyn, g.pyp), zs = in_slab(k, g.nz, g.pzn, g.pzp);
    const int bg = p.bg.mat;
    const bool ux = kBg || (m0 == mj && m0 == mk && m0 == mjk);
    const bool uy = kBg || (m0 == mi && m0 == mk && m0 == mik);
    const bool uz = kBg || (m0 == mi && m0 == mj && m0 == mij);
    const bool on_bg = kBg || m0 == bg;
    const Coef3 cx = e_coef<!kBg>(p, 0, ux, m0, mj, mk, mjk, i, j, k);
    const Coef3 cy = e_coef<!kBg>(p, 1, uy, m0, mi, mk, mik, i, j, k);
    const Coef3 cz = e_coef<!kBg>(p, 2, uz, m0, mi, mj, mij, i, j, k);

    // design gradient: lambda here is dJ/dE^{m+1}; E^m and E^{m+1} come from the saved design E
    if (!kBg && st.acc) {  // background nodes lie outside the design edge box
        const int* d = p.dbox;
        const int ei = i - d[0], ej = j - d[1], ek = k - d[2];
        const int bx = d[3] - d[0] + 1, by = d[4] - d[1] + 1, bzz = d[5] - d[2] + 1;
        if (ei >= 0 && ej >= 0 && ek >= 0 && ei < bx && ej < by && ek < bzz) {
            const long long e = ((long long)ek * by + ej) * bx + ei, ne = (long long)bx * by * bzz;
            const float lam[3] = {lx, ly, lz};
            const Coef3 cc[3] = {cx, cy, cz};
            const bool on[3] = {ex_m, ey_m, ez_m};
            const int mm[3][4] = {{m0, mj, mk, mjk}, {m0, mi, mk, mik}, {m0, mi, mj, mij}};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (!on[c] || !has_design(p, mm[c][0], mm[c][1], mm[c][2], mm[c][3])) continue;
                float eps, sig;
                edge_material(p, c, i, j, k, mm[c][0], mm[c][1], mm[c][2], mm[c][3], eps, sig);
                const double e0 = g.eps0, dt = g.dt;
                const double den = 2.0 * (double)eps * e0 + dt * (double)sig;
                const double dca = 4.0 * e0 * dt * (double)sig / (den * den);
                const double em = st.e_old[c * ne + e], ep = st.e_new[c * ne + e];
                const double v = (double)lam[c] * (dca * em - 2.0 * e0 / den * (ep - (double)cc[c].a * em));
                st.acc[c * ne + e] += v;
            }
        }
    }

    const BgCurl& B = p.bg;
    int side;
    float g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f, g4 = 0.f, g5 = 0.f;
    if (ex_m) {  // Ex: c1 on dHz_j (y CPML), c2 on dHy_k (z CPML)
        PsiTerm t1{nullptr, 0, 0, 0, 0}, t2{nullptr, 0, 0, 0, 0};
        if (ys) { const int q = psi_off_y(g, i, j, k, side); t1 = psi_term(psa.f[2 + side].e[0] + q, p.bey[j], p.aey[j], __fmul_rn(cx.bp, g.dy)); }
        if (zs) { const int q = psi_off_z(g, i, j, k, side); t2 = psi_term(psa.f[4 + side].e[0] + q, p.bez[k], p.aez[k], __fmul_rn(cx.bm, g.dz)); }
        const float c1 = ys ? kdiv(cx.bp, ux && on_bg, B.e[1][0], p.key, j) : cx.bp;
        const float c2 = zs ? kdiv(cx.bm, ux && on_bg, B.e[2][0], p.kez, k) : cx.bm;
        lx = adj_comp(lx, cx.a, c1, c2, t1, t2, g0, g1);
    }
    if (ey_m) {  // Ey: c1 on dHx_k (z CPML), c2 on dHz_i (x CPML)
        PsiTerm t1{nullptr, 0, 0, 0, 0}, t2{nullptr, 0, 0, 0, 0};
        if (zs) { const int q = psi_off_z(g, i, j, k, side); t1 = psi_term(psa.f[4 + side].e[1] + q, p.bez[k], p.aez[k], __fmul_rn(cy.bp, g.dz)); }
        if (xs) { const int q = psi_off_x(g, i, j, k, side); t2 = psi_term(psa.f[side].e[0] + q, p.bex[i], p.aex[i], __fmul_rn(cy.bm, g.dx)); }
        const float c1 = zs ? kdiv(cy.bp, uy && on_bg, B.e[2][1], p.kez, k) : cy.bp;
        const float c2 = xs ? kdiv(cy.bm, uy && on_bg, B.e[0][0], p.kex, i) : cy.bm;
        ly = adj_comp(ly, cy.a, c1, c2, t1, t2, g2, g3);
    }
    if (ez_m) {  // Ez: c1 on dHy_i (x CPML), c2 on dHx_j (y CPML); lumped edges override a, c1, c2
        PsiTerm t1{nullptr, 0, 0, 0, 0}, t2{nullptr, 0, 0, 0, 0};
        if (xs) { const int q = psi_off_x(g, i, j, k, side); t1 = psi_term(psa.f[side].e[1] + q, p.bex[i], p.aex[i], __fmul_rn(cz.bp, g.dx)); }
        if (ys) { const int q = psi_off_y(g, i, j, k, side); t2 = psi_term(psa.f[2 + side].e[1] + q, p.bey[j], p.aey[j], __fmul_rn(cz.bm, g.dy)); }
        const bool plane_lumped = !kBg && p.lumped_k[k] < p.lumped_k[k + 1];  // background nodes carry none
        const LumpedEdge* L = plane_lumped ? find_lumped(p, i, j, k, 2) : nullptr;  // design handles have no Ex edges
        float aa, c1, c2;
        if (L) { aa = L->ceze; c1 = L->cezhy; c2 = L->cezhx; }
        else {
            aa = cz.a;
            c1 = xs ? kdiv(cz.bp, uz && on_bg, B.e[0][1], p.kex, i) : cz.bp;
            c2 = ys ? kdiv(cz.bm, uz && on_bg, B.e[1][1], p.key, j) : cz.bm;
        }
        lz = adj_comp(lz, aa, c1, c2, t1, t2, g4, g5);
    }
    a.l[0][n] = lx; a.l[1][n] = ly; a.l[2][n] = lz;
    a.ge[0][n] = g0; a.ge[1][n] = g1; a.ge[2][n] = g2; a.ge[3][n] = g3; a.ge[4][n] = g4; a.ge[5][n] = g5;
}

__global__ void __launch_bounds__(256, FDTD_ADJ_MIN_BLOCKS) k_adj_e(const __grid_constant__ StepParams p, AdjState a,
                                               const __grid_constant__ PsiSet psa, AdjStep st) {
    const DeviceGrid& g = p.g;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.nx || j >= g.ny) return;
    const long long n = node(g, i, j, k);
    const long long P = g.plane, R = g.pitch;
    // finish the transpose of calc_h: gather G_H
    float lx = a.l[0][n] + (k > 0 ? a.gh[3][n - P] : 0.f) - a.gh[3][n] + (j > 0 ? a.gh[4][n - R] : 0.f) - a.gh[4][n];
    float ly = a.l[1][n] + (k > 0 ? a.gh[0][n - P] : 0.f) - a.gh[0][n] + (i > 0 ? a.gh[5][n - 1] : 0.f) - a.gh[5][n];
    float lz = a.l[2][n] + (j > 0 ? a.gh[1][n - R] : 0.f) - a.gh[1][n] + (i > 0 ? a.gh[2][n - 1] : 0.f) - a.gh[2][n];
    if (n == st.probe) lz += st.source;  // dJ/dEz(p) of the sample taken in this step

    const int c = p.cls[n];
    if (c < kUniformGeneral) {  // fast-path node: table coefficients, every component, no CPML,
                                // no lumped edge, outside the design edge box
        const MatCoef* mc = p.coef + c;
        const float4 x = __ldg(&mc->e[0]), y = __ldg(&mc->e[1]), z = __ldg(&mc->e[2]);
        a.l[0][n] = x.x * lx; a.l[1][n] = y.x * ly; a.l[2][n] = z.x * lz;
        a.ge[0][n] = x.y * lx; a.ge[1][n] = x.z * lx; a.ge[2][n] = y.y * ly;
        a.ge[3][n] = y.z * ly; a.ge[4][n] = z.y * lz; a.ge[5][n] = z.z * lz;
        return;
    }
    if (c == kUniformGeneral + p.bg.mat) adj_e_general<true>(p, a, psa, st, i, j, k, n, c, lx, ly, lz);
    else adj_e_general<false>(p, a, psa, st, i, j, k, n, c, lx, ly, lz);
}

// After a forward step: the FoM sample Ez(p) and, when `snap` is set, the E components over the
// design edge box [d0, d3] x [d1, d4] x [d2, d5] (three arrays of the box volume).
__global__ void k_after_step(const float* ex, const float* ey, const float* ez, DeviceGrid g, long long probe,
                             float* sample, int d0, int d1, int d2, int bx, int by, int bz, float* snap) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q == 0 && sample) *sample = ez[probe];
    if (!snap) return;
    const long long ne = (long long)bx * by * bz;
    if (q >= ne) return;
    const int ei = (int)(q % bx), ej = (int)((q / bx) % by), ek = (int)(q / ((long long)bx * by));
    const int i = d0 + ei, j = d1 + ej, k = d2 + ek;
    if (i >= g.nx || j >= g.ny || k >= g.nz) { snap[q] = 0.f; snap[ne + q] = 0.f; snap[2 * ne + q] = 0.f; return; }
    const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
    snap[q] = ex[n];
    snap[ne + q] = ey[n];
    snap[2 * ne + q] = ez[n];
}

// dJ/deps_r of each design cell: a quarter of the accumulated edge terms of its twelve E edges.
__global__ void k_grad_finalize(const double* acc, int dx, int dy, int dz, double* grad) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)dx * dy * dz) return;
    const int ci = (int)(q % dx), cj = (int)((q / dx) % dy), ck = (int)(q / ((long long)dx * dy));
    const int bx = dx + 1, by = dy + 1, bz = dz + 1;
    const long long ne = (long long)bx * by * bz;
    auto at = [&](int c, int i, int j, int k) { return acc[c * ne + ((long long)k * by + j) * bx + i]; };
    double s = 0.0;
    // Ex edges (ci, cj..cj+1, ck..ck+1); Ey edges (ci..ci+1, cj, ck..ck+1); Ez (ci..ci+1, cj..cj+1, ck)
    for (int b = 0; b < 2; ++b)
        for (int c = 0; c < 2; ++c) {
            s += at(0, ci, cj + b, ck + c);
            s += at(1, ci + b, cj, ck + c);
            s += at(2, ci + b, cj + c, ck);
        }
    grad[q] = 0.25 * s;
}

cudaError_t launch_adj_step(const StepParams& p, const AdjState& a, const PsiSet& psa, const AdjStep& st,
                            cudaStream_t s) {
    dim3 block(32, 8, 1);
    dim3 grid((p.g.nx + 31) / 32, (p.g.ny + 7) / 8, p.g.nz);
    k_adj_h<<<grid, block, 0, s>>>(p, a, psa);
    k_adj_e<<<grid, block, 0, s>>>(p, a, psa, st);
    return cudaGetLastError();
}

cudaError_t launch_after_step(const float* ex, const float* ey, const float* ez, const DeviceGrid& g, long long probe,
                              float* sample, const int dbox[6], float* snap, cudaStream_t s) {
    const int bx = dbox[3] - dbox[0] + 1, by = dbox[4] - dbox[1] + 1, bz = dbox[5] - dbox[2] + 1;
    const long long ne = snap ? (long long)bx * by * bz : 1;
    k_after_step<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(ex, ey, ez, g, probe, sample, dbox[0], dbox[1], dbox[2],
                                                             bx, by, bz, snap);
    return cudaGetLastError();
}

// The six field components over node box b, to (save) or from a packed buffer of 6 x box volume
// floats (component-major, x fastest).
__global__ void k_box_state(FieldPtrs f, DeviceGrid g, NodeBox b, float* buf, bool save) {
    const int bx = b.x1 - b.x0, by = b.y1 - b.y0;
    const long long nb = (long long)bx * by * (b.z1 - b.z0);
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= nb) return;
    const int i = b.x0 + (int)(q % bx), j = b.y0 + (int)((q / bx) % by), k = b.z0 + (int)(q / ((long long)bx * by));
    const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
    float* c[6] = {f.ex, f.ey, f.ez, f.hx, f.hy, f.hz};
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        if (save) buf[r * nb + q] = c[r][n];
        else c[r][n] = buf[r * nb + q];
    }
}

cudaError_t launch_box_state(const FieldPtrs& f, const DeviceGrid& g, const NodeBox& b, float* buf, bool save,
                             cudaStream_t s) {
    if (b.x0 < 0 || b.y0 < 0 || b.z0 < 0 || b.x1 > g.nx || b.y1 > g.ny || b.z1 > g.nz) return cudaErrorInvalidValue;
    const long long nb = (long long)(b.x1 - b.x0) * (b.y1 - b.y0) * (b.z1 - b.z0);
    if (nb <= 0) return cudaSuccess;
    k_box_state<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(f, g, b, buf, save);
    return cudaGetLastError();
}

cudaError_t launch_grad_finalize(const double* acc, const int dbox[6], double* grad, cudaStream_t s) {
    const int dx = dbox[3] - dbox[0], dy = dbox[4] - dbox[1], dz = dbox[5] - dbox[2];
    const long long n = (long long)dx * dy * dz;
    k_grad_finalize<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(acc, dx, dy, dz, grad);
    return cudaGetLastError();
}

}  // namespace fdtd
