// Two-pass schedule: an E pass then an H pass per time step, both in place, one thread per node.
//
// This is the reference's own order of work (calc_e then calc_h, solver fdtdrav.h:3222-3333)
// expressed over the compact data layout: coefficients rebuilt from the uint8 material index,
// CPML memory in face slabs, lumped elements and probes bucketed by plane. It runs at any grid
// size and is the schedule the fused sweep is checked against bit for bit.
#include "yee_common.cuh"
#include "yee_kernels.h"

namespace fdtd {

__global__ void __launch_bounds__(256) k_update_e(StepParams p, FieldPtrs f, PsiSet ps, long long m) {
    const DeviceGrid& g = p.g;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.nx || j >= g.ny) return;
    const bool ex_m = i < g.nx - 1 && j > 0 && j < g.ny - 1 && k > 0 && k < g.nz - 1;
    const bool ey_m = i > 0 && i < g.nx - 1 && j < g.ny - 1 && k > 0 && k < g.nz - 1;
    const bool ez_m = i > 0 && i < g.nx - 1 && j > 0 && j < g.ny - 1 && k < g.nz - 1;
    if (!(ex_m || ey_m || ez_m)) return;
    const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
    const long long P = g.plane, R = g.pitch;
    const long long row = m % p.ring_cap;
    const uint8_t* mat = p.mat;
    const int m0 = mat[n];
    const int mi = i > 0 ? mat[n - 1] : 0;
    const int mj = j > 0 ? mat[n - R] : 0;
    const int mk = k > 0 ? mat[n - P] : 0;
    const bool xs = in_slab(i, g.nx, g.pxn, g.pxp);
    const bool ys = in_slab(j, g.ny, g.pyn, g.pyp);
    const bool zs = in_slab(k, g.nz, g.pzn, g.pzp);
    int side;

    if (ex_m) {  // Ex (fdtdrav.h:665-676), CPML y then z (fdtdrav.h:790-808, 829-850)
        const Coef3 c = e_coef(p, 0, m0, mj, mk, mat[n - R - P]);
        float cy = c.bp, cz = c.bm, py = 0.f, pz = 0.f;
        if (ys) { py = __fmul_rn(c.bp, g.dy); cy = __fdiv_rn(c.bp, p.key[j]); }
        if (zs) { pz = __fmul_rn(c.bm, g.dz); cz = __fdiv_rn(c.bm, p.kez[k]); }
        const float dHz = __fsub_rn(f.hz[n], f.hz[n - R]);
        const float dHy = __fsub_rn(f.hy[n], f.hy[n - P]);
        float v = upd3(c.a, f.ex[n], cy, dHz, cz, dHy);
        if (p.probe_k[k] < p.probe_k[k + 1]) sample(p, row, 0, i, j, k, v);
        if (ys) {
            const long long q = psi_index_y(g, i, j, k, side);
            float* a = ps.f[2 + side].e[0];
            const float s = psi_upd(p.bey[j], a[q], p.aey[j], dHz);
            a[q] = s;
            v = psi_add(v, py, s);
        }
        if (zs) {
            const long long q = psi_index_z(g, i, j, k, side);
            float* a = ps.f[4 + side].e[0];
            const float s = psi_upd(p.bez[k], a[q], p.aez[k], dHy);
            a[q] = s;
            v = psi_add(v, pz, s);
        }
        f.ex[n] = v;
    }
    if (ey_m) {  // Ey (fdtdrav.h:696-707), CPML x then z
        const Coef3 c = e_coef(p, 1, m0, mi, mk, mat[n - 1 - P]);
        float cz = c.bp, cx = c.bm, pzv = 0.f, pxv = 0.f;
        if (zs) { pzv = __fmul_rn(c.bp, g.dz); cz = __fdiv_rn(c.bp, p.kez[k]); }
        if (xs) { pxv = __fmul_rn(c.bm, g.dx); cx = __fdiv_rn(c.bm, p.kex[i]); }
        const float dHx = __fsub_rn(f.hx[n], f.hx[n - P]);
        const float dHz = __fsub_rn(f.hz[n], f.hz[n - 1]);
        float v = upd3(c.a, f.ey[n], cz, dHx, cx, dHz);
        if (p.probe_k[k] < p.probe_k[k + 1]) sample(p, row, 1, i, j, k, v);
        if (xs) {
            const long long q = psi_index_x(g, i, j, k, side);
            float* a = ps.f[side].e[0];
            const float s = psi_upd(p.bex[i], a[q], p.aex[i], dHz);
            a[q] = s;
            v = psi_add(v, pxv, s);
        }
        if (zs) {
            const long long q = psi_index_z(g, i, j, k, side);
            float* a = ps.f[4 + side].e[1];
            const float s = psi_upd(p.bez[k], a[q], p.aez[k], dHx);
            a[q] = s;
            v = psi_add(v, pzv, s);
        }
        f.ey[n] = v;
    }
    if (ez_m) {  // Ez with lumped elements (fdtdrav.h:720-741), CPML x then y
        const Coef3 c = e_coef(p, 2, m0, mi, mj, mat[n - 1 - R]);
        float cx = c.bp, cy = c.bm, pxv = 0.f, pyv = 0.f;
        if (xs) { pxv = __fmul_rn(c.bp, g.dx); cx = __fdiv_rn(c.bp, p.kex[i]); }
        if (ys) { pyv = __fmul_rn(c.bm, g.dy); cy = __fdiv_rn(c.bm, p.key[j]); }
        const float dHy = __fsub_rn(f.hy[n], f.hy[n - 1]);
        const float dHx = __fsub_rn(f.hx[n], f.hx[n - R]);
        const float ez = f.ez[n];
        float v;
        const LumpedEdge* L = (p.lumped_k[k] < p.lumped_k[k + 1]) ? find_lumped(p, i, j, k) : nullptr;
        if (L) {
            if (L->source >= 0) {
                const float s = m < p.wave_len[L->source] ? p.waves[L->source][m] : 0.f;
                v = upd4(L->ceze, ez, L->cezhy, dHy, L->cezhx, dHx, L->cezj, s);
            } else {
                v = upd3(L->ceze, ez, L->cezhy, dHy, L->cezhx, dHx);
            }
        } else {
            v = upd3(c.a, ez, cx, dHy, cy, dHx);
        }
        if (p.probe_k[k] < p.probe_k[k + 1]) sample(p, row, 2, i, j, k, v);
        if (xs) {
            const long long q = psi_index_x(g, i, j, k, side);
            float* a = ps.f[side].e[1];
            const float s = psi_upd(p.bex[i], a[q], p.aex[i], dHy);
            a[q] = s;
            v = psi_add(v, pxv, s);
        }
        if (ys) {
            const long long q = psi_index_y(g, i, j, k, side);
            float* a = ps.f[2 + side].e[1];
            const float s = psi_upd(p.bey[j], a[q], p.aey[j], dHx);
            a[q] = s;
            v = psi_add(v, pyv, s);
        }
        f.ez[n] = v;
    }
}

__global__ void __launch_bounds__(256) k_update_h(StepParams p, FieldPtrs f, PsiSet ps, long long m) {
    const DeviceGrid& g = p.g;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.nx || j >= g.ny) return;
    const bool hx_m = j < g.ny - 1 && k < g.nz - 1;
    const bool hy_m = i < g.nx - 1 && k < g.nz - 1;
    const bool hz_m = i < g.nx - 1 && j < g.ny - 1;
    if (!(hx_m || hy_m || hz_m)) return;
    const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
    const long long P = g.plane, R = g.pitch;
    const long long row = m % p.ring_cap;
    const uint8_t* mat = p.mat;
    const int m0 = mat[n];
    const bool xs = in_slab(i, g.nx, g.pxn, g.pxp);
    const bool ys = in_slab(j, g.ny, g.pyn, g.pyp);
    const bool zs = in_slab(k, g.nz, g.pzn, g.pzp);
    int side;

    if (hx_m) {  // Hx (fdtdrav.h:328-348), CPML y then z (fdtdrav.h:445-486, 489-528)
        const Coef3 c = h_coef(p, 0, i == 0, m0, i > 0 ? mat[n - 1] : 0);
        float cz = c.bp, cy = c.bm, pzv = 0.f, pyv = 0.f;
        if (zs) { pzv = __fmul_rn(c.bp, g.dz); cz = __fdiv_rn(c.bp, p.kmz[k]); }
        if (ys) { pyv = __fmul_rn(c.bm, g.dy); cy = __fdiv_rn(c.bm, p.kmy[j]); }
        const float dEy = __fsub_rn(f.ey[n + P], f.ey[n]);
        const float dEz = __fsub_rn(f.ez[n + R], f.ez[n]);
        float v = upd3_hx(c.a, f.hx[n], cz, dEy, cy, dEz);
        if (p.probe_k[k] < p.probe_k[k + 1]) sample(p, row, 3, i, j, k, v);
        if (ys) {
            const long long q = psi_index_y(g, i, j, k, side);
            float* a = ps.f[2 + side].h[0];
            const float s = psi_upd(p.bmy[j], a[q], p.amy[j], dEz);
            a[q] = s;
            v = psi_add(v, pyv, s);
        }
        if (zs) {
            const long long q = psi_index_z(g, i, j, k, side);
            float* a = ps.f[4 + side].h[0];
            const float s = psi_upd(p.bmz[k], a[q], p.amz[k], dEy);
            a[q] = s;
            v = psi_add(v, pzv, s);
        }
        f.hx[n] = v;
    }
    if (hy_m) {  // Hy (fdtdrav.h:357-373), CPML x then z
        const Coef3 c = h_coef(p, 1, j == 0, m0, j > 0 ? mat[n - R] : 0);
        float cx = c.bp, cz = c.bm, pxv = 0.f, pzv = 0.f;
        if (xs) { pxv = __fmul_rn(c.bp, g.dx); cx = __fdiv_rn(c.bp, p.kmx[i]); }
        if (zs) { pzv = __fmul_rn(c.bm, g.dz); cz = __fdiv_rn(c.bm, p.kmz[k]); }
        const float dEz = __fsub_rn(f.ez[n + 1], f.ez[n]);
        const float dEx = __fsub_rn(f.ex[n + P], f.ex[n]);
        float v = upd3(c.a, f.hy[n], cx, dEz, cz, dEx);
        if (p.probe_k[k] < p.probe_k[k + 1]) sample(p, row, 4, i, j, k, v);
        if (xs) {
            const long long q = psi_index_x(g, i, j, k, side);
            float* a = ps.f[side].h[0];
            const float s = psi_upd(p.bmx[i], a[q], p.amx[i], dEz);
            a[q] = s;
            v = psi_add(v, pxv, s);
        }
        if (zs) {
            const long long q = psi_index_z(g, i, j, k, side);
            float* a = ps.f[4 + side].h[1];
            const float s = psi_upd(p.bmz[k], a[q], p.amz[k], dEx);
            a[q] = s;
            v = psi_add(v, pzv, s);
        }
        f.hy[n] = v;
    }
    if (hz_m) {  // Hz (fdtdrav.h:382-392), CPML x then y
        const Coef3 c = h_coef(p, 2, k == 0, m0, k > 0 ? mat[n - P] : 0);
        float cy = c.bp, cx = c.bm, pyv = 0.f, pxv = 0.f;
        if (ys) { pyv = __fmul_rn(c.bp, g.dy); cy = __fdiv_rn(c.bp, p.kmy[j]); }
        if (xs) { pxv = __fmul_rn(c.bm, g.dx); cx = __fdiv_rn(c.bm, p.kmx[i]); }
        const float dEx = __fsub_rn(f.ex[n + R], f.ex[n]);
        const float dEy = __fsub_rn(f.ey[n + 1], f.ey[n]);
        float v = upd3(c.a, f.hz[n], cy, dEx, cx, dEy);
        if (p.probe_k[k] < p.probe_k[k + 1]) sample(p, row, 5, i, j, k, v);
        if (xs) {
            const long long q = psi_index_x(g, i, j, k, side);
            float* a = ps.f[side].h[1];
            const float s = psi_upd(p.bmx[i], a[q], p.amx[i], dEy);
            a[q] = s;
            v = psi_add(v, pxv, s);
        }
        if (ys) {
            const long long q = psi_index_y(g, i, j, k, side);
            float* a = ps.f[2 + side].h[1];
            const float s = psi_upd(p.bmy[j], a[q], p.amy[j], dEx);
            a[q] = s;
            v = psi_add(v, pyv, s);
        }
        f.hz[n] = v;
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
