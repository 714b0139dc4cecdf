// Fused schedule: one z-marching sweep per time step over ping-pong field buffers.
//
// A work item is a 32 x 8 column of nodes and a range of planes [k0, k1). Planes stream through a
// 5-stage shared-memory ring filled by TMA (cp.async.bulk.tensor, 3-D tiles from this GPU's HBM,
// two planes ahead of the one being computed). At plane k the CTA
//   1. computes E(k) on the tile plus one column / row beyond its high x / y edges (the H update of
//      the tile needs those E values; the extra ones are recomputed from the old fields instead of
//      being exchanged), storing only the tile's own nodes;
//   2. computes H(k-1) of its own nodes from E(k-1), E(k) (shared memory) and H(k-1) (the ring).
// Old fields and old CPML memory are read from buffer A, new ones written to buffer B, so any
// partition of the grid into items is valid and CTAs never see each other's partial results. Each
// field value crosses HBM once per step in each direction: 24 B read + 24 B written per cell, plus
// the uint8 material index and the CPML memory.
//
// Two instantiations split the items: the interior kernel covers items whose every node is away
// from the grid boundary and the CPML slabs (table coefficients, an out-of-line call at material
// interfaces, the lumped-source override); the general kernel covers the rest with e_update /
// h_update. Keeping the general code out of the interior kernel halves the interior kernel's
// registers and instruction footprint. Both use the arithmetic of yee_common.cuh, so the result is
// bit-identical to the two-pass schedule. All waits on the TMA barriers are bounded: on timeout
// the kernel records an error in the status word, drains its own copies (again bounded) and exits.
#include <cuda.h>

#include "yee_common.cuh"
#include "yee_kernels.h"

namespace fdtd {

namespace {

constexpr int TX = 32, TY = 8;              // tile of nodes owned by a CTA
constexpr int NTH = TX * TY;                // one thread per owned node
constexpr int NSTAGE = 5;                   // planes resident in the ring
constexpr int AHEAD = 2;                    // planes loaded ahead of the one computed (<= NSTAGE - 3)
constexpr int HW = TX + 8, HH = TY + 2;     // H tile: x in [x0-4, x0+TX+4), y in [y0-1, y0+TY+1)
constexpr int EW = TX + 4, EH = TY + 1;     // old-E tile: x in [x0, x0+TX+4), y in [y0, y0+TY+1)
constexpr int MW = TX + 32, MH = TY + 2;    // material tile: x in [x0-16, x0+TX+16), y in [y0-1, ...)
constexpr int NW = TX + 1, NH = TY + 1;     // new-E plane: x in [x0, x0+TX], y in [y0, y0+TY]

constexpr int round128(int b) { return (b + 127) / 128 * 128; }
constexpr int H_BYTES = round128(HW * HH * 4);
constexpr int E_BYTES = round128(EW * EH * 4);
constexpr int M_BYTES = round128(MW * MH);
constexpr int STAGE_BYTES = 3 * H_BYTES + 3 * E_BYTES + M_BYTES;
constexpr unsigned TX_BYTES = 3u * HW * HH * 4 + 3u * EW * EH * 4 + MW * MH;  // bytes the TMA boxes carry
constexpr int N_FLOATS = NW * NH;
constexpr int ENEW_BYTES = 2 * 3 * N_FLOATS * 4;
constexpr int SMEM_BYTES = NSTAGE * STAGE_BYTES + ENEW_BYTES + NSTAGE * 8;
constexpr int NWARP = NTH / 32, NHALO = N_FLOATS - NTH;

constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for a barrier phase; false after kWaitCycles.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > kWaitCycles) return false;
    return true;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(saddr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(saddr(bar))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Arrays of one ring stage: H tile (3), old-E tile (3), material tile, at fixed offsets.
struct StageView {
    const unsigned char* base;
    __device__ explicit StageView(const unsigned char* b) : base(b) {}
    __device__ const float* h(int c) const { return reinterpret_cast<const float*>(base + c * H_BYTES); }
    __device__ const float* e(int c) const { return reinterpret_cast<const float*>(base + 3 * H_BYTES + c * E_BYTES); }
    __device__ const uint8_t* m() const { return base + 3 * H_BYTES + 3 * E_BYTES; }
};

// E update of an interior node (all three components updated, no CPML) with the lumped override.
__device__ __forceinline__ void e_interior(const StepParams& p, const ENbr& n, int i, int j, int k, long long m,
                                           bool plane_lumped, float out[3]) {
    const DeviceGrid& g = p.g;
    const float dHz_j = __fsub_rn(n.hz, n.hz_jm), dHy_k = __fsub_rn(n.hy, n.hy_km);
    const float dHx_k = __fsub_rn(n.hx, n.hx_km), dHz_i = __fsub_rn(n.hz, n.hz_im);
    const float dHy_i = __fsub_rn(n.hy, n.hy_im), dHx_j = __fsub_rn(n.hx, n.hx_jm);
    const MatCoef* mc = p.coef + n.m0;
    Coef3 cx, cy, cz;
    if (n.m0 == n.mj && n.m0 == n.mk && n.m0 == n.mjk) { const float4 c = __ldg(&mc->e[0]); cx = Coef3{c.x, c.y, c.z}; }
    else cx = e_coef_mixed(p.props, n.m0, n.mj, n.mk, n.mjk, g.dt, g.eps0, g.dy, g.dz);
    if (n.m0 == n.mi && n.m0 == n.mk && n.m0 == n.mik) { const float4 c = __ldg(&mc->e[1]); cy = Coef3{c.x, c.y, c.z}; }
    else cy = e_coef_mixed(p.props, n.m0, n.mi, n.mk, n.mik, g.dt, g.eps0, g.dz, g.dx);
    if (n.m0 == n.mi && n.m0 == n.mj && n.m0 == n.mij) { const float4 c = __ldg(&mc->e[2]); cz = Coef3{c.x, c.y, c.z}; }
    else cz = e_coef_mixed(p.props, n.m0, n.mi, n.mj, n.mij, g.dt, g.eps0, g.dx, g.dy);
    out[0] = upd3(cx.a, n.ex, cx.bp, dHz_j, cx.bm, dHy_k);
    out[1] = upd3(cy.a, n.ey, cy.bp, dHx_k, cy.bm, dHz_i);
    const LumpedEdge* L = plane_lumped ? find_lumped(p, i, j, k) : nullptr;
    if (L) {
        if (L->source >= 0) {
            const float s = m < p.wave_len[L->source] ? p.waves[L->source][m] : 0.f;
            out[2] = upd4(L->ceze, n.ez, L->cezhy, dHy_i, L->cezhx, dHx_j, L->cezj, s);
        } else {
            out[2] = upd3(L->ceze, n.ez, L->cezhy, dHy_i, L->cezhx, dHx_j);
        }
    } else {
        out[2] = upd3(cz.a, n.ez, cz.bp, dHy_i, cz.bm, dHx_j);
    }
}

// H update of an interior node (no reference-default faces, no CPML).
__device__ __forceinline__ void h_interior(const StepParams& p, const HNbr& n, float out[3]) {
    const DeviceGrid& g = p.g;
    const MatCoef* mc = p.coef + n.m0;
    Coef3 cx, cy, cz;
    if (n.m0 == n.mi) { const float4 c = __ldg(&mc->h[0]); cx = Coef3{c.x, c.y, c.z}; }
    else cx = h_coef_mixed(p.props, n.m0, n.mi, g.dt, g.mu0, g.dz, g.dy);
    if (n.m0 == n.mj) { const float4 c = __ldg(&mc->h[1]); cy = Coef3{c.x, c.y, c.z}; }
    else cy = h_coef_mixed(p.props, n.m0, n.mj, g.dt, g.mu0, g.dx, g.dz);
    if (n.m0 == n.mk) { const float4 c = __ldg(&mc->h[2]); cz = Coef3{c.x, c.y, c.z}; }
    else cz = h_coef_mixed(p.props, n.m0, n.mk, g.dt, g.mu0, g.dy, g.dx);
    out[0] = upd3_hx(cx.a, n.hx, cx.bp, __fsub_rn(n.ey_kp, n.ey), cx.bm, __fsub_rn(n.ez_jp, n.ez));
    out[1] = upd3(cy.a, n.hy, cy.bp, __fsub_rn(n.ez_ip, n.ez), cy.bm, __fsub_rn(n.ex_kp, n.ex));
    out[2] = upd3(cz.a, n.hz, cz.bp, __fsub_rn(n.ex_jp, n.ex), cz.bm, __fsub_rn(n.ey_ip, n.ey));
}

}  // namespace

// One sweep over the items of `items` (int4 {x0, y0, k0, k1}, one per CTA). INTERIOR selects the
// interior instantiation (all nodes of its items are interior by construction of the list).
template <bool INTERIOR>
__global__ void __launch_bounds__(NTH, 4)
k_fused(const __grid_constant__ FusedMaps maps, const __grid_constant__ StepParams p, FieldPtrs fo,
        const __grid_constant__ PsiSet psi_in, const __grid_constant__ PsiSet psi_out,
        const int4* __restrict__ items, long long m) {
    extern __shared__ __align__(128) unsigned char smem[];
    float* enew = reinterpret_cast<float*>(smem + NSTAGE * STAGE_BYTES);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + NSTAGE * STAGE_BYTES + ENEW_BYTES);
    const DeviceGrid& g = p.g;
    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int4 it = items[blockIdx.x];
    const int x0 = it.x, y0 = it.y, k0 = it.z, k1 = it.w;
    const int kfirst = k0 - 1, klast = k1;  // planes streamed through the ring
    const long long row = m % p.ring_cap;

    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    auto issue = [&](int k, int s) {
        unsigned char* st = smem + s * STAGE_BYTES;
        mbar_expect_tx(&bars[s], TX_BYTES);
        for (int c = 0; c < 3; ++c) tma_load_3d(st + c * H_BYTES, &maps.h[c], &bars[s], x0 - 4, y0 - 1, k);
        for (int c = 0; c < 3; ++c) tma_load_3d(st + 3 * H_BYTES + c * E_BYTES, &maps.e[c], &bars[s], x0, y0, k);
        tma_load_3d(st + 3 * H_BYTES + 3 * E_BYTES, &maps.mat, &bars[s], x0 - 16, y0 - 1, k);
    };
    // stage of plane k is (k - kfirst) % NSTAGE: kept as rotating counters
    if (tid == 0)
        for (int q = 0; q < AHEAD && kfirst + q <= klast; ++q) issue(kfirst + q, q);

    const PsiIO io_core{psi_in.f, psi_out.f, true};
    const PsiIO io_halo{psi_in.f, psi_out.f, false};
    int s_cur = 0, s_prv = NSTAGE - 1, s_pp = NSTAGE - 2, s_next = AHEAD % NSTAGE;
    uint32_t parity = 0;

    for (int k = kfirst; k <= klast; ++k) {
        if (tid == 0 && k + AHEAD <= klast) {
            fence_proxy_async();  // generic reads of the recycled stage precede the async writes
            issue(k + AHEAD, s_next);
        }
        const bool ok = mbar_wait(&bars[s_cur], parity);
        const StageView cur(smem + s_cur * STAGE_BYTES);
        const StageView prv(smem + s_prv * STAGE_BYTES);
        float* en_cur = enew + (k & 1) * 3 * N_FLOATS;
        const float* en_prv = enew + ((k - 1) & 1) * 3 * N_FLOATS;

        // ---- E(k) on the tile and its high-x column / high-y row ----
        if (k >= k0 && k < g.nz) {
            const bool store = k < k1;
            const bool plane_lumped = p.lumped_k[k] < p.lumped_k[k + 1];
            const bool plane_probe = p.probe_k[k] < p.probe_k[k + 1];
            // pass 0: the thread's own node; pass 1: one of the TX + TY + 1 halo positions, dealt
            // round-robin over the warps (halo h -> lane h / NWARP of warp h % NWARP)
            for (int pass = 0; pass < 2; ++pass) {
                int px, py;
                if (pass == 0) { px = tx; py = ty; }
                else {
                    const int h = (tid % 32) * NWARP + tid / 32;
                    if (h >= NHALO) break;
                    if (h < TY + 1) { px = TX; py = h; } else { px = h - (TY + 1); py = TY; }
                }
                const int i = x0 + px, j = y0 + py;
                if (i >= g.nx || j >= g.ny) continue;
                const int hi = (py + 1) * HW + px + 4;   // (i, j) in the H tile
                const int ei = py * EW + px;             // (i, j) in the old-E tile
                const int mi = (py + 1) * MW + px + 16;  // cell (i, j) in the material tile
                ENbr nb;
                nb.ex = cur.e(0)[ei]; nb.ey = cur.e(1)[ei]; nb.ez = cur.e(2)[ei];
                nb.hx = cur.h(0)[hi]; nb.hy = cur.h(1)[hi]; nb.hz = cur.h(2)[hi];
                nb.hx_jm = cur.h(0)[hi - HW]; nb.hx_km = prv.h(0)[hi];
                nb.hy_im = cur.h(1)[hi - 1]; nb.hy_km = prv.h(1)[hi];
                nb.hz_im = cur.h(2)[hi - 1]; nb.hz_jm = cur.h(2)[hi - HW];
                nb.m0 = cur.m()[mi]; nb.mi = cur.m()[mi - 1]; nb.mj = cur.m()[mi - MW]; nb.mij = cur.m()[mi - MW - 1];
                nb.mk = prv.m()[mi]; nb.mik = prv.m()[mi - 1]; nb.mjk = prv.m()[mi - MW];
                const bool own = store && pass == 0;
                float out[3], pre[3];
                if (INTERIOR) {
                    e_interior(p, nb, i, j, k, m, plane_lumped, out);
                    pre[0] = out[0]; pre[1] = out[1]; pre[2] = out[2];
                } else {
                    e_update(p, nb, i, j, k, m, plane_lumped, own ? io_core : io_halo, out, pre);
                }
                const int ni = py * NW + px;
                en_cur[ni] = out[0]; en_cur[N_FLOATS + ni] = out[1]; en_cur[2 * N_FLOATS + ni] = out[2];
                if (own) {
                    const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
                    fo.ex[n] = out[0]; fo.ey[n] = out[1]; fo.ez[n] = out[2];
                    if (plane_probe)
                        for (int c = 0; c < 3; ++c) sample(p, row, c, i, j, k, pre[c]);
                }
            }
        }

        // ---- H(k-1) on the tile ----
        const int kh = k - 1;
        if (kh >= k0 && kh < k1) {
            const int i = x0 + tx, j = y0 + ty;
            if (i < g.nx && j < g.ny) {
                const StageView mst(smem + s_pp * STAGE_BYTES);  // plane kh - 1
                const int hi = (ty + 1) * HW + tx + 4;
                const int mi = (ty + 1) * MW + tx + 16;
                const int ni = ty * NW + tx;
                HNbr nb;
                nb.hx = prv.h(0)[hi]; nb.hy = prv.h(1)[hi]; nb.hz = prv.h(2)[hi];
                nb.ex = en_prv[ni]; nb.ey = en_prv[N_FLOATS + ni]; nb.ez = en_prv[2 * N_FLOATS + ni];
                nb.ey_kp = en_cur[N_FLOATS + ni];
                nb.ex_kp = en_cur[ni];
                nb.ez_jp = en_prv[2 * N_FLOATS + ni + NW];
                nb.ex_jp = en_prv[ni + NW];
                nb.ez_ip = en_prv[2 * N_FLOATS + ni + 1];
                nb.ey_ip = en_prv[N_FLOATS + ni + 1];
                nb.m0 = prv.m()[mi]; nb.mi = prv.m()[mi - 1]; nb.mj = prv.m()[mi - MW]; nb.mk = mst.m()[mi];
                float out[3], pre[3];
                if (INTERIOR) {
                    h_interior(p, nb, out);
                    pre[0] = out[0]; pre[1] = out[1]; pre[2] = out[2];
                } else {
                    h_update(p, nb, i, j, kh, io_core, out, pre);
                }
                const long long n = (long long)kh * g.plane + (long long)j * g.pitch + i;
                fo.hx[n] = out[0]; fo.hy[n] = out[1]; fo.hz[n] = out[2];
                if (p.probe_k[kh] < p.probe_k[kh + 1])
                    for (int c = 0; c < 3; ++c) sample(p, row, 3 + c, i, j, kh, pre[c]);
            }
        }

        if (__syncthreads_or(!ok)) {
            // A plane never arrived: record it, wait (bounded) for the copies still in flight, exit.
            if (tid == 0) {
                atomic_flag(p.status, 1);
                int s = s_cur;
                uint32_t par = parity;
                for (int q = k + 1; q <= min(klast, k + AHEAD); ++q) {
                    if (++s == NSTAGE) { s = 0; par ^= 1u; }
                    mbar_wait(&bars[s], par);
                }
            }
            __syncthreads();
            return;
        }
        // rotate the ring counters
        s_pp = s_prv; s_prv = s_cur;
        if (++s_cur == NSTAGE) { s_cur = 0; parity ^= 1u; }
        if (++s_next == NSTAGE) s_next = 0;
    }
}

int fused_smem_bytes() { return SMEM_BYTES; }
int fused_tile_x() { return TX; }
int fused_tile_y() { return TY; }

cudaError_t fused_configure() {
    cudaError_t e = cudaFuncSetAttribute(k_fused<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_fused<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
}

cudaError_t launch_fused(const FusedMaps& maps, const StepParams& p, const FieldPtrs& fo, const PsiSet& psi_in,
                         const PsiSet& psi_out, long long m, const FusedWork& w, cudaStream_t st) {
    if (w.n_interior > 0)
        k_fused<true><<<w.n_interior, NTH, SMEM_BYTES, st>>>(maps, p, fo, psi_in, psi_out, w.interior, m);
    if (w.n_general > 0)
        k_fused<false><<<w.n_general, NTH, SMEM_BYTES, st>>>(maps, p, fo, psi_in, psi_out, w.general, m);
    return cudaGetLastError();
}

// Tensor maps of the buffers a sweep reads: H tiles with a one-node halo (x widened to 16-byte
// boundaries), old-E tiles, material tiles. Coordinates outside the arrays load as zeros.
int encode_fused_maps(FusedMaps* out, const DeviceGrid& g, float* const h[3], float* const e[3], const uint8_t* mat,
                      void* encode_fn) {
    auto encode = reinterpret_cast<CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                                CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                                CUtensorMapFloatOOBfill)>(encode_fn);
    const cuuint64_t dims[3] = {(cuuint64_t)g.pitch, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    const cuuint64_t fstr[2] = {(cuuint64_t)g.pitch * 4, (cuuint64_t)g.plane * 4};
    const cuuint64_t mstr[2] = {(cuuint64_t)g.pitch, (cuuint64_t)g.plane};
    const cuuint32_t hbox[3] = {HW, HH, 1}, ebox[3] = {EW, EH, 1}, mbox[3] = {MW, MH, 1}, es[3] = {1, 1, 1};
    for (int c = 0; c < 3; ++c) {
        if (encode(&out->h[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, h[c], dims, fstr, hbox, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return -1;
        if (encode(&out->e[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, e[c], dims, fstr, ebox, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return -1;
    }
    if (encode(&out->mat, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, (void*)mat, dims, mstr, mbox, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return -1;
    return 0;
}

// Split the grid into items: tiles whose E positions (x0..x0+TX, y0..y0+TY) lie in the x / y
// interior get their interior planes as interior items (chunks of at most kc planes); everything
// else (boundary / CPML tiles, and the z-boundary and z-CPML planes of interior tiles) becomes
// general items. The E positions of plane k1 of an item are recomputed, so a chunk must also keep
// its top plane in the interior range to stay interior.
void plan_fused(const DeviceGrid& g, int kc, std::vector<int4>& interior_items, std::vector<int4>& general_items) {
    interior_items.clear();
    general_items.clear();
    auto inside = [](int q, int n, int pn, int pp) {
        const int lo = pn > 1 ? pn : 1, hi = (n - 1 - pp < n - 2) ? n - 1 - pp : n - 2;
        return q >= lo && q <= hi;
    };
    const int zlo = g.pzn > 1 ? g.pzn : 1;
    const int zhi = (g.nz - 1 - g.pzp < g.nz - 2) ? g.nz - 1 - g.pzp : g.nz - 2;  // last interior plane
    auto chunks = [&](std::vector<int4>& out, int x0, int y0, int a, int b) {  // planes [a, b)
        for (int k = a; k < b; k += kc) out.push_back(make_int4(x0, y0, k, k + kc < b ? k + kc : b));
    };
    for (int y0 = 0; y0 < g.ny; y0 += TY)
        for (int x0 = 0; x0 < g.nx; x0 += TX) {
            const bool tile_int = inside(x0, g.nx, g.pxn, g.pxp) && inside(x0 + TX, g.nx, g.pxn, g.pxp) &&
                                  inside(y0, g.ny, g.pyn, g.pyp) && inside(y0 + TY, g.ny, g.pyn, g.pyp);
            // interior items cover planes [zlo, zhi) so that the recomputed top plane <= zhi
            if (tile_int && zhi > zlo) {
                chunks(general_items, x0, y0, 0, zlo);
                chunks(interior_items, x0, y0, zlo, zhi);
                chunks(general_items, x0, y0, zhi, g.nz);
            } else {
                chunks(general_items, x0, y0, 0, g.nz);
            }
        }
}

}  // namespace fdtd
