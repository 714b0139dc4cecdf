// Fused schedule: per time step, one z-marching sweep over the interior plus two passes over the
// shell (CPML slabs, boundary planes, strips beside the interior tiles), all reading buffer A and
// writing buffer B.
//
// Interior sweep. A work item is a 32 x 16 column of nodes and a plane range [k0, k1) inside the
// interior (no CPML, no boundary planes). Planes stream through a 3-stage shared-memory ring
// filled by TMA (cp.async.bulk.tensor, 3-D tiles of this GPU's HBM, one plane ahead of the one
// computed): H with a one-node halo, old E, and the coefficient row of each node (16 bits:
// StepParams::rec). At plane k the CTA
//   1. computes E(k) on its tile plus one column / row beyond the high x / y edges (the H update
//      needs those E values; they are recomputed from the old fields instead of being exchanged),
//      storing only its own nodes;
//   2. computes H(k-1) of its own nodes from E(k-1), E(k) (shared memory) and H(k-1) (the ring).
// Each thread owns two nodes of a plane (rows ty and ty + 8), which gives every warp two
// independent update chains and halves the per-plane overhead per node. Each field value crosses
// HBM once per step in each direction (24 B read + 24 B written per cell) plus the 2-byte row.
// Fast-path and interface nodes update from their coefficient row; the other nodes (lumped
// edges, plates) leave the fast path through an out-of-line call. The shell passes
// (yee_two_pass.cu) run before (E) and after (H) the sweep, one node per thread. A z-marching
// sweep over the CPML tiles with the recurrences inside measured two to five times slower per node
// than those passes (its general path's dependent load chains sit behind a per-plane barrier).
// All schedules use the arithmetic of yee_common.cuh, so the results are bit-identical. Every
// wait on a TMA barrier is bounded: on timeout the kernel records an error in the status word,
// drains its own copies (again bounded) and exits.
#include <cuda.h>

#include <algorithm>

#include "planner.h"
#include "yee_common.cuh"
#include "yee_kernels.h"

namespace fdtd {

namespace {

constexpr int NTH = 256;                    // threads per CTA
#ifndef FDTD_FUSED_NSTAGE
#define FDTD_FUSED_NSTAGE 3
#endif
#ifndef FDTD_FUSED_AHEAD
#define FDTD_FUSED_AHEAD 1
#endif
#ifndef FDTD_FUSED_MIN_BLOCKS
#define FDTD_FUSED_MIN_BLOCKS 3
#endif
constexpr int NSTAGE = FDTD_FUSED_NSTAGE;   // planes resident in the ring
constexpr int AHEAD = FDTD_FUSED_AHEAD;     // planes loaded ahead of the one computed (<= NSTAGE - 2)
static_assert(NSTAGE >= AHEAD + 2, "the ring recycles the stage of plane k - 2 at plane k");

constexpr int round128(int b) { return (b + 127) / 128 * 128; }

// Shared-memory layout of a sweep over TXv-wide columns (NTH / TXv rows between a thread's two
// nodes, TY = 2 * NTH / TXv rows per column).
template <int TXv>
struct Tile {
    static constexpr int TX = TXv, RSTEP = NTH / TXv, TY = 2 * RSTEP;
    static constexpr int HW = TX + 8, HH = TY + 2;  // H tile: x in [x0-4, x0+TX+4), y in [y0-1, y0+TY+1)
    static constexpr int EW = TX + 4, EH = TY + 1;  // old-E tile: x in [x0, x0+TX+4), y in [y0, y0+TY+1)
    // row tile: x in [xr, xr+MW) with xr = x0 rounded down to a multiple of 8, y in [y0-1, y0+TY+1)
    static constexpr int MW = TX + 8, MH = TY + 2;
    static constexpr int NW = TX + 1, NH = TY + 1;  // new-E plane: x in [x0, x0+TX], y in [y0, y0+TY]
    static constexpr int H_BYTES = round128(HW * HH * 4);
    static constexpr int E_BYTES = round128(EW * EH * 4);
    static constexpr int M_BYTES = round128(MW * MH * 2);
    static constexpr int STAGE_BYTES = 3 * H_BYTES + 3 * E_BYTES + M_BYTES;
    static constexpr unsigned TX_BYTES = 3u * HW * HH * 4 + 3u * EW * EH * 4 + MW * MH * 2;  // bytes the TMA boxes carry
    static constexpr int N_FLOATS = NW * NH;
    static constexpr int ENEW_BYTES = 2 * 3 * N_FLOATS * 4;
    static constexpr int NHALO = TX + TY + 1;  // row y0 + TY (first TX threads) and column x0 + TX
    static constexpr int SMEM = NSTAGE * STAGE_BYTES + ENEW_BYTES + NSTAGE * 8 + kMaxItemPlanes;
    static_assert(NHALO <= 64, "halo nodes live on the first two warps");
};
using TileW = Tile<kTileX>;
static_assert(TileW::TY == kTileY, "planner and kernel agree on the tile shape");

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

// Arrays of one ring stage: H tile (3), old-E tile (3), coefficient-row tile, at fixed offsets.
template <class T>
struct StageView {
    const unsigned char* base;
    __device__ explicit StageView(const unsigned char* b) : base(b) {}
    __device__ const float* h(int c) const { return reinterpret_cast<const float*>(base + c * T::H_BYTES); }
    __device__ const float* e(int c) const { return reinterpret_cast<const float*>(base + 3 * T::H_BYTES + c * T::E_BYTES); }
    __device__ const uint16_t* m() const { return reinterpret_cast<const uint16_t*>(base + 3 * T::H_BYTES + 3 * T::E_BYTES); }
};

// Slow paths of the interior kernel, out of line: nodes on the general path (lumped edges, plate
// nodes, interface nodes beyond the coefficient table's capacity). The cell materials come from the index in global memory; the
// coefficients are the table entry where the cells of an edge agree and the reference's averages
// otherwise (e_coef_mixed / h_coef_mixed), then the lumped override (calc_e fdtdrav.h:720-741).
static __device__ __noinline__ float3 e_slow(const StepParams* pp, int i, int j, int k, long long m, int plane_lumped,
                                             float ex, float ey, float ez, float dHz_j, float dHy_k, float dHx_k,
                                             float dHz_i, float dHy_i, float dHx_j) {
    const StepParams& p = *pp;
    const DeviceGrid& g = p.g;
    const long long R = g.pitch, P = g.plane, n = (long long)k * P + (long long)j * R + i;
    const uint8_t* mat = p.mat;
    const int m0 = mat[n], mi = mat[n - 1], mj = mat[n - R], mk = mat[n - P];
    const int mij = mat[n - 1 - R], mik = mat[n - 1 - P], mjk = mat[n - R - P];
    Coef3 cx = e_coef(p, 0, m0 == mj && m0 == mk && m0 == mjk, m0, mj, mk, mjk, i, j, k);
    Coef3 cy = e_coef(p, 1, m0 == mi && m0 == mk && m0 == mik, m0, mi, mk, mik, i, j, k);
    Coef3 cz = e_coef(p, 2, m0 == mi && m0 == mj && m0 == mij, m0, mi, mj, mij, i, j, k);
    if (plane_has_plate(p, k)) {
        Coef3 pc[3];
        const int hit = e_plate(&p, i, j, k, m0, mi, mj, mk, mij, mik, mjk, pc);
        if (hit & 1) cx = pc[0];
        if (hit & 2) cy = pc[1];
        if (hit & 4) cz = pc[2];
    }
    float3 r;
    const LumpedEdge* Lx = plane_lumped ? find_lumped(p, i, j, k, 0) : nullptr;  // defineSourceX edge
    r.x = Lx ? upd3(Lx->ceze, ex, Lx->cezhy, dHz_j, Lx->cezhx, dHy_k) : upd3(cx.a, ex, cx.bp, dHz_j, cx.bm, dHy_k);
    r.y = upd3(cy.a, ey, cy.bp, dHx_k, cy.bm, dHz_i);
    const LumpedEdge* L = plane_lumped ? find_lumped(p, i, j, k, 2) : nullptr;
    if (L) {
        if (L->source >= 0) {
            const float s = m < p.wave_len[L->source] ? p.waves[L->source][m] : 0.f;
            r.z = upd4(L->ceze, ez, L->cezhy, dHy_i, L->cezhx, dHx_j, L->cezj, s);
        } else {
            r.z = upd3(L->ceze, ez, L->cezhy, dHy_i, L->cezhx, dHx_j);
        }
    } else {
        r.z = upd3(cz.a, ez, cz.bp, dHy_i, cz.bm, dHx_j);
    }
    return r;
}

static __device__ __noinline__ float3 h_slow(const StepParams* pp, int i, int j, int k, float hx, float hy, float hz,
                                             float dEy_k, float dEz_j, float dEz_i, float dEx_k, float dEx_j,
                                             float dEy_i) {
    const StepParams& p = *pp;
    const DeviceGrid& g = p.g;
    const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
    const int m0 = p.mat[n], mi = p.mat[n - 1], mj = p.mat[n - g.pitch], mk = p.mat[n - g.plane];
    const MatCoef* mc = p.coef + m0;
    Coef3 cx, cy, cz;
    if (m0 == mi) { const float4 c = __ldg(&mc->h[0]); cx = Coef3{c.x, c.y, c.z}; }
    else cx = h_coef_mixed(p.props, 0, m0, mi, g.dt, g.mu0, g.dz, g.dy);
    if (m0 == mj) { const float4 c = __ldg(&mc->h[1]); cy = Coef3{c.x, c.y, c.z}; }
    else cy = h_coef_mixed(p.props, 1, m0, mj, g.dt, g.mu0, g.dx, g.dz);
    if (m0 == mk) { const float4 c = __ldg(&mc->h[2]); cz = Coef3{c.x, c.y, c.z}; }
    else cz = h_coef_mixed(p.props, 2, m0, mk, g.dt, g.mu0, g.dy, g.dx);
    return make_float3(upd3_hx(cx.a, hx, cx.bp, dEy_k, cx.bm, dEz_j), upd3(cy.a, hy, cy.bp, dEz_i, cy.bm, dEx_k),
                       upd3(cz.a, hz, cz.bp, dEx_j, cz.bm, dEy_i));
}

// Inputs of one E node read from the ring: old E, the six H differences and the coefficient row.
struct EIn {
    float ex, ey, ez, dHz_j, dHy_k, dHx_k, dHz_i, dHy_i, dHx_j;
    int c;
};
template <class T>
__device__ __forceinline__ EIn e_load(const StageView<T>& cur, const StageView<T>& prv, int hi, int ei, int mi) {
    const float* H0 = cur.h(0);
    const float* H1 = cur.h(1);
    const float* H2 = cur.h(2);
    const float hx = H0[hi], hy = H1[hi], hz = H2[hi];
    EIn r;
    r.dHz_j = __fsub_rn(hz, H2[hi - T::HW]); r.dHy_k = __fsub_rn(hy, prv.h(1)[hi]);
    r.dHx_k = __fsub_rn(hx, prv.h(0)[hi]); r.dHz_i = __fsub_rn(hz, H2[hi - 1]);
    r.dHy_i = __fsub_rn(hy, H1[hi - 1]); r.dHx_j = __fsub_rn(hx, H0[hi - T::HW]);
    r.ex = cur.e(0)[ei]; r.ey = cur.e(1)[ei]; r.ez = cur.e(2)[ei];
    r.c = cur.m()[mi];
    return r;
}
__device__ __forceinline__ float3 e_fast(const StepParams& p, const EIn& a) {
    const MatCoef* mc = p.coef + a.c;
    const float4 x = __ldg(&mc->e[0]), y = __ldg(&mc->e[1]), z = __ldg(&mc->e[2]);
    return make_float3(upd3(x.x, a.ex, x.y, a.dHz_j, x.z, a.dHy_k), upd3(y.x, a.ey, y.y, a.dHx_k, y.z, a.dHz_i),
                       upd3(z.x, a.ez, z.y, a.dHy_i, z.z, a.dHx_j));
}
__device__ __forceinline__ float3 e_any(const StepParams& p, const EIn& a, int i, int j, int k, long long m, int lumped) {
    if (a.c < kRecGeneral) return e_fast(p, a);
    return e_slow(&p, i, j, k, m, lumped, a.ex, a.ey, a.ez, a.dHz_j, a.dHy_k, a.dHx_k, a.dHz_i, a.dHy_i, a.dHx_j);
}

// Inputs of one H node: old H, the six new-E differences (from the E planes k-1 and k in shared
// memory) and the coefficient row.
struct HIn {
    float hx, hy, hz, dEy_k, dEz_j, dEz_i, dEx_k, dEx_j, dEy_i;
    int c;
};
template <class T>
__device__ __forceinline__ HIn h_load(const StageView<T>& prv, const float* en_prv, const float* en_cur, int hi, int mi,
                                      int ni) {
    constexpr int NF = T::N_FLOATS;
    HIn r;
    const float ex = en_prv[ni], ey = en_prv[NF + ni], ez = en_prv[2 * NF + ni];
    r.dEy_k = __fsub_rn(en_cur[NF + ni], ey); r.dEz_j = __fsub_rn(en_prv[2 * NF + ni + T::NW], ez);
    r.dEz_i = __fsub_rn(en_prv[2 * NF + ni + 1], ez); r.dEx_k = __fsub_rn(en_cur[ni], ex);
    r.dEx_j = __fsub_rn(en_prv[ni + T::NW], ex); r.dEy_i = __fsub_rn(en_prv[NF + ni + 1], ey);
    r.hx = prv.h(0)[hi]; r.hy = prv.h(1)[hi]; r.hz = prv.h(2)[hi];
    r.c = prv.m()[mi];
    return r;
}
__device__ __forceinline__ float3 h_fast(const StepParams& p, const HIn& a) {
    const MatCoef* mc = p.coef + a.c;
    const float4 x = __ldg(&mc->h[0]), y = __ldg(&mc->h[1]), z = __ldg(&mc->h[2]);
    return make_float3(upd3_hx(x.x, a.hx, x.y, a.dEy_k, x.z, a.dEz_j), upd3(y.x, a.hy, y.y, a.dEz_i, y.z, a.dEx_k),
                       upd3(z.x, a.hz, z.y, a.dEx_j, z.z, a.dEy_i));
}
__device__ __forceinline__ float3 h_any(const StepParams& p, const HIn& a, int i, int j, int k) {
    if (a.c < kRecGeneral) return h_fast(p, a);
    return h_slow(&p, i, j, k, a.hx, a.hy, a.hz, a.dEy_k, a.dEz_j, a.dEz_i, a.dEx_k, a.dEx_j, a.dEy_i);
}

__device__ __forceinline__ void store3(float* a, float* b, float* c, long long n, float3 v) {
    a[n] = v.x; b[n] = v.y; c[n] = v.z;
}

}  // namespace

// Interior sweep over `items` (int4 {x0, y0, k0, k1}, one per CTA; the planner puts only interior
// columns and planes here). Per-thread ring offsets are fixed for the whole item, nothing is bounds-
// checked, and the per-plane lumped / probe flags are read once into shared memory.
__global__ void __launch_bounds__(NTH, FDTD_FUSED_MIN_BLOCKS)
k_sweep_interior(const __grid_constant__ FusedMaps maps, const __grid_constant__ StepParams p, FieldPtrs fo,
                 const int4* __restrict__ items, long long m) {
    using T = TileW;
    constexpr int TX = T::TX, TY = T::TY, RSTEP = T::RSTEP, HW = T::HW, EW = T::EW, MW = T::MW, NW = T::NW;
    constexpr int NF = T::N_FLOATS;
    extern __shared__ __align__(128) unsigned char smem[];
    float* enew = reinterpret_cast<float*>(smem + NSTAGE * T::STAGE_BYTES);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + NSTAGE * T::STAGE_BYTES + T::ENEW_BYTES);
    uint8_t* pflags = reinterpret_cast<uint8_t*>(bars + NSTAGE);  // per plane: bit 0 lumped edges, bit 1 probes
    const DeviceGrid& g = p.g;
    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int4 it = items[blockIdx.x];
    const int x0 = it.x, y0 = it.y, k0 = it.z, k1 = it.w;
    const int kfirst = k0 - 1, klast = k1;
    const long long row = m % p.ring_cap;
    // own nodes (tx, ty + r * RSTEP); ring / new-E offsets of row r are these plus r * RSTEP rows
    const int i = x0 + tx, j = y0 + ty;
    const int xoff = x0 & 7;  // column of x0 in the row tile
    const int hi = (ty + 1) * HW + tx + 4, ei = ty * EW + tx, mi = (ty + 1) * MW + tx + xoff, ni = ty * NW + tx;
    // halo node of the first NHALO threads: row y0 + TY (warp 0), column x0 + TX (warp 1)
    const bool halo = tid < T::NHALO;
    const int hpx = tid < TX ? tid : TX, hpy = tid < TX ? TY : tid - TX;
    const int hhi = (hpy + 1) * HW + hpx + 4, hei = hpy * EW + hpx, hmi = (hpy + 1) * MW + hpx + xoff, hni = hpy * NW + hpx;
    const long long n_own = (long long)j * g.pitch + i;
    const long long n_row = (long long)RSTEP * g.pitch;

    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int q = tid; q <= klast - kfirst; q += NTH) {  // klast - kfirst < kMaxItemPlanes (plan_chunk)
        const int k = kfirst + q;
        pflags[q] = (p.lumped_k[k] < p.lumped_k[k + 1] ? 1 : 0) | (p.probe_k[k] < p.probe_k[k + 1] ? 2 : 0);
    }
    __syncthreads();
    auto issue = [&](int k, int s) {
        unsigned char* st = smem + s * T::STAGE_BYTES;
        mbar_expect_tx(&bars[s], T::TX_BYTES);
        for (int c = 0; c < 3; ++c) tma_load_3d(st + c * T::H_BYTES, &maps.h[c], &bars[s], x0 - 4, y0 - 1, k);
        for (int c = 0; c < 3; ++c) tma_load_3d(st + 3 * T::H_BYTES + c * T::E_BYTES, &maps.e[c], &bars[s], x0, y0, k);
        tma_load_3d(st + 3 * T::H_BYTES + 3 * T::E_BYTES, &maps.rec, &bars[s], x0 - xoff, y0 - 1, k);
    };
    if (tid == 0)
        for (int q = 0; q < AHEAD && kfirst + q <= klast; ++q) issue(kfirst + q, q);

    int s_cur = 0, s_prv = NSTAGE - 1, s_next = AHEAD % NSTAGE;
    uint32_t parity = 0;
    for (int k = kfirst; k <= klast; ++k) {
        if (tid == 0 && k + AHEAD <= klast) {
            fence_proxy_async();  // generic reads of the recycled stage precede the async writes
            issue(k + AHEAD, s_next);
        }
        const bool ok = mbar_wait(&bars[s_cur], parity);
        const StageView<T> cur(smem + s_cur * T::STAGE_BYTES);
        const StageView<T> prv(smem + s_prv * T::STAGE_BYTES);
        float* en_cur = enew + (k & 1) * 3 * NF;
        const float* en_prv = enew + ((k - 1) & 1) * 3 * NF;
        if (k >= k0) {
            // ---- E(k): own nodes (stored below plane k1), then the halo nodes ----
            const int fl = pflags[k - kfirst];
            const EIn a0 = e_load(cur, prv, hi, ei, mi);
            const EIn a1 = e_load(cur, prv, hi + RSTEP * HW, ei + RSTEP * EW, mi + RSTEP * MW);
            float3 v0, v1;
            if (a0.c < kRecGeneral && a1.c < kRecGeneral) {
                v0 = e_fast(p, a0);
                v1 = e_fast(p, a1);
            } else {
                v0 = e_any(p, a0, i, j, k, m, fl & 1);
                v1 = e_any(p, a1, i, j + RSTEP, k, m, fl & 1);
            }
            en_cur[ni] = v0.x; en_cur[NF + ni] = v0.y; en_cur[2 * NF + ni] = v0.z;
            const int ni1 = ni + RSTEP * NW;
            en_cur[ni1] = v1.x; en_cur[NF + ni1] = v1.y; en_cur[2 * NF + ni1] = v1.z;
            if (k < k1) {
                const long long n = (long long)k * g.plane + n_own;
                store3(fo.ex, fo.ey, fo.ez, n, v0);
                store3(fo.ex, fo.ey, fo.ez, n + n_row, v1);
                if (fl & 2) {
                    sample(p, row, 0, i, j, k, v0.x); sample(p, row, 1, i, j, k, v0.y); sample(p, row, 2, i, j, k, v0.z);
                    sample(p, row, 0, i, j + RSTEP, k, v1.x); sample(p, row, 1, i, j + RSTEP, k, v1.y);
                    sample(p, row, 2, i, j + RSTEP, k, v1.z);
                }
            }
            if (halo) {
                const EIn a = e_load(cur, prv, hhi, hei, hmi);
                const float3 w = e_any(p, a, x0 + hpx, y0 + hpy, k, m, fl & 1);
                en_cur[hni] = w.x; en_cur[NF + hni] = w.y; en_cur[2 * NF + hni] = w.z;
            }
        }
        if (k > k0) {
            // ---- H(k-1) of the own nodes from E(k-1), E(k) and the old H(k-1) ----
            const int kh = k - 1;
            const HIn a0 = h_load(prv, en_prv, en_cur, hi, mi, ni);
            const HIn a1 = h_load(prv, en_prv, en_cur, hi + RSTEP * HW, mi + RSTEP * MW, ni + RSTEP * NW);
            float3 v0, v1;
            if (a0.c < kRecGeneral && a1.c < kRecGeneral) {
                v0 = h_fast(p, a0);
                v1 = h_fast(p, a1);
            } else {
                v0 = h_any(p, a0, i, j, kh);
                v1 = h_any(p, a1, i, j + RSTEP, kh);
            }
            const long long n = (long long)kh * g.plane + n_own;
            store3(fo.hx, fo.hy, fo.hz, n, v0);
            store3(fo.hx, fo.hy, fo.hz, n + n_row, v1);
            if (pflags[kh - kfirst] & 2) {
                sample(p, row, 3, i, j, kh, v0.x); sample(p, row, 4, i, j, kh, v0.y); sample(p, row, 5, i, j, kh, v0.z);
                sample(p, row, 3, i, j + RSTEP, kh, v1.x); sample(p, row, 4, i, j + RSTEP, kh, v1.y);
                sample(p, row, 5, i, j + RSTEP, kh, v1.z);
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
        s_prv = s_cur;
        if (++s_cur == NSTAGE) { s_cur = 0; parity ^= 1u; }
        if (++s_next == NSTAGE) s_next = 0;
    }
}


// ---- CPML sweep ----------------------------------------------------------------------------
// The z-march of k_sweep_interior over columns whose x range (E halo included) is interior but
// whose planes or rows may lie in the z or y CPML slabs or on the boundary planes and rows: the
// planes below and above the interior z range of every interior tile, and the y bands beside the
// swept rectangle. Per plane step it computes E(k) and H(k-1) as the interior sweep does, with
// the rules of e_update / h_update that such nodes need, decided per plane (z slab, boundary
// plane) and per row (y slab, boundary row):
//   * the coefficients come from the node's coefficient row (the material row of nodes of one
//     material, the row of its seven-cell key otherwise); a curl coefficient along a CPML axis is
//     divided by that axis' kappa here (the same correctly rounded division the general path and
//     the background tables make, so the same bits); the H faces on the low boundary plane / row
//     take the default entry;
//   * the CPML memory of the y and z faces streams through a two-slot shared-memory ring filled by
//     TMA with the plane's tiles (slot k & 1: psi of E(k) and of H(k-1)); the new values go to
//     buffer B with the fields;
//   * components the boundary masks keep are copied;
//   * nodes without a coefficient row (lumped edges, plates, interface keys beyond the table)
//     take e_update / h_update out of line on their neighbourhood from the ring.
namespace {

template <class T>
struct CpmlLayout {
    static constexpr int PE_BYTES = round128(T::EW * T::EH * 4);  // psi of E: an E-tile box
    static constexpr int PH_BYTES = round128(T::TX * T::TY * 4);  // psi of H: the own nodes
    static constexpr unsigned PE_TX = T::EW * T::EH * 4, PH_TX = T::TX * T::TY * 4;  // box bytes
    static constexpr int AXIS_BYTES = 2 * PE_BYTES + 2 * PH_BYTES;  // E arrays 0, 1, then H arrays 0, 1
    static constexpr int SLOT_BYTES = 2 * AXIS_BYTES;               // y face, then z face
    static constexpr int PSI_OFF = NSTAGE * T::STAGE_BYTES;
    static constexpr int ENEW_OFF = PSI_OFF + 2 * SLOT_BYTES;
    static constexpr int BAR_OFF = ENEW_OFF + T::ENEW_BYTES;
    static constexpr int SMEM = BAR_OFF + NSTAGE * 8 + kMaxItemPlanes;
};
using CpmlW = CpmlLayout<TileW>;

#ifndef FDTD_CPML_MIN_BLOCKS
#define FDTD_CPML_MIN_BLOCKS 2
#endif

// z side of plane q: 0 / 1 inside the low / high z slab, -1 outside (or outside the grid).
__device__ __forceinline__ int z_side(const DeviceGrid& g, int q) {
    if (q < 0 || q >= g.nz) return -1;
    return q < g.pzn ? 0 : q >= g.nz - g.pzp ? 1 : -1;
}

// Per plane: the E (or H) rules of plane q.
struct CPlane {
    int zs;             // z face side, -1 outside the z slabs
    bool in, lt, low;   // 0 < q < nz - 1; q < nz - 1; q == 0
    float kap, b, a;    // kappa, b, a of the plane (E or H profiles) when zs >= 0
    float t0, t1;       // the background's kappa-divided z curl coefficients (E: Ex, Ey; H: Hx, Hy)
    int kz;             // plane index within its z face
};
__device__ __forceinline__ CPlane c_plane(const StepParams& p, int q, bool h) {
    const DeviceGrid& g = p.g;
    CPlane r;
    r.zs = z_side(g, q);
    r.in = q > 0 && q < g.nz - 1;
    r.lt = q < g.nz - 1;
    r.low = q == 0;
    r.kz = r.zs == 1 ? q - (g.nz - g.pzp) : q;
    r.kap = r.b = r.a = r.t0 = r.t1 = 0.f;
    if (r.zs >= 0) {
        r.kap = __ldg((h ? p.kmz : p.kez) + q);
        r.b = __ldg((h ? p.bmz : p.bez) + q);
        r.a = __ldg((h ? p.amz : p.aez) + q);
        r.t0 = __ldg((h ? p.bg.h[2][0] : p.bg.e[2][0]) + q);
        r.t1 = __ldg((h ? p.bg.h[2][1] : p.bg.e[2][1]) + q);
    }
    return r;
}
// Per row j of a tile whose rows meet the y face yside (-1: none): the E and H rules of the row.
struct CRow {
    bool ok, ys, in, lt, low;   // row of the grid; in the tile's y slab; 0 < j < ny - 1; j < ny - 1; j == 0
    float ke, be, ae, km, bm, am;
    float te0, te1, th0, th1;   // the background's kappa-divided y curl coefficients (Ex, Ez; Hx, Hz)
    int jy;                     // row within its y face
};
__device__ __forceinline__ CRow c_row(const StepParams& p, int j, int yside) {
    const DeviceGrid& g = p.g;
    CRow r;
    r.ok = j >= 0 && j < g.ny;
    r.ys = yside >= 0 && r.ok && in_slab(j, g.ny, g.pyn, g.pyp) && (j < g.pyn ? 0 : 1) == yside;
    r.in = j > 0 && j < g.ny - 1;
    r.lt = j < g.ny - 1;
    r.low = j == 0;
    r.jy = j < g.pyn ? j : j - (g.ny - g.pyp);
    r.ke = r.be = r.ae = r.km = r.bm = r.am = r.te0 = r.te1 = r.th0 = r.th1 = 0.f;
    if (r.ys) {
        r.ke = __ldg(p.key + j); r.be = __ldg(p.bey + j); r.ae = __ldg(p.aey + j);
        r.km = __ldg(p.kmy + j); r.bm = __ldg(p.bmy + j); r.am = __ldg(p.amy + j);
        r.te0 = __ldg(p.bg.e[1][0] + j); r.te1 = __ldg(p.bg.e[1][1] + j);
        r.th0 = __ldg(p.bg.h[1][0] + j); r.th1 = __ldg(p.bg.h[1][1] + j);
    }
    return r;
}

// psi tiles of one ring slot for the current plane step: E arrays (E-tile index), H arrays (own
// index), for the y and the z face.
struct CPsi {
    const float *ey0, *ey1, *hy0, *hy1, *ez0, *ez1, *hz0, *hz1;
};
__device__ __forceinline__ CPsi c_psi(const unsigned char* slot) {
    using L = CpmlW;
    CPsi r;
    const unsigned char* y = slot;
    const unsigned char* z = slot + L::AXIS_BYTES;
    r.ey0 = reinterpret_cast<const float*>(y);
    r.ey1 = reinterpret_cast<const float*>(y + L::PE_BYTES);
    r.hy0 = reinterpret_cast<const float*>(y + 2 * L::PE_BYTES);
    r.hy1 = reinterpret_cast<const float*>(y + 2 * L::PE_BYTES + L::PH_BYTES);
    r.ez0 = reinterpret_cast<const float*>(z);
    r.ez1 = reinterpret_cast<const float*>(z + L::PE_BYTES);
    r.hz0 = reinterpret_cast<const float*>(z + 2 * L::PE_BYTES);
    r.hz1 = reinterpret_cast<const float*>(z + 2 * L::PE_BYTES + L::PH_BYTES);
    return r;
}

// E of a node with a coefficient row (e_update's arithmetic for nodes outside the x slabs).
// ei: the node's E-tile index; w: store the new psi (own node of a stored plane) at global
// offsets qy (y face yside) / qz (z face of the plane).
__device__ __forceinline__ void e_cpml_fast(const StepParams& p, const PsiSet& pout, const EIn& a, const CPlane& zp,
                                            const CRow& yr, int yside, const CPsi& ps, int ei, bool w, int qy, int qz,
                                            float3& out, float3& pre) {
    const DeviceGrid& g = p.g;
    const MatCoef* mc = p.coef + a.c;
    const float4 cx = __ldg(&mc->e[0]), cy = __ldg(&mc->e[1]), cz = __ldg(&mc->e[2]);
    const bool zs = zp.zs >= 0, ys = yr.ys, bg = a.c == p.bg.mat;
    // curl coefficients along a CPML axis over kappa: tabulated for the background row
    float xp = cx.y, xm = cx.z, yp = cy.y, zm = cz.z;
    if (ys) {
        if (bg) { xp = yr.te0; zm = yr.te1; }
        else { xp = __fdiv_rn(cx.y, yr.ke); zm = __fdiv_rn(cz.z, yr.ke); }
    }
    if (zs) {
        if (bg) { xm = zp.t0; yp = zp.t1; }
        else { xm = __fdiv_rn(cx.z, zp.kap); yp = __fdiv_rn(cy.y, zp.kap); }
    }
    float vx = upd3(cx.x, a.ex, xp, a.dHz_j, xm, a.dHy_k);
    float vy = upd3(cy.x, a.ey, yp, a.dHx_k, cy.z, a.dHz_i);
    float vz = upd3(cz.x, a.ez, cz.y, a.dHy_i, zm, a.dHx_j);
    const bool exm = yr.in && zp.in, eym = yr.lt && zp.in, ezm = yr.in && zp.lt;
    pre = make_float3(exm ? vx : a.ex, eym ? vy : a.ey, ezm ? vz : a.ez);
    if (ys && (exm || ezm)) {  // fdtdrav.h:790-827
        const PsiFace& o = pout.f[2 + yside];
        if (exm) {
            const float s = psi_upd(yr.be, ps.ey0[ei], yr.ae, a.dHz_j);
            if (w) o.e[0][qy] = s;
            vx = psi_add(vx, __fmul_rn(cx.y, g.dy), s);
        }
        if (ezm) {
            const float s = psi_upd(yr.be, ps.ey1[ei], yr.ae, a.dHx_j);
            if (w) o.e[1][qy] = s;
            vz = psi_add(vz, __fmul_rn(cz.z, g.dy), s);
        }
    }
    if (zs && (exm || eym)) {  // fdtdrav.h:829-911
        const PsiFace& o = pout.f[4 + zp.zs];
        if (exm) {
            const float s = psi_upd(zp.b, ps.ez0[ei], zp.a, a.dHy_k);
            if (w) o.e[0][qz] = s;
            vx = psi_add(vx, __fmul_rn(cx.z, g.dz), s);
        }
        if (eym) {
            const float s = psi_upd(zp.b, ps.ez1[ei], zp.a, a.dHx_k);
            if (w) o.e[1][qz] = s;
            vy = psi_add(vy, __fmul_rn(cy.y, g.dz), s);
        }
    }
    out = make_float3(exm ? vx : a.ex, eym ? vy : a.ey, ezm ? vz : a.ez);
}

// H of a node with a coefficient row (h_update's arithmetic for nodes outside the x slabs); c:
// the row; oi: the node's own-tile index.
__device__ __forceinline__ void h_cpml_fast(const StepParams& p, const PsiSet& pout, const HIn& a, const CPlane& zp,
                                            const CRow& yr, int yside, const CPsi& ps, int oi, int qy, int qz,
                                            float3& out, float3& pre) {
    const DeviceGrid& g = p.g;
    const float4 cx = __ldg(&p.coef[a.c].h[0]);
    const float4 cy = __ldg(&p.coef[yr.low ? kDefaultEntry : a.c].h[1]);  // face on the low boundary row
    const float4 cz = __ldg(&p.coef[zp.low ? kDefaultEntry : a.c].h[2]);  // face on the low boundary plane
    const bool zs = zp.zs >= 0, ys = yr.ys, bg = a.c == p.bg.mat;
    // as for E; the default entries of the boundary row / plane are not the background's
    float xp = cx.y, xm = cx.z, ym = cy.z, zp_ = cz.y;
    if (zs) {
        xp = bg ? zp.t0 : __fdiv_rn(cx.y, zp.kap);
        ym = bg && !yr.low ? zp.t1 : __fdiv_rn(cy.z, zp.kap);
    }
    if (ys) {
        xm = bg ? yr.th0 : __fdiv_rn(cx.z, yr.km);
        zp_ = bg && !zp.low ? yr.th1 : __fdiv_rn(cz.y, yr.km);
    }
    float vx = upd3_hx(cx.x, a.hx, xp, a.dEy_k, xm, a.dEz_j);
    float vy = upd3(cy.x, a.hy, cy.y, a.dEz_i, ym, a.dEx_k);
    float vz = upd3(cz.x, a.hz, zp_, a.dEx_j, cz.z, a.dEy_i);
    const bool hxm = yr.lt && zp.lt, hym = zp.lt, hzm = yr.lt;
    pre = make_float3(hxm ? vx : a.hx, hym ? vy : a.hy, hzm ? vz : a.hz);
    if (ys && (hxm || hzm)) {  // fdtdrav.h:445-486
        const PsiFace& o = pout.f[2 + yside];
        if (hxm) {
            const float s = psi_upd(yr.bm, ps.hy0[oi], yr.am, a.dEz_j);
            o.h[0][qy] = s;
            vx = psi_add(vx, __fmul_rn(cx.z, g.dy), s);
        }
        if (hzm) {
            const float s = psi_upd(yr.bm, ps.hy1[oi], yr.am, a.dEx_j);
            o.h[1][qy] = s;
            vz = psi_add(vz, __fmul_rn(cz.y, g.dy), s);
        }
    }
    if (zs && (hxm || hym)) {  // fdtdrav.h:489-562
        const PsiFace& o = pout.f[4 + zp.zs];
        if (hxm) {
            const float s = psi_upd(zp.b, ps.hz0[oi], zp.a, a.dEy_k);
            o.h[0][qz] = s;
            vx = psi_add(vx, __fmul_rn(cx.y, g.dz), s);
        }
        if (hym) {
            const float s = psi_upd_hyz(zp.b, ps.hz1[oi], zp.a, a.dEx_k);
            o.h[1][qz] = s;
            vy = psi_add(vy, __fmul_rn(cy.z, g.dz), s);
        }
    }
    out = make_float3(hxm ? vx : a.hx, hym ? vy : a.hy, hzm ? vz : a.hz);
}

// E of a node without a coefficient row: e_update on its neighbourhood from the ring (cur / prv
// stage bases, H-tile index hi), cell materials and CPML memory from global memory (psi of buffer
// A; the new psi stored when `write`). Plate nodes take their plate coefficients; k_plate_e
// stores them and their psi, so neither is written here. Returns out (x, y, z) then pre.
static __device__ __noinline__ void e_cpml_slow(const StepParams* pp, const PsiSet* pin, const PsiSet* pout,
                                                const unsigned char* curb, const unsigned char* prvb, int hi, float ex,
                                                float ey, float ez, int i, int j, int k, long long m, int lumped,
                                                bool write, int cls, float* r6) {
    const StepParams& p = *pp;
    const DeviceGrid& g = p.g;
    const StageView<TileW> cur(curb), prv(prvb);
    constexpr int HW = TileW::HW;
    ENbr nb;
    nb.ex = ex; nb.ey = ey; nb.ez = ez;
    nb.hx = cur.h(0)[hi]; nb.hy = cur.h(1)[hi]; nb.hz = cur.h(2)[hi];
    nb.hx_jm = cur.h(0)[hi - HW]; nb.hx_km = prv.h(0)[hi];
    nb.hy_im = cur.h(1)[hi - 1]; nb.hy_km = prv.h(1)[hi];
    nb.hz_im = cur.h(2)[hi - 1]; nb.hz_jm = cur.h(2)[hi - HW];
    const long long R = g.pitch, P = g.plane, n = (long long)k * P + (long long)j * R + i;
    const uint8_t* mat = p.mat;
    nb.m0 = mat[n];
    nb.mi = mat[n - 1];  // i > 0: the column is interior
    nb.mj = j > 0 ? mat[n - R] : 0;
    nb.mk = k > 0 ? mat[n - P] : 0;
    nb.mij = j > 0 ? mat[n - 1 - R] : 0;
    nb.mik = k > 0 ? mat[n - 1 - P] : 0;
    nb.mjk = (j > 0 && k > 0) ? mat[n - R - P] : 0;
    const PsiIO io{pin->f, pout->f, write && cls != kPlateNode};
    float out[3], pre[3];
    e_update<false, false, true, false, 6>(p, nb, i, j, k, m, lumped != 0, io, out, pre);
    r6[0] = out[0]; r6[1] = out[1]; r6[2] = out[2];
    r6[3] = pre[0]; r6[4] = pre[1]; r6[5] = pre[2];
}

// H of a node without a coefficient row: h_update on its neighbourhood (old H from the prv stage,
// new E of planes kh and kh + 1 from the new-E tiles, index ni), CPML memory from global memory.
static __device__ __noinline__ void h_cpml_slow(const StepParams* pp, const PsiSet* pin, const PsiSet* pout,
                                                const unsigned char* prvb, int hi, const float* en_prv,
                                                const float* en_cur, int ni, int i, int j, int kh, float* r6) {
    const StepParams& p = *pp;
    const DeviceGrid& g = p.g;
    const StageView<TileW> prv(prvb);
    constexpr int NF = TileW::N_FLOATS, NW = TileW::NW;
    HNbr nb;
    nb.hx = prv.h(0)[hi]; nb.hy = prv.h(1)[hi]; nb.hz = prv.h(2)[hi];
    nb.ex = en_prv[ni]; nb.ey = en_prv[NF + ni]; nb.ez = en_prv[2 * NF + ni];
    nb.ey_kp = en_cur[NF + ni]; nb.ex_kp = en_cur[ni];
    nb.ez_jp = en_prv[2 * NF + ni + NW]; nb.ex_jp = en_prv[ni + NW];
    nb.ez_ip = en_prv[2 * NF + ni + 1]; nb.ey_ip = en_prv[NF + ni + 1];
    const long long R = g.pitch, P = g.plane, n = (long long)kh * P + (long long)j * R + i;
    const uint8_t* mat = p.mat;
    nb.m0 = mat[n];
    nb.mi = mat[n - 1];
    nb.mj = j > 0 ? mat[n - R] : 0;
    nb.mk = kh > 0 ? mat[n - P] : 0;
    const PsiIO io{pin->f, pout->f, true};
    float out[3], pre[3];
    h_update<false, false, 6>(p, nb, i, j, kh, io, out, pre);
    r6[0] = out[0]; r6[1] = out[1]; r6[2] = out[2];
    r6[3] = pre[0]; r6[4] = pre[1]; r6[5] = pre[2];
}

}  // namespace

// CPML sweep over `items` (int4 {x0, y0, k0, k1}, planner.h's CPML items: 32 x 16 columns with an
// interior x range, planes [k0, k1) anywhere in [0, nz)). Rows outside the grid are neither
// computed nor stored. Plane -1, plane nz and rows outside the grid load as zeros (TMA fill): the
// coefficient row of plane nz, where E is computed for H below it, reads as 0, so those nodes take
// the fast path; they are never stored. Every wait is bounded as in k_sweep_interior.
__global__ void __launch_bounds__(NTH, FDTD_CPML_MIN_BLOCKS)
k_sweep_cpml(const __grid_constant__ CpmlMaps maps, const __grid_constant__ StepParams p, FieldPtrs fo,
             const __grid_constant__ PsiSet pin, const __grid_constant__ PsiSet pout, const int4* __restrict__ items,
             long long m) {
    using T = TileW;
    using L = CpmlW;
    constexpr int TX = T::TX, TY = T::TY, RSTEP = T::RSTEP, HW = T::HW, EW = T::EW, MW = T::MW, NW = T::NW;
    constexpr int NF = T::N_FLOATS;
    extern __shared__ __align__(128) unsigned char smem[];
    float* enew = reinterpret_cast<float*>(smem + L::ENEW_OFF);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L::BAR_OFF);
    uint8_t* pflags = reinterpret_cast<uint8_t*>(bars + NSTAGE);  // per plane: bit 0 lumped edges, bit 1 probes
    const DeviceGrid& g = p.g;
    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int4 it = items[blockIdx.x];
    const int x0 = it.x, y0 = it.y, k0 = it.z, k1 = it.w;
    const int kfirst = k0 - 1, klast = k1;
    const long long row = m % p.ring_cap;
    const int i = x0 + tx, j = y0 + ty;
    const int xoff = x0 & 7;
    const int hi = (ty + 1) * HW + tx + 4, ei = ty * EW + tx, mi = (ty + 1) * MW + tx + xoff, ni = ty * NW + tx;
    const int oi = ty * TX + tx;
    const bool halo = tid < T::NHALO;
    const int hpx = tid < TX ? tid : TX, hpy = tid < TX ? TY : tid - TX;
    const int hhi = (hpy + 1) * HW + hpx + 4, hei = hpy * EW + hpx, hmi = (hpy + 1) * MW + hpx + xoff, hni = hpy * NW + hpx;
    const long long n_own = (long long)j * g.pitch + i;
    const long long n_row = (long long)RSTEP * g.pitch;
    // the tile's y face (its rows, E halo row included, meet at most one): side, first row; only a
    // face with CPML cells has maps (maps.faces)
    const int yside = (g.pyn > 0 && y0 < g.pyn) ? 0 : (g.pyp > 0 && y0 + TY >= g.ny - g.pyp) ? 1 : -1;
    const int ybase = yside == 1 ? g.ny - g.pyp : 0;
    const CRow r0 = c_row(p, j, yside), r1 = c_row(p, j + RSTEP, yside);
    const CRow rh = c_row(p, y0 + hpy, yside);
    // CPML memory offsets of the own nodes within a y face plane / a z face plane
    const int qy0 = r0.jy * g.pitch + i, qy1 = r1.jy * g.pitch + i;
    const int qz0 = j * g.pitch + i, qz1 = (j + RSTEP) * g.pitch + i;

    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int q = tid; q <= klast - kfirst; q += NTH) {  // klast - kfirst < kMaxItemPlanes (planner)
        const int k = kfirst + q;
        pflags[q] = (k < 0 || k >= g.nz) ? 0
                    : (p.lumped_k[k] < p.lumped_k[k + 1] ? 1 : 0) | (p.probe_k[k] < p.probe_k[k + 1] ? 2 : 0);
    }
    __syncthreads();
    auto issue = [&](int k, int s) {
        unsigned char* st = smem + s * T::STAGE_BYTES;
        unsigned char* ps = smem + L::PSI_OFF + (k & 1) * L::SLOT_BYTES;
        const bool ne = k >= k0, nh = k > k0;  // E(k), H(k-1) computed at this step
        int ze = ne ? z_side(g, k) : -1, zh = nh ? z_side(g, k - 1) : -1;
        if (ze >= 0 && !((maps.faces >> (2 + ze)) & 1)) ze = -1;
        if (zh >= 0 && !((maps.faces >> (2 + zh)) & 1)) zh = -1;
        const bool yok = yside >= 0 && ((maps.faces >> yside) & 1);
        const bool ye = ne && yok, yh = nh && yok;
        const unsigned bytes = T::TX_BYTES + (ye ? 2 * L::PE_TX : 0) + (yh ? 2 * L::PH_TX : 0) +
                               (ze >= 0 ? 2 * L::PE_TX : 0) + (zh >= 0 ? 2 * L::PH_TX : 0);
        mbar_expect_tx(&bars[s], bytes);
        for (int c = 0; c < 3; ++c) tma_load_3d(st + c * T::H_BYTES, &maps.base.h[c], &bars[s], x0 - 4, y0 - 1, k);
        for (int c = 0; c < 3; ++c) tma_load_3d(st + 3 * T::H_BYTES + c * T::E_BYTES, &maps.base.e[c], &bars[s], x0, y0, k);
        tma_load_3d(st + 3 * T::H_BYTES + 3 * T::E_BYTES, &maps.base.rec, &bars[s], x0 - xoff, y0 - 1, k);
        for (int a = 0; a < 2; ++a) {
            if (ye) tma_load_3d(ps + a * L::PE_BYTES, &maps.ye[yside][a], &bars[s], x0, y0 - ybase, k);
            if (yh) tma_load_3d(ps + 2 * L::PE_BYTES + a * L::PH_BYTES, &maps.yh[yside][a], &bars[s], x0, y0 - ybase, k - 1);
            if (ze >= 0)
                tma_load_3d(ps + L::AXIS_BYTES + a * L::PE_BYTES, &maps.ze[ze][a], &bars[s], x0, y0,
                            ze == 1 ? k - (g.nz - g.pzp) : k);
            if (zh >= 0)
                tma_load_3d(ps + L::AXIS_BYTES + 2 * L::PE_BYTES + a * L::PH_BYTES, &maps.zh[zh][a], &bars[s], x0, y0,
                            zh == 1 ? k - 1 - (g.nz - g.pzp) : k - 1);
        }
    };
    if (tid == 0)
        for (int q = 0; q < AHEAD && kfirst + q <= klast; ++q) issue(kfirst + q, q);

    int s_cur = 0, s_prv = NSTAGE - 1, s_next = AHEAD % NSTAGE;
    uint32_t parity = 0;
    for (int k = kfirst; k <= klast; ++k) {
        if (tid == 0 && k + AHEAD <= klast) {
            fence_proxy_async();  // generic reads of the recycled stage and psi slot precede the async writes
            issue(k + AHEAD, s_next);
        }
        const bool ok = mbar_wait(&bars[s_cur], parity);
        const unsigned char* curb = smem + s_cur * T::STAGE_BYTES;
        const unsigned char* prvb = smem + s_prv * T::STAGE_BYTES;
        const StageView<T> cur(curb);
        const StageView<T> prv(prvb);
        const CPsi ps = c_psi(smem + L::PSI_OFF + (k & 1) * L::SLOT_BYTES);
        float* en_cur = enew + (k & 1) * 3 * NF;
        const float* en_prv = enew + ((k - 1) & 1) * 3 * NF;
        if (k >= k0) {
            // ---- E(k): own nodes (stored, with their psi, below plane k1), then the halo nodes ----
            const int fl = pflags[k - kfirst];
            const bool st = k < k1;
            const CPlane zp = c_plane(p, k, false);
            const int qz = zp.kz * g.ny * g.pitch;
            const int qy = k * (yside == 1 ? g.pyp : g.pyn) * g.pitch;
            float3 v[2], w[2];
            bool plate[2];
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const CRow& yr = r ? r1 : r0;
                plate[r] = true;  // rows outside the grid: nothing stored
                if (!yr.ok) continue;
                const EIn a = e_load(cur, prv, hi + r * RSTEP * HW, ei + r * RSTEP * EW, mi + r * RSTEP * MW);
                plate[r] = a.c == (kRecGeneral | kPlateNode);
                if (a.c < kRecGeneral) {
                    e_cpml_fast(p, pout, a, zp, yr, yside, ps, ei + r * RSTEP * EW, st, qy + (r ? qy1 : qy0),
                                qz + (r ? qz1 : qz0), v[r], w[r]);
                } else {
                    float r6[6];
                    e_cpml_slow(&p, &pin, &pout, curb, prvb, hi + r * RSTEP * HW, a.ex, a.ey, a.ez, i, j + r * RSTEP, k,
                                m, fl & 1, st, a.c & 0xff, r6);
                    v[r] = make_float3(r6[0], r6[1], r6[2]);
                    w[r] = make_float3(r6[3], r6[4], r6[5]);
                }
                const int nn = ni + r * RSTEP * NW;
                en_cur[nn] = v[r].x; en_cur[NF + nn] = v[r].y; en_cur[2 * NF + nn] = v[r].z;
            }
            if (st) {
                const long long n = (long long)k * g.plane + n_own;
#pragma unroll
                for (int r = 0; r < 2; ++r)
                    if (!plate[r]) store3(fo.ex, fo.ey, fo.ez, n + r * n_row, v[r]);  // k_plate_e stores plate nodes
                if (fl & 2) {
                    if (r0.ok) {
                        sample(p, row, 0, i, j, k, w[0].x); sample(p, row, 1, i, j, k, w[0].y);
                        sample(p, row, 2, i, j, k, w[0].z);
                    }
                    if (r1.ok) {
                        sample(p, row, 0, i, j + RSTEP, k, w[1].x); sample(p, row, 1, i, j + RSTEP, k, w[1].y);
                        sample(p, row, 2, i, j + RSTEP, k, w[1].z);
                    }
                }
            }
            if (halo && rh.ok) {
                const EIn a = e_load(cur, prv, hhi, hei, hmi);
                float3 hv, hw;
                if (a.c < kRecGeneral) {
                    e_cpml_fast(p, pout, a, zp, rh, yside, ps, hei, false, 0, 0, hv, hw);
                } else {
                    float r6[6];
                    e_cpml_slow(&p, &pin, &pout, curb, prvb, hhi, a.ex, a.ey, a.ez, x0 + hpx, y0 + hpy, k, m, fl & 1,
                                false, a.c & 0xff, r6);
                    hv = make_float3(r6[0], r6[1], r6[2]);
                }
                en_cur[hni] = hv.x; en_cur[NF + hni] = hv.y; en_cur[2 * NF + hni] = hv.z;
            }
        }
        if (k > k0) {
            // ---- H(k-1) of the own nodes from E(k-1), E(k) and the old H(k-1) ----
            const int kh = k - 1;
            const CPlane zp = c_plane(p, kh, true);
            const int qz = zp.kz * g.ny * g.pitch;
            const int qy = kh * (yside == 1 ? g.pyp : g.pyn) * g.pitch;
            const long long n = (long long)kh * g.plane + n_own;
            float3 v[2], w[2];
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const CRow& yr = r ? r1 : r0;
                if (!yr.ok) continue;
                const int nn = ni + r * RSTEP * NW;
                const HIn a = h_load(prv, en_prv, en_cur, hi + r * RSTEP * HW, mi + r * RSTEP * MW, nn);
                if (a.c < kRecGeneral) {
                    h_cpml_fast(p, pout, a, zp, yr, yside, ps, oi + r * RSTEP * TX, qy + (r ? qy1 : qy0),
                                qz + (r ? qz1 : qz0), v[r], w[r]);
                } else {
                    float r6[6];
                    h_cpml_slow(&p, &pin, &pout, prvb, hi + r * RSTEP * HW, en_prv, en_cur, nn, i, j + r * RSTEP, kh, r6);
                    v[r] = make_float3(r6[0], r6[1], r6[2]);
                    w[r] = make_float3(r6[3], r6[4], r6[5]);
                }
                store3(fo.hx, fo.hy, fo.hz, n + r * n_row, v[r]);
            }
            if (pflags[kh - kfirst] & 2) {
                if (r0.ok) {
                    sample(p, row, 3, i, j, kh, w[0].x); sample(p, row, 4, i, j, kh, w[0].y);
                    sample(p, row, 5, i, j, kh, w[0].z);
                }
                if (r1.ok) {
                    sample(p, row, 3, i, j + RSTEP, kh, w[1].x); sample(p, row, 4, i, j + RSTEP, kh, w[1].y);
                    sample(p, row, 5, i, j + RSTEP, kh, w[1].z);
                }
            }
        }
        if (__syncthreads_or(!ok)) {
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
        s_prv = s_cur;
        if (++s_cur == NSTAGE) { s_cur = 0; parity ^= 1u; }
        if (++s_next == NSTAGE) s_next = 0;
    }
}

int fused_smem_bytes() { return TileW::SMEM; }
int cpml_smem_bytes() { return CpmlW::SMEM; }

cudaError_t fused_configure() {
    cudaError_t e = cudaFuncSetAttribute(k_sweep_interior, cudaFuncAttributeMaxDynamicSharedMemorySize, TileW::SMEM);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_sweep_cpml, cudaFuncAttributeMaxDynamicSharedMemorySize, CpmlW::SMEM);
    return e;
}

// One fused step: per-node E of the shell items (CPML slabs, boundary planes, strips beside the
// interior tiles, tiles around a design region), the design region's and the plates' E, the
// interior sweep and the CPML sweep, per-node H of the shell items (which reads the new E of its
// neighbours, written by the sweeps). With a fork the sweeps run beside the shell E pass on the
// second stream.
cudaError_t launch_fused(const FusedMaps& maps, const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo,
                         const PsiSet& psi_in, const PsiSet& psi_out, long long m, const FusedWork& w, cudaStream_t st,
                         const FusedFork* fork, const CpmlMaps* cmaps) {
    cudaError_t e = cudaSuccess;
    if (w.n_cpml > 0 && !cmaps) return cudaErrorInvalidValue;
    const bool split = fork && w.n_interior > 0;
    if (split) {
        e = cudaEventRecord(fork->fork, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(fork->aux, fork->fork, 0);
        if (e != cudaSuccess) return e;
        k_sweep_interior<<<w.n_interior, NTH, TileW::SMEM, fork->aux>>>(maps, p, fo, w.interior, m);
        if (w.n_cpml > 0)
            k_sweep_cpml<<<w.n_cpml, NTH, CpmlW::SMEM, fork->aux>>>(*cmaps, p, fo, psi_in, psi_out, w.cpml, m);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(fork->join, fork->aux);
        if (e != cudaSuccess) return e;
    }
    e = launch_shell(true, p, fi, fo, psi_in, psi_out, w.shell, m, st);
    if (e == cudaSuccess) e = launch_design_e(p, fi, fo, psi_in, psi_out, m, st);
    if (e == cudaSuccess) e = launch_plate_e(p, fi, fo, psi_in, psi_out, m, st);
    if (e != cudaSuccess) return e;
    if (split) {
        e = cudaStreamWaitEvent(st, fork->join, 0);
    } else if (w.n_interior > 0) {
        k_sweep_interior<<<w.n_interior, NTH, TileW::SMEM, st>>>(maps, p, fo, w.interior, m);
        if (w.n_cpml > 0) k_sweep_cpml<<<w.n_cpml, NTH, CpmlW::SMEM, st>>>(*cmaps, p, fo, psi_in, psi_out, w.cpml, m);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
    return launch_shell(false, p, fi, fo, psi_in, psi_out, w.shell, m, st);
}

namespace {

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                              const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Tensor maps of one tile shape: H tiles with a one-node halo (x widened to 16-byte boundaries),
// old-E tiles, coefficient-row tiles. Coordinates outside the arrays load as zeros.
template <class T>
int encode_tile_maps(FusedMaps* out, const DeviceGrid& g, float* const h[3], float* const e[3], const uint16_t* rec,
                     EncodeFn encode) {
    const cuuint64_t dims[3] = {(cuuint64_t)g.pitch, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    const cuuint64_t fstr[2] = {(cuuint64_t)g.pitch * 4, (cuuint64_t)g.plane * 4};
    const cuuint64_t mstr[2] = {(cuuint64_t)g.pitch * 2, (cuuint64_t)g.plane * 2};
    const cuuint32_t hbox[3] = {T::HW, T::HH, 1}, ebox[3] = {T::EW, T::EH, 1}, mbox[3] = {T::MW, T::MH, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    for (int c = 0; c < 3; ++c) {
        if (encode(&out->h[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, h[c], dims, fstr, hbox, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return -1;
        if (encode(&out->e[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, e[c], dims, fstr, ebox, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return -1;
    }
    if (encode(&out->rec, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, (void*)rec, dims, mstr, mbox, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return -1;
    return 0;
}

}  // namespace

int encode_fused_maps(FusedMaps* out, const DeviceGrid& g, float* const h[3], float* const e[3], const uint16_t* rec,
                      void* encode_fn) {
    return encode_tile_maps<TileW>(out, g, h, e, rec, reinterpret_cast<EncodeFn>(encode_fn));
}

// CPML memory maps of the y faces ((nz, P, pitch) arrays) and z faces ((P, ny, pitch)): E arrays in
// E-tile boxes, H arrays in own-node boxes. Coordinates outside an array load as zeros.
int encode_cpml_maps(CpmlMaps* out, const DeviceGrid& g, float* const h[3], float* const e[3], const uint16_t* rec,
                     const PsiSet& psi, void* encode_fn) {
    using T = TileW;
    const EncodeFn encode = reinterpret_cast<EncodeFn>(encode_fn);
    *out = CpmlMaps{};
    if (encode_tile_maps<T>(&out->base, g, h, e, rec, encode) != 0) return -1;
    const cuuint32_t ebox[3] = {T::EW, T::EH, 1}, hbox[3] = {T::TX, T::TY, 1}, es[3] = {1, 1, 1};
    auto map = [&](CUtensorMap* m, float* base, const cuuint64_t* dims, const cuuint64_t* str, const cuuint32_t* box) {
        return encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, str, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
                       CUDA_SUCCESS
                   ? 0
                   : -1;
    };
    for (int s = 0; s < 2; ++s) {
        const int py = s ? g.pyp : g.pyn, pz = s ? g.pzp : g.pzn;
        if (py > 0) {
            out->faces |= 1 << s;
            const cuuint64_t dims[3] = {(cuuint64_t)g.pitch, (cuuint64_t)py, (cuuint64_t)g.nz};
            const cuuint64_t str[2] = {(cuuint64_t)g.pitch * 4, (cuuint64_t)py * g.pitch * 4};
            const PsiFace& f = psi.f[2 + s];
            for (int a = 0; a < 2; ++a)
                if (map(&out->ye[s][a], f.e[a], dims, str, ebox) || map(&out->yh[s][a], f.h[a], dims, str, hbox)) return -1;
        }
        if (pz > 0) {
            out->faces |= 4 << s;
            const cuuint64_t dims[3] = {(cuuint64_t)g.pitch, (cuuint64_t)g.ny, (cuuint64_t)pz};
            const cuuint64_t str[2] = {(cuuint64_t)g.pitch * 4, (cuuint64_t)g.ny * g.pitch * 4};
            const PsiFace& f = psi.f[4 + s];
            for (int a = 0; a < 2; ++a)
                if (map(&out->ze[s][a], f.e[a], dims, str, ebox) || map(&out->zh[s][a], f.h[a], dims, str, hbox)) return -1;
        }
    }
    return 0;
}

}  // namespace fdtd
