// Fused schedule: per time step, z-marching sweeps over the whole grid (plus a per-node pass over
// the tiles around a design region), all reading buffer A and writing buffer B.
//
// A sweep work item is a TX x TY column of nodes and a plane range [k0, k1). Planes stream through
// a 3-stage shared-memory ring filled by TMA (cp.async.bulk.tensor, 3-D tiles of this GPU's HBM,
// one plane ahead of the one computed): H with a one-node halo, old E, and the coefficient row of
// each node (16 bits: StepParams::rec). At plane k the CTA
//   1. computes E(k) on its tile plus one column / row beyond the high x / y edges (the H update
//      needs those E values; they are recomputed from the old fields instead of being exchanged),
//      storing only its own nodes;
//   2. computes H(k-1) of its own nodes from E(k-1), E(k) (shared memory) and H(k-1) (the ring).
// Each thread owns two nodes of a plane (rows ty and ty + TY / 2), which gives every warp two
// independent update chains and halves the per-plane overhead per node. Each field value crosses
// HBM once per step in each direction (24 B read + 24 B written per cell) plus the 2-byte row.
//
// Two kernels share this structure (the work planner, planner.cpp, assigns the items):
//   * k_sweep_interior, 32 x 16 columns whose nodes and E halo are all interior: fast-path and
//     interface nodes update from their coefficient row; the other nodes (lumped edges, plates,
//     interface nodes beyond the table) leave the fast path through an out-of-line call;
//   * k_sweep_general, 32 x 16 or 16 x 32 columns anywhere in the grid (CPML slabs, boundary
//     planes, the bands beside the interior): nodes on the general path take the shared
//     e_update / h_update, CPML recurrences included, with their CPML memory read from A and
//     written to B in the same pass (background CPML nodes inline, the rest out of line); masks
//     keep the boundary planes' components, and columns, rows and planes outside the grid or the
//     item are neither computed from memory nor stored.
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
#ifndef FDTD_GENERAL_MIN_BLOCKS
#define FDTD_GENERAL_MIN_BLOCKS 3
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
using TileN = Tile<kNarrowX>;
static_assert(TileW::TY == kTileY && TileN::TY == kNarrowY, "planner and kernels agree on the tile shapes");

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
    r.x = upd3(cx.a, ex, cx.bp, dHz_j, cx.bm, dHy_k);
    r.y = upd3(cy.a, ey, cy.bp, dHx_k, cy.bm, dHz_i);
    const LumpedEdge* L = plane_lumped ? find_lumped(p, i, j, k) : nullptr;
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

// ---- general sweep: nodes of any class, CPML memory included ----

// The seven cell materials of a general E node of class `cls` (shared by all seven for classes
// kUniformGeneral + m; from the index otherwise; cells outside the grid read as 0, never used).
__device__ __forceinline__ void e_cells(const StepParams& p, int cls, int i, int j, int k, ENbr& n) {
    if (cls >= kUniformGeneral && cls < kInterfaceNode) {
        n.m0 = n.mi = n.mj = n.mk = n.mij = n.mik = n.mjk = cls - kUniformGeneral;
        return;
    }
    const DeviceGrid& g = p.g;
    const long long R = g.pitch, P = g.plane, q = (long long)k * P + (long long)j * R + i;
    const uint8_t* mat = p.mat;
    n.m0 = mat[q];
    n.mi = i > 0 ? mat[q - 1] : 0;
    n.mj = j > 0 ? mat[q - R] : 0;
    n.mk = k > 0 ? mat[q - P] : 0;
    n.mij = (i > 0 && j > 0) ? mat[q - 1 - R] : 0;
    n.mik = (i > 0 && k > 0) ? mat[q - 1 - P] : 0;
    n.mjk = (j > 0 && k > 0) ? mat[q - R - P] : 0;
}
__device__ __forceinline__ void h_cells(const StepParams& p, int cls, int i, int j, int k, HNbr& n) {
    if (cls >= kUniformGeneral && cls < kInterfaceNode) {
        n.m0 = n.mi = n.mj = n.mk = cls - kUniformGeneral;
        return;
    }
    const DeviceGrid& g = p.g;
    const long long q = (long long)k * g.plane + (long long)j * g.pitch + i;
    n.m0 = p.mat[q];
    n.mi = i > 0 ? p.mat[q - 1] : 0;
    n.mj = j > 0 ? p.mat[q - g.pitch] : 0;
    n.mk = k > 0 ? p.mat[q - g.plane] : 0;
}

// One general E node of the sweep from the ring, written to the new-E plane (slot nn), to the
// fields (store) and to the probe ring (probes): nodes other than fast-path, interface and
// background CPML nodes (lumped edges, plates, material interfaces inside the CPML, materials
// other than the background's). Out of line, self-contained: it reads its neighbourhood from the
// ring and writes its results itself, so that no local of the calling loop lives in memory.
template <class T>
static __device__ __noinline__ void e_general(const StepParams* pp, const PsiSet* pin, const PsiSet* pout,
                                              const unsigned char* cur_base, const unsigned char* prv_base, int hi,
                                              int ei, int mi, int nn, float* en_cur, int i, int j, int k, long long m,
                                              int lumped, int store, float* fex, float* fey, float* fez, long long row,
                                              int probes) {
    const StepParams& p = *pp;
    const StageView<T> cur(cur_base), prv(prv_base);
    const int cls = cur.m()[mi] & 0xff;
    ENbr n;
    n.hx = cur.h(0)[hi]; n.hy = cur.h(1)[hi]; n.hz = cur.h(2)[hi];
    n.hx_jm = cur.h(0)[hi - T::HW]; n.hx_km = prv.h(0)[hi];
    n.hy_im = cur.h(1)[hi - 1]; n.hy_km = prv.h(1)[hi];
    n.hz_im = cur.h(2)[hi - 1]; n.hz_jm = cur.h(2)[hi - T::HW];
    n.ex = cur.e(0)[ei]; n.ey = cur.e(1)[ei]; n.ez = cur.e(2)[ei];
    e_cells(p, cls, i, j, k, n);
    const PsiIO io{pin->f, pout->f, store != 0};
    float out[3], pre[3];
    if (cls == kPlateNode) e_update<false, false, true>(p, n, i, j, k, m, lumped != 0, io, out, pre);
    else e_update<false, false, false>(p, n, i, j, k, m, lumped != 0, io, out, pre);
    constexpr int NF = T::N_FLOATS;
    en_cur[nn] = out[0]; en_cur[NF + nn] = out[1]; en_cur[2 * NF + nn] = out[2];
    if (store) {
        const long long q = (long long)k * p.g.plane + (long long)j * p.g.pitch + i;
        fex[q] = out[0]; fey[q] = out[1]; fez[q] = out[2];
        if (probes) {
            sample(p, row, 0, i, j, k, pre[0]); sample(p, row, 1, i, j, k, pre[1]); sample(p, row, 2, i, j, k, pre[2]);
        }
    }
}

// One general H node of the sweep (the H counterpart of e_general), stored with its samples.
template <class T>
static __device__ __noinline__ void h_general(const StepParams* pp, const PsiSet* pin, const PsiSet* pout,
                                              const unsigned char* prv_base, const float* en_prv, const float* en_cur,
                                              int hi, int mi, int ni, int i, int j, int k, float* fhx, float* fhy,
                                              float* fhz, long long row, int probes) {
    const StepParams& p = *pp;
    const StageView<T> prv(prv_base);
    constexpr int NF = T::N_FLOATS;
    const int cls = prv.m()[mi] & 0xff;
    HNbr n;
    n.hx = prv.h(0)[hi]; n.hy = prv.h(1)[hi]; n.hz = prv.h(2)[hi];
    n.ex = en_prv[ni]; n.ey = en_prv[NF + ni]; n.ez = en_prv[2 * NF + ni];
    n.ey_kp = en_cur[NF + ni]; n.ez_jp = en_prv[2 * NF + ni + T::NW];
    n.ez_ip = en_prv[2 * NF + ni + 1]; n.ex_kp = en_cur[ni];
    n.ex_jp = en_prv[ni + T::NW]; n.ey_ip = en_prv[NF + ni + 1];
    h_cells(p, cls, i, j, k, n);
    const PsiIO io{pin->f, pout->f, true};
    float out[3], pre[3];
    h_update<false>(p, n, i, j, k, io, out, pre);
    const long long q = (long long)k * p.g.plane + (long long)j * p.g.pitch + i;
    fhx[q] = out[0]; fhy[q] = out[1]; fhz[q] = out[2];
    if (probes) {
        sample(p, row, 3, i, j, k, pre[0]); sample(p, row, 4, i, j, k, pre[1]); sample(p, row, 5, i, j, k, pre[2]);
    }
}

// One E node of the general sweep from the ring: table update for fast-path and interface nodes,
// e_update for background CPML nodes (inline), e_general for the rest. Returns false when
// e_general has written the node's results itself; otherwise v holds the new E and pre the values
// before the CPML corrections (the probe samples). write: store the node's CPML memory (own nodes;
// recomputed halo nodes only read it).
template <class T>
__device__ __forceinline__ bool e_node_ring(const StepParams& p, const PsiSet& pin, const PsiSet& pout,
                                            const unsigned char* cur_base, const unsigned char* prv_base, int hi, int ei,
                                            int mi, int nn, float* en_cur, int i, int j, int k, long long m, int lumped,
                                            bool write, const FieldPtrs& fo, long long row, int probes, float3& v,
                                            float3& pre) {
    const StageView<T> cur(cur_base), prv(prv_base);
    const int c = cur.m()[mi];
    const float hx = cur.h(0)[hi], hy = cur.h(1)[hi], hz = cur.h(2)[hi];
    const float ex = cur.e(0)[ei], ey = cur.e(1)[ei], ez = cur.e(2)[ei];
    if (c < kRecGeneral) {
        float out[3];
        e_update_interior(p, c, ex, ey, ez, __fsub_rn(hz, cur.h(2)[hi - T::HW]), __fsub_rn(hy, prv.h(1)[hi]),
                          __fsub_rn(hx, prv.h(0)[hi]), __fsub_rn(hz, cur.h(2)[hi - 1]), __fsub_rn(hy, cur.h(1)[hi - 1]),
                          __fsub_rn(hx, cur.h(0)[hi - T::HW]), out);
        v = make_float3(out[0], out[1], out[2]);
        pre = v;
        return true;
    }
    if ((c & 0xff) == kUniformGeneral + p.bg.mat) {
        ENbr n;
        n.hx = hx; n.hy = hy; n.hz = hz;
        n.hx_jm = cur.h(0)[hi - T::HW]; n.hx_km = prv.h(0)[hi];
        n.hy_im = cur.h(1)[hi - 1]; n.hy_km = prv.h(1)[hi];
        n.hz_im = cur.h(2)[hi - 1]; n.hz_jm = cur.h(2)[hi - T::HW];
        n.ex = ex; n.ey = ey; n.ez = ez;
        n.m0 = n.mi = n.mj = n.mk = n.mij = n.mik = n.mjk = p.bg.mat;
        const PsiIO io{pin.f, pout.f, write};
        float out[3], pr[3];
        e_update<false, false, false, true>(p, n, i, j, k, m, false, io, out, pr);
        v = make_float3(out[0], out[1], out[2]);
        pre = make_float3(pr[0], pr[1], pr[2]);
        return true;
    }
    e_general<T>(&p, &pin, &pout, cur_base, prv_base, hi, ei, mi, nn, en_cur, i, j, k, m, lumped, write ? 1 : 0, fo.ex,
                 fo.ey, fo.ez, row, probes);
    return false;
}

// One H node of the general sweep: old H from the ring, new E from the planes k and k+1. Returns
// false when h_general has stored the node itself.
template <class T>
__device__ __forceinline__ bool h_node_ring(const StepParams& p, const PsiSet& pin, const PsiSet& pout,
                                            const unsigned char* prv_base, const float* en_prv, const float* en_cur,
                                            int hi, int mi, int ni, int i, int j, int k, const FieldPtrs& fo,
                                            long long row, int probes, float3& v, float3& pre) {
    constexpr int NF = T::N_FLOATS;
    const StageView<T> prv(prv_base);
    const int c = prv.m()[mi];
    const float hx = prv.h(0)[hi], hy = prv.h(1)[hi], hz = prv.h(2)[hi];
    const float ex = en_prv[ni], ey = en_prv[NF + ni], ez = en_prv[2 * NF + ni];
    const float ey_kp = en_cur[NF + ni], ez_jp = en_prv[2 * NF + ni + T::NW], ez_ip = en_prv[2 * NF + ni + 1];
    const float ex_kp = en_cur[ni], ex_jp = en_prv[ni + T::NW], ey_ip = en_prv[NF + ni + 1];
    if (c < kRecGeneral) {
        float out[3];
        h_update_interior(p, c, hx, hy, hz, __fsub_rn(ey_kp, ey), __fsub_rn(ez_jp, ez), __fsub_rn(ez_ip, ez),
                          __fsub_rn(ex_kp, ex), __fsub_rn(ex_jp, ex), __fsub_rn(ey_ip, ey), out);
        v = make_float3(out[0], out[1], out[2]);
        pre = v;
        return true;
    }
    if ((c & 0xff) == kUniformGeneral + p.bg.mat) {
        HNbr n;
        n.hx = hx; n.hy = hy; n.hz = hz;
        n.ex = ex; n.ey = ey; n.ez = ez;
        n.ey_kp = ey_kp; n.ez_jp = ez_jp; n.ez_ip = ez_ip; n.ex_kp = ex_kp; n.ex_jp = ex_jp; n.ey_ip = ey_ip;
        n.m0 = n.mi = n.mj = n.mk = p.bg.mat;
        const PsiIO io{pin.f, pout.f, true};
        float out[3], pr[3];
        h_update<false, true>(p, n, i, j, k, io, out, pr);
        v = make_float3(out[0], out[1], out[2]);
        pre = make_float3(pr[0], pr[1], pr[2]);
        return true;
    }
    h_general<T>(&p, &pin, &pout, prv_base, en_prv, en_cur, hi, mi, ni, i, j, k, fo.hx, fo.hy, fo.hz, row, probes);
    return false;
}

}  // namespace

// Interior sweep over `items` (int4 {x0, y0, k0, k1}, one per CTA; the planner puts only interior
// columns and planes here). Per-thread ring offsets are fixed for the whole item, nothing is bounds-
// checked, and the per-plane lumped / probe flags are read once into shared memory.
__global__ void __launch_bounds__(NTH, FDTD_FUSED_MIN_BLOCKS)
k_sweep_interior(const __grid_constant__ TileMaps maps, const __grid_constant__ StepParams p, FieldPtrs fo,
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

// General sweep over `items` ({x0 | w << 16, y0 | h << 16, k0, k1}: a T::TX x T::TY column of which
// the first w columns and h rows are the item's): the item's nodes are stored, the other in-grid
// nodes of the column and its halo are recomputed for the H update (their CPML memory read, not
// written), and nodes outside the grid are skipped (zero in the new-E planes; the boundary masks
// keep every value that would read them out of the result).
template <class T>
__global__ void __launch_bounds__(NTH, FDTD_GENERAL_MIN_BLOCKS)
k_sweep_general(const __grid_constant__ TileMaps maps, const __grid_constant__ StepParams p,
                const __grid_constant__ PsiSet pin, const __grid_constant__ PsiSet pout, FieldPtrs fo,
                const int4* __restrict__ items, long long m) {
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
    const int x0 = it.x & 0xffff, w = it.x >> 16, y0 = it.y & 0xffff, h = it.y >> 16, k0 = it.z, k1 = it.w;
    const int kfirst = k0 - 1, klast = k1;
    const long long row = m % p.ring_cap;
    const int i = x0 + tx, j = y0 + ty;
    const int xoff = x0 & 7;
    const int hi = (ty + 1) * HW + tx + 4, ei = ty * EW + tx, mi = (ty + 1) * MW + tx + xoff, ni = ty * NW + tx;
    // rows r = 0, 1 (j and j + RSTEP): bit r of `inside` when the node lies in the grid, of `own`
    // when it is the item's
    const int inside = (i < g.nx) ? ((j < g.ny ? 1 : 0) | (j + RSTEP < g.ny ? 2 : 0)) : 0;
    const int own = (tx < w) ? ((ty < h ? 1 : 0) | (ty + RSTEP < h ? 2 : 0)) : 0;
    const bool halo = tid < T::NHALO;
    const int hpx = tid < TX ? tid : TX, hpy = tid < TX ? TY : tid - TX;
    const int hhi = (hpy + 1) * HW + hpx + 4, hei = hpy * EW + hpx, hmi = (hpy + 1) * MW + hpx + xoff, hni = hpy * NW + hpx;
    const bool halo_inside = halo && x0 + hpx < g.nx && y0 + hpy < g.ny;
    const long long n_own = (long long)j * g.pitch + i;

    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int q = tid; q <= klast - kfirst; q += NTH) {  // klast - kfirst < kMaxItemPlanes (plan_chunk)
        const int k = kfirst + q;
        pflags[q] = (k < 0 || k >= g.nz) ? 0
                                         : (p.lumped_k[k] < p.lumped_k[k + 1] ? 1 : 0) | (p.probe_k[k] < p.probe_k[k + 1] ? 2 : 0);
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
        const unsigned char* cur_base = smem + s_cur * T::STAGE_BYTES;
        const unsigned char* prv_base = smem + s_prv * T::STAGE_BYTES;
        float* en_cur = enew + (k & 1) * 3 * NF;
        const float* en_prv = enew + ((k - 1) & 1) * 3 * NF;
        if (k >= k0) {
            // ---- E(k): the column's nodes (the item's stored below plane k1), then the halo ----
            const int fl = pflags[k - kfirst];
            const bool plane_in = k < g.nz;
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const int o = r * RSTEP;
                const int nn = ni + o * NW;
                float3 v = make_float3(0.f, 0.f, 0.f), pre;
                bool mine = true;  // results still to be written here
                const bool store = ((own >> r) & 1) && k < k1;
                if (plane_in && ((inside >> r) & 1)) {
                    mine = e_node_ring<T>(p, pin, pout, cur_base, prv_base, hi + o * HW, ei + o * EW, mi + o * MW, nn,
                                          en_cur, i, j + o, k, m, fl & 1, store, fo, row, fl & 2, v, pre);
                    if (mine && store) {
                        store3(fo.ex, fo.ey, fo.ez, (long long)k * g.plane + n_own + (long long)o * g.pitch, v);
                        if (fl & 2) {
                            sample(p, row, 0, i, j + o, k, pre.x); sample(p, row, 1, i, j + o, k, pre.y);
                            sample(p, row, 2, i, j + o, k, pre.z);
                        }
                    }
                }
                if (mine) { en_cur[nn] = v.x; en_cur[NF + nn] = v.y; en_cur[2 * NF + nn] = v.z; }
            }
            if (halo) {
                float3 v = make_float3(0.f, 0.f, 0.f), pre;
                bool mine = true;
                if (plane_in && halo_inside)
                    mine = e_node_ring<T>(p, pin, pout, cur_base, prv_base, hhi, hei, hmi, hni, en_cur, x0 + hpx, y0 + hpy,
                                          k, m, fl & 1, false, fo, row, 0, v, pre);
                if (mine) { en_cur[hni] = v.x; en_cur[NF + hni] = v.y; en_cur[2 * NF + hni] = v.z; }
            }
        }
        if (k > k0) {
            // ---- H(k-1) of the item's nodes from E(k-1), E(k) and the old H(k-1) ----
            const int kh = k - 1;
            const int fl = pflags[kh - kfirst];
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                if (!((own >> r) & 1)) continue;
                const int o = r * RSTEP;
                float3 v, pre;
                if (h_node_ring<T>(p, pin, pout, prv_base, en_prv, en_cur, hi + o * HW, mi + o * MW, ni + o * NW, i, j + o,
                                   kh, fo, row, fl & 2, v, pre)) {
                    store3(fo.hx, fo.hy, fo.hz, (long long)kh * g.plane + n_own + (long long)o * g.pitch, v);
                    if (fl & 2) {
                        sample(p, row, 3, i, j + o, kh, pre.x); sample(p, row, 4, i, j + o, kh, pre.y);
                        sample(p, row, 5, i, j + o, kh, pre.z);
                    }
                }
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

int fused_smem_bytes() { return TileW::SMEM; }

cudaError_t fused_configure() {
    cudaError_t e = cudaFuncSetAttribute(k_sweep_interior, cudaFuncAttributeMaxDynamicSharedMemorySize, TileW::SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_sweep_general<TileW>, cudaFuncAttributeMaxDynamicSharedMemorySize, TileW::SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_sweep_general<TileN>, cudaFuncAttributeMaxDynamicSharedMemorySize, TileN::SMEM);
    return e;
}

// One fused step: per-node E of the shell items (tiles around a design region), the design
// region's and the plates' E, the three sweeps, per-node H of the shell items (which reads the new
// E of its neighbours, written by the sweeps).
cudaError_t launch_fused(const FusedMaps& maps, const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo,
                         const PsiSet& psi_in, const PsiSet& psi_out, long long m, const FusedWork& w, cudaStream_t st) {
    cudaError_t e = launch_shell(true, p, fi, fo, psi_in, psi_out, w.general, w.n_general, m, st);
    if (e == cudaSuccess) e = launch_design_e(p, fi, fo, psi_in, psi_out, m, st);
    if (e == cudaSuccess) e = launch_plate_e(p, fi, fo, psi_in, psi_out, m, st);
    if (e != cudaSuccess) return e;
    if (w.n_interior > 0) k_sweep_interior<<<w.n_interior, NTH, TileW::SMEM, st>>>(maps.wide, p, fo, w.interior, m);
    if (w.n_wide > 0)
        k_sweep_general<TileW><<<w.n_wide, NTH, TileW::SMEM, st>>>(maps.wide, p, psi_in, psi_out, fo, w.wide, m);
    if (w.n_narrow > 0)
        k_sweep_general<TileN><<<w.n_narrow, NTH, TileN::SMEM, st>>>(maps.narrow, p, psi_in, psi_out, fo, w.narrow, m);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_shell(false, p, fi, fo, psi_in, psi_out, w.general, w.n_general, m, st);
}

namespace {

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                              const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Tensor maps of one tile shape: H tiles with a one-node halo (x widened to 16-byte boundaries),
// old-E tiles, coefficient-row tiles. Coordinates outside the arrays load as zeros.
template <class T>
int encode_tile_maps(TileMaps* out, const DeviceGrid& g, float* const h[3], float* const e[3], const uint16_t* rec,
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
    const EncodeFn encode = reinterpret_cast<EncodeFn>(encode_fn);
    if (encode_tile_maps<TileW>(&out->wide, g, h, e, rec, encode) != 0) return -1;
    return encode_tile_maps<TileN>(&out->narrow, g, h, e, rec, encode);
}

}  // namespace fdtd
