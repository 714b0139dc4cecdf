// Fused schedule: one z-marching sweep per time step over ping-pong field buffers.
//
// Every CTA owns a 32 x 8 column of nodes and a chunk of planes [k0, k1). Planes stream through a
// 5-stage shared-memory ring filled by TMA (cp.async.bulk.tensor, 3-D tiles from this GPU's HBM,
// two planes ahead of the one being computed). At plane k the CTA
//   1. computes E(k) on the tile plus one column / row beyond its high x / y edges (the H update of
//      the tile needs those E values; the extra ones are recomputed from the old fields instead of
//      being exchanged), storing only the tile's own nodes;
//   2. computes H(k-1) of its own nodes from E(k-1), E(k) (shared memory) and H(k-1) (the ring).
// Old fields and old CPML memory are read from buffer A, new ones written to buffer B, so CTAs
// never see each other's partial results. Each field value crosses HBM once per step in each
// direction: 24 B read + 24 B written per cell, plus the uint8 material index and the CPML memory.
//
// The per-node arithmetic is e_update / h_update (yee_common.cuh), shared with the two-pass
// schedule, so both produce identical bits. All waits on the TMA barriers are bounded: on timeout
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

struct StageView {
    const float* h[3];
    const float* e[3];
    const uint8_t* m;
    __device__ StageView(const unsigned char* base) {
        for (int c = 0; c < 3; ++c) {
            h[c] = reinterpret_cast<const float*>(base + c * H_BYTES);
            e[c] = reinterpret_cast<const float*>(base + 3 * H_BYTES + c * E_BYTES);
        }
        m = base + 3 * H_BYTES + 3 * E_BYTES;
    }
};

}  // namespace

__global__ void __launch_bounds__(NTH, 3)
k_fused(const __grid_constant__ FusedMaps maps, StepParams p, FieldPtrs fo, PsiSet psi_in, PsiSet psi_out,
        long long m, int kc) {
    extern __shared__ __align__(128) unsigned char smem[];
    float* enew = reinterpret_cast<float*>(smem + NSTAGE * STAGE_BYTES);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + NSTAGE * STAGE_BYTES + ENEW_BYTES);
    const DeviceGrid& g = p.g;
    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int k0 = blockIdx.z * kc;
    const int k1 = min(g.nz, k0 + kc);
    const int kfirst = k0 - 1, klast = k1;  // planes streamed through the ring
    const long long row = m % p.ring_cap;

    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    auto stage_of = [&](int k) { return (k - kfirst) % NSTAGE; };
    auto parity_of = [&](int k) { return (uint32_t)(((k - kfirst) / NSTAGE) & 1); };
    auto issue = [&](int k) {
        const int s = stage_of(k);
        unsigned char* st = smem + s * STAGE_BYTES;
        mbar_expect_tx(&bars[s], TX_BYTES);
        for (int c = 0; c < 3; ++c) tma_load_3d(st + c * H_BYTES, &maps.h[c], &bars[s], x0 - 4, y0 - 1, k);
        for (int c = 0; c < 3; ++c) tma_load_3d(st + 3 * H_BYTES + c * E_BYTES, &maps.e[c], &bars[s], x0, y0, k);
        tma_load_3d(st + 3 * H_BYTES + 3 * E_BYTES, &maps.mat, &bars[s], x0 - 16, y0 - 1, k);
    };
    if (tid == 0)
        for (int k = kfirst; k < kfirst + AHEAD && k <= klast; ++k) issue(k);

    const PsiIO io_core{psi_in.f, psi_out.f, true};
    const PsiIO io_halo{psi_in.f, psi_out.f, false};

    for (int k = kfirst; k <= klast; ++k) {
        if (tid == 0 && k + AHEAD <= klast) {
            fence_proxy_async();  // generic reads of the recycled stage precede the async writes
            issue(k + AHEAD);
        }
        const bool ok = mbar_wait(&bars[stage_of(k)], parity_of(k));
        const StageView cur(smem + stage_of(k) * STAGE_BYTES);
        float* en_cur = enew + (k & 1) * 3 * N_FLOATS;
        const float* en_prv = enew + ((k - 1) & 1) * 3 * N_FLOATS;

        // ---- E(k) on the tile and its high-x column / high-y row ----
        if (k >= k0 && k < g.nz) {
            const StageView prv(smem + stage_of(k - 1) * STAGE_BYTES);
            const bool store = k < k1;
            // plane-uniform facts: lumped edges or probes in this plane, plane inside the z range of
            // the fast path (1 <= k <= nz-2, outside the z slabs)
            const bool plane_lumped = p.lumped_k[k] < p.lumped_k[k + 1];
            const bool plane_probe = p.probe_k[k] < p.probe_k[k + 1];
            const bool plane_fast = !plane_lumped && k >= 1 && k <= g.nz - 2 && !in_slab(k, g.nz, g.pzn, g.pzp);
            for (int pos = tid; pos < N_FLOATS; pos += NTH) {
                int px, py;
                if (pos < NTH) { px = pos % TX; py = pos / TX; }
                else {
                    const int h = pos - NTH;
                    if (h < TY + 1) { px = TX; py = h; } else { px = h - (TY + 1); py = TY; }
                }
                const int i = x0 + px, j = y0 + py;
                if (i >= g.nx || j >= g.ny) continue;
                const int hi = (py + 1) * HW + px + 4;   // (i, j) in the H tile
                const int ei = py * EW + px;             // (i, j) in the old-E tile
                const int mi = (py + 1) * MW + px + 16;  // cell (i, j) in the material tile
                ENbr nb;
                nb.ex = cur.e[0][ei]; nb.ey = cur.e[1][ei]; nb.ez = cur.e[2][ei];
                nb.hx = cur.h[0][hi]; nb.hy = cur.h[1][hi]; nb.hz = cur.h[2][hi];
                nb.hx_jm = cur.h[0][hi - HW]; nb.hx_km = prv.h[0][hi];
                nb.hy_im = cur.h[1][hi - 1]; nb.hy_km = prv.h[1][hi];
                nb.hz_im = cur.h[2][hi - 1]; nb.hz_jm = cur.h[2][hi - HW];
                nb.m0 = cur.m[mi]; nb.mi = cur.m[mi - 1]; nb.mj = cur.m[mi - MW]; nb.mij = cur.m[mi - MW - 1];
                nb.mk = prv.m[mi]; nb.mik = prv.m[mi - 1]; nb.mjk = prv.m[mi - MW];
                const bool own = store && pos < NTH;
                float out[3], pre[3];
                const bool fast = plane_fast && i >= 1 && i <= g.nx - 2 && j >= 1 && j <= g.ny - 2 &&
                                  !in_slab(i, g.nx, g.pxn, g.pxp) && !in_slab(j, g.ny, g.pyn, g.pyp) && e_fast_ok(nb);
                if (fast) {
                    e_update_fast(p, nb, out);
                    pre[0] = out[0]; pre[1] = out[1]; pre[2] = out[2];
                } else {
                    e_update(p, nb, i, j, k, m, own ? io_core : io_halo, out, pre);
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
                const StageView hst(smem + stage_of(kh) * STAGE_BYTES);
                const StageView mst(smem + stage_of(kh - 1) * STAGE_BYTES);
                const int hi = (ty + 1) * HW + tx + 4;
                const int mi = (ty + 1) * MW + tx + 16;
                const int ni = ty * NW + tx;
                HNbr nb;
                nb.hx = hst.h[0][hi]; nb.hy = hst.h[1][hi]; nb.hz = hst.h[2][hi];
                nb.ex = en_prv[ni]; nb.ey = en_prv[N_FLOATS + ni]; nb.ez = en_prv[2 * N_FLOATS + ni];
                nb.ey_kp = en_cur[N_FLOATS + ni];
                nb.ex_kp = en_cur[ni];
                nb.ez_jp = en_prv[2 * N_FLOATS + ni + NW];
                nb.ex_jp = en_prv[ni + NW];
                nb.ez_ip = en_prv[2 * N_FLOATS + ni + 1];
                nb.ey_ip = en_prv[N_FLOATS + ni + 1];
                nb.m0 = hst.m[mi]; nb.mi = hst.m[mi - 1]; nb.mj = hst.m[mi - MW]; nb.mk = mst.m[mi];
                float out[3], pre[3];
                const bool fast = i >= 1 && i <= g.nx - 2 && j >= 1 && j <= g.ny - 2 && kh >= 1 && kh <= g.nz - 2 &&
                                  !in_slab(i, g.nx, g.pxn, g.pxp) && !in_slab(j, g.ny, g.pyn, g.pyp) &&
                                  !in_slab(kh, g.nz, g.pzn, g.pzp) && h_fast_ok(nb);
                if (fast) {
                    h_update_fast(p, nb, out);
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
                for (int q = k + 1; q <= min(klast, k + AHEAD); ++q) mbar_wait(&bars[stage_of(q)], parity_of(q));
            }
            __syncthreads();
            return;
        }
    }
}

int fused_smem_bytes() { return SMEM_BYTES; }
int fused_tile_x() { return TX; }
int fused_tile_y() { return TY; }

cudaError_t fused_configure() {
    return cudaFuncSetAttribute(k_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
}

cudaError_t launch_fused(const FusedMaps& maps, const StepParams& p, const FieldPtrs& fo, const PsiSet& psi_in,
                         const PsiSet& psi_out, long long m, int kc, cudaStream_t st) {
    dim3 grid((p.g.nx + TX - 1) / TX, (p.g.ny + TY - 1) / TY, (p.g.nz + kc - 1) / kc);
    k_fused<<<grid, NTH, SMEM_BYTES, st>>>(maps, p, fo, psi_in, psi_out, m, kc);
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

}  // namespace fdtd
