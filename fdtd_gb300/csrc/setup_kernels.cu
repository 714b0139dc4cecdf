// Setup kernels: CPML profiles, per-material coefficient tables, lumped-edge coefficients,
// material painting and fills. They run once per simulation (fdtd_prepare).
//
// The CPML profile and lumped-element expressions are evaluated on the device with the same
// float/double mix and the same device powf/expf as the reference's setABCPML and defineSourceZ /
// defineResistor, so the resulting tables equal the reference's bit for bit.
#include "yee_common.cuh"
#include "yee_kernels.h"

namespace fdtd {

// Planes per CTA of the grid-sized setup kernels (one node per thread and plane).
constexpr int kSetupPlanes = 8;

// One axis of setABCPML (fdtdrav.h:1774-1891 for x_n, 1912-1941 for x_p, and the y / z mirrors).
// prof = {b_e, a_e, b_m, a_m, kappa_e, kappa_m}, each n entries. Nodes outside both slabs keep
// b = a = 1.2e-38 (setZero) and kappa = 1.
// r0 > 0 (not the reference's): sigma_max from the reflection coefficient r0 of a slab of P cells
// with grading order m, sigma_max = -(m + 1) ln(r0) / (2 eta0 P delta), eta0 = sqrt(mu0 / eps0)
// (Gedney's polynomial grading); kappa, alpha and the recurrences as the reference's.
__global__ void k_cpml_axis(float* be, float* ae, float* bm, float* am, float* ke, float* km, int n,
                            int pn_i, int pp_i, float delta, float dt, float eps_0, float mu_0, float pi, float r0) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    // parameters of fdtdrav.h:1774-1812, as float locals
    float npml = 3;
    float sigma_factor = 1.5;
    float kappa_max = 5;
    float alpha_max = 0.05;
    float alpha_min = 0.00;
    float sigma_opt = (npml + 1) / (150 * pi * 1 * delta);
    float sigma_max = sigma_factor * sigma_opt;
    const float pn = (float)pn_i, pp = (float)pp_i;
    float roe, rom;
    bool in = false;
    if (q < pn_i) {
        roe = (pn - q - 0.75) / pn;
        rom = (pn - q - 0.25) / pn;
        in = true;
        if (r0 > 0.f) sigma_max = -(npml + 1) * logf(r0) / (2.0f * sqrtf(mu_0 / eps_0) * pn * delta);
    } else if (q >= n - pp_i) {
        roe = (q - (n - pp - 1) - 0.75) / pp;
        rom = (q - (n - pp - 1) - 0.25) / pp;
        in = true;
        if (r0 > 0.f) sigma_max = -(npml + 1) * logf(r0) / (2.0f * sqrtf(mu_0 / eps_0) * pp * delta);
    }
    if (!in) {
        be[q] = kTiny; ae[q] = kTiny; bm[q] = kTiny; am[q] = kTiny; ke[q] = 1.0f; km[q] = 1.0f;
        return;
    }
    float sigma_pe = sigma_max * powf(roe, npml);
    float sigma_pm = sigma_max * powf(rom, npml);
    sigma_pm = sigma_pm * (mu_0 / eps_0);
    float kappa_e = 1 + (kappa_max - 1) * powf(roe, npml);
    float kappa_m = 1 + (kappa_max - 1) * powf(rom, npml);
    float alpha_e = alpha_min + (alpha_max - alpha_min) * (1 - roe);
    float alpha_m = alpha_min + (alpha_max - alpha_min) * (1 - rom);
    alpha_m = alpha_m * (mu_0 / eps_0);
    float b_e = expf((-dt / eps_0) * ((sigma_pe / kappa_e) + alpha_e));
    float a_e = (1 / delta) * (b_e - 1) * sigma_pe / (kappa_e * (sigma_pe + kappa_e * alpha_e));
    float b_m = expf((-dt / mu_0) * ((sigma_pm / kappa_m) + alpha_m));
    float a_m = (1 / delta) * (b_m - 1) * sigma_pm / (kappa_m * (sigma_pm + kappa_m * alpha_m));
    be[q] = b_e; ae[q] = a_e; bm[q] = b_m; am[q] = a_m; ke[q] = kappa_e; km[q] = kappa_m;
}

cudaError_t launch_cpml_profiles(const DeviceGrid& g, float pi, float r0, float* const prof[18], cudaStream_t st) {
    const int ns[3] = {g.nx, g.ny, g.nz};
    const int pn[3] = {g.pxn, g.pyn, g.pzn};
    const int pp[3] = {g.pxp, g.pyp, g.pzp};
    const float d[3] = {g.dx, g.dy, g.dz};
    for (int a = 0; a < 3; ++a) {
        float* const* P = prof + 6 * a;
        k_cpml_axis<<<(ns[a] + 127) / 128, 128, 0, st>>>(P[0], P[1], P[2], P[3], P[4], P[5], ns[a], pn[a], pp[a],
                                                         d[a], g.dt, g.eps0, g.mu0, pi, r0);
    }
    return cudaGetLastError();
}

// Coefficients of edges whose surrounding cells share material m (the averages of four / two equal
// values computed with the reference's formulas), plus the default entry for H faces on the low
// boundary of their axis (mu = 1, sigma_m = 1.2e-38).
__global__ void k_material_tables(const MatProps* props, int n, MatCoef* coef, DeviceGrid g) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m > kMaxMaterials) return;
    MatCoef c;
    const float dp_e[3] = {g.dy, g.dz, g.dx}, dm_e[3] = {g.dz, g.dx, g.dy};
    const float dp_h[3] = {g.dz, g.dx, g.dy}, dm_h[3] = {g.dy, g.dz, g.dx};
    for (int q = 0; q < 3; ++q) {  // component q averages the values of axis q
        MatAxis a{1.0f, kTiny, 1.0f, kTiny};
        if (m < n && m != kDefaultEntry) a = props[m].a[q];
        const float eps = avg4(a.eps, a.eps, a.eps, a.eps);
        const float sig = avg4(a.sig, a.sig, a.sig, a.sig);
        const float mu = m == kDefaultEntry ? 1.0f : harm2(a.mu, a.mu);
        const float sm = m == kDefaultEntry ? kTiny : harm2(a.sigm, a.sigm);
        Coef3 e = coef3(eps, sig, g.dt, g.eps0, dp_e[q], dm_e[q]);
        c.e[q] = make_float4(e.a, e.bp, e.bm, 0.0f);
        Coef3 h = coef3(mu, sm, g.dt, g.mu0, dp_h[q], dm_h[q]);
        c.h[q] = make_float4(h.a, h.bp, h.bm, 0.0f);
    }
    coef[m] = c;
}

cudaError_t launch_material_tables(const DeviceGrid& g, const MatProps* props, int n, MatCoef* coef,
                                   cudaStream_t st) {
    k_material_tables<<<(kMaxMaterials + 1 + 127) / 128, 128, 0, st>>>(props, n, coef, g);
    return cudaGetLastError();
}

// Lumped-edge coefficient overrides (defineSourceZ fdtdrav.h:1368-1426 for sources,
// defineResistor fdtdrav.h:1429-1483 for resistors), from the edge-averaged eps_z / sigma_z; for
// Ex edges defineSourceX's (fdtdrav.h:1311-1365) from eps_x / sigma_x, with its per-component
// resistance (1 + je - js)(1 + ke - ks) / (ie - is) * rs and factor dt dx / (r dz dy).
// boxes: per owner {is,js,ks,ie,je,ke}; owner[e] = index of the element an edge belongs to.
__global__ void k_lumped_coefs(DeviceGrid g, const uint8_t* mat, const MatProps* props, LumpedEdge* edges,
                               const int* boxes, const float* resist, const int* owner, int n_edges) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_edges) return;
    LumpedEdge L = edges[e];
    const int* b = boxes + 6 * owner[e];
    float dt = g.dt, dx = g.dx, dy = g.dy, dz = g.dz, eps_0 = g.eps0;
    float rs = resist[owner[e]];
    float _is = (float)b[0], _js = (float)b[1], _ks = (float)b[2];
    float _ie = (float)b[3], _je = (float)b[4], _ke = (float)b[5];
    const long long n = (long long)L.k * g.plane + (long long)L.j * g.pitch + L.i;
    if (L.comp == 0) {
        float r_comp = (1 + _je - _js) * (1 + _ke - _ks) / (_ie - _is);
        r_comp = r_comp * rs;
        float rfactor = (dt * dx) / (r_comp * dz * dy);
        // eps_x / sigma_x of the edge: average of cells (i,j,k), (i,j-1,k), (i,j,k-1), (i,j-1,k-1)
        const MatAxis a = props[mat[n]].a[0], bb = props[mat[n - g.pitch]].a[0], c = props[mat[n - g.plane]].a[0],
                      d = props[mat[n - g.pitch - g.plane]].a[0];
        float eps_x = avg4(a.eps, bb.eps, c.eps, d.eps);
        float sig_x = avg4(a.sig, bb.sig, c.sig, d.sig);
        float den = __fadd_rn(__fmaf_rn(2.0f * eps_x, eps_0, __fmul_rn(dt, sig_x)), rfactor);
        float num = __fsub_rn(__fmaf_rn(2.0f * eps_x, eps_0, -__fmul_rn(dt, sig_x)), rfactor);
        L.ceze = __fdiv_rn(num, den);
        L.cezhy = __fdiv_rn(__fdiv_rn(2.0f * dt, dy), den);
        L.cezhx = __fdiv_rn(__fdiv_rn(-2.0f * dt, dz), den);
        L.cezj = 0.0f;  // the reference computes Cexj but never injects (calc_e, fdtdrav.h:681-685)
        edges[e] = L;
        return;
    }
    float r_comp = (1 + _ie - _is) * (1 + _je - _js) / (_ke - _ks);
    r_comp = r_comp * rs;
    float rfactor = (dt * dz) / (r_comp * dx * dy);
    float rfactor_aux = (r_comp * dx * dy);
    // eps_z / sigma_z of the edge: average of cells (i,j), (i-1,j), (i,j-1), (i-1,j-1) in plane k
    const MatAxis a = props[mat[n]].a[2], bb = props[mat[n - 1]].a[2], c = props[mat[n - g.pitch]].a[2],
                  d = props[mat[n - 1 - g.pitch]].a[2];
    float eps_z = avg4(a.eps, bb.eps, c.eps, d.eps);
    float sig_z = avg4(a.sig, bb.sig, c.sig, d.sig);
    float den = __fadd_rn(__fmaf_rn(2.0f * eps_z, eps_0, __fmul_rn(dt, sig_z)), rfactor);
    float num = __fsub_rn(__fmaf_rn(2.0f * eps_z, eps_0, -__fmul_rn(dt, sig_z)), rfactor);
    L.ceze = __fdiv_rn(num, den);
    L.cezhy = __fdiv_rn(__fdiv_rn(2.0f * dt, dx), den);
    L.cezhx = __fdiv_rn(__fdiv_rn(-2.0f * dt, dy), den);
    L.cezj = L.source >= 0 ? __fdiv_rn(__fdiv_rn(-2.0f * dt, rfactor_aux), den) : 0.0f;
    edges[e] = L;
}

cudaError_t launch_lumped_coefs(const DeviceGrid& g, const uint8_t* mat, const MatProps* props,
                                LumpedEdge* edges, const int* boxes, const float* resist, const int* owner,
                                int n_edges, cudaStream_t st) {
    if (n_edges == 0) return cudaSuccess;
    k_lumped_coefs<<<(n_edges + 127) / 128, 128, 0, st>>>(g, mat, props, edges, boxes, resist, owner, n_edges);
    return cudaGetLastError();
}

// Kappa-divided curl coefficients of material `bg` along each axis (the division setABCPML applies
// in its slabs, fdtdrav.h:1893-1906; kappa = 1 elsewhere leaves the coefficient unchanged).
// out[axis][slot]: E then H slots as documented on BgCurl.
__global__ void k_bg_curl(const MatCoef* coef, int bg, DeviceGrid g, const float* const* kappa, float* const* out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int a = blockIdx.y;
    const int n = a == 0 ? g.nx : a == 1 ? g.ny : g.nz;
    if (q >= n) return;
    const MatCoef c = coef[bg];
    const float ke = kappa[2 * a][q], km = kappa[2 * a + 1][q];
    // E slots: x {Ey minus, Ez plus}, y {Ex plus, Ez minus}, z {Ex minus, Ey plus}
    const float e0[3] = {c.e[1].z, c.e[0].y, c.e[0].z};
    const float e1[3] = {c.e[2].y, c.e[2].z, c.e[1].y};
    // H slots: x {Hy plus, Hz minus}, y {Hx minus, Hz plus}, z {Hx plus, Hy minus}
    const float h0[3] = {c.h[1].y, c.h[0].z, c.h[0].y};
    const float h1[3] = {c.h[2].z, c.h[2].y, c.h[1].z};
    out[4 * a + 0][q] = __fdiv_rn(e0[a], ke);
    out[4 * a + 1][q] = __fdiv_rn(e1[a], ke);
    out[4 * a + 2][q] = __fdiv_rn(h0[a], km);
    out[4 * a + 3][q] = __fdiv_rn(h1[a], km);
}

cudaError_t launch_bg_curl(const DeviceGrid& g, const MatCoef* coef, int bg, const float* const* kappa_dev,
                           float* const* out_dev, cudaStream_t st) {
    const int nmax = max(g.nx, max(g.ny, g.nz));
    k_bg_curl<<<dim3((nmax + 127) / 128, 3), 128, 0, st>>>(coef, bg, g, kappa_dev, out_dev);
    return cudaGetLastError();
}

__global__ void k_fill(float* p, long long n, float v) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        p[q] = v;
}

cudaError_t launch_fill(float* p, long long n, float v, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    k_fill<<<(int)blocks, 256, 0, st>>>(p, n, v);
    return cudaGetLastError();
}

// The row padding of a field array (columns nx .. pitch-1 of every row) set to v.
__global__ void k_fill_padding(float* p, DeviceGrid g, float v) {
    const int w = g.pitch - g.nx;
    const long long n = (long long)w * g.ny * g.nz;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        p[(q / w) * g.pitch + g.nx + q % w] = v;
}

cudaError_t launch_fill_padding(float* p, const DeviceGrid& g, float v, cudaStream_t st) {
    const long long n = (long long)(g.pitch - g.nx) * g.ny * g.nz;
    if (n <= 0) return cudaSuccess;
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    k_fill_padding<<<(int)blocks, 256, 0, st>>>(p, g, v);
    return cudaGetLastError();
}

// setBrick (fdtdrav.h:1524-1571) on the material index: cells [is,ie) x [js,je) x [ks,ke).
__global__ void k_paint(uint8_t* mat, DeviceGrid g, int is, int js, int ks, int ie, int je, int ke, uint8_t v) {
    const int i = is + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = js + blockIdx.y * blockDim.y + threadIdx.y;
    const int k = ks + blockIdx.z;
    if (i < ie && j < je && k < ke) mat[(long long)k * g.plane + (long long)j * g.pitch + i] = v;
}

// Largest material index of the grid's cells (row padding excluded) into *out (atomicMax; *out
// starts at 0).
__global__ void k_index_max(const uint8_t* __restrict__ mat, DeviceGrid g, int* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    int v = 0;
    if (i < g.nx && j < g.ny)
        for (int k = blockIdx.z * kSetupPlanes, k1 = min(g.nz, k + kSetupPlanes); k < k1; ++k)
            v = max(v, (int)mat[(long long)k * g.plane + (long long)j * g.pitch + i]);
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v > 0) atomicMax(out, v);
}

cudaError_t launch_index_max(const uint8_t* mat, const DeviceGrid& g, int* out, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    const dim3 block(32, 8, 1), grid((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + kSetupPlanes - 1) / kSetupPlanes);
    k_index_max<<<grid, block, 0, st>>>(mat, g, out);
    return cudaGetLastError();
}

cudaError_t launch_paint(uint8_t* mat, const DeviceGrid& g, const int box[6], uint8_t value, cudaStream_t st) {
    const int is = box[0] < 0 ? 0 : box[0], js = box[1] < 0 ? 0 : box[1], ks = box[2] < 0 ? 0 : box[2];
    const int ie = box[3] > g.nx ? g.nx : box[3], je = box[4] > g.ny ? g.ny : box[4], ke = box[5] > g.nz ? g.nz : box[5];
    if (is >= ie || js >= je || ks >= ke) return cudaSuccess;
    dim3 block(32, 8, 1);
    dim3 grid((ie - is + 31) / 32, (je - js + 7) / 8, ke - ks);
    k_paint<<<grid, block, 0, st>>>(mat, g, is, js, ks, ie, je, ke, value);
    return cudaGetLastError();
}

}  // namespace fdtd

namespace fdtd {

// Node class (StepParams::cls): material id of nodes that take the fast path (interior, seven cells
// of one material below kUniformGeneral), kInterfaceNode for the other interior nodes,
// kUniformGeneral + m for the other nodes whose seven cells all hold material m, kGeneral
// otherwise. Lumped edges (k_class_lumped) and plates turn their nodes general afterwards.
// The seven cells are those the three E edge averages read, (i,j,k) (i-1,j,k) (i,j-1,k) (i,j,k-1)
// (i-1,j-1,k) (i-1,j,k-1) (i,j-1,k-1); the four cells of the H faces are among them.
// Nodes of the design region's edge box [dlo, dhi] get kDesignNode.
__device__ __forceinline__ void node_class(const uint8_t* __restrict__ mat, uint8_t* __restrict__ cls,
                                           const DeviceGrid& g, int4 dlo, int4 dhi, int i, int j, int k) {
    const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
    uint8_t c = kGeneral;
    // the seven cells as the general path reads them (cells outside the grid count as material 0)
    const long long R = g.pitch, P = g.plane;
    const int m0 = mat[n];
    const int mi = i > 0 ? mat[n - 1] : 0, mj = j > 0 ? mat[n - R] : 0, mk = k > 0 ? mat[n - P] : 0;
    const int mij = (i > 0 && j > 0) ? mat[n - 1 - R] : 0, mik = (i > 0 && k > 0) ? mat[n - 1 - P] : 0;
    const int mjk = (j > 0 && k > 0) ? mat[n - R - P] : 0;
    const bool uniform = mi == m0 && mj == m0 && mk == m0 && mij == m0 && mik == m0 && mjk == m0;
    const bool inner = interior(i, g.nx, g.pxn, g.pxp) && interior(j, g.ny, g.pyn, g.pyp) && interior(k, g.nz, g.pzn, g.pzp);
    if (uniform && inner && m0 < kUniformGeneral)
        c = (uint8_t)m0;  // fast path
    else if (inner)
        c = kInterfaceNode;  // table update with the coefficient row of its seven cells
    else if (uniform && m0 < kInterfaceNode - kUniformGeneral)
        c = (uint8_t)(kUniformGeneral + m0);  // general path without the cell-material loads
    if (i >= dlo.x && i <= dhi.x && j >= dlo.y && j <= dhi.y && k >= dlo.z && k <= dhi.z) c = kDesignNode;
    cls[n] = c;
}

// One CTA per 32 x 8 block of kSetupPlanes planes (one node per thread and plane): a CTA per
// block of one plane made the grid-sized setup kernels bound by launching CTAs.
__global__ void k_node_class(const uint8_t* __restrict__ mat, uint8_t* __restrict__ cls, DeviceGrid g, int4 dlo,
                             int4 dhi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nx || j >= g.ny) return;
    for (int k = blockIdx.z * kSetupPlanes, k1 = min(g.nz, k + kSetupPlanes); k < k1; ++k)
        node_class(mat, cls, g, dlo, dhi, i, j, k);
}

__global__ void k_class_lumped(uint8_t* cls, DeviceGrid g, const LumpedEdge* edges, int n_edges) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n_edges) cls[(long long)edges[q].k * g.plane + (long long)edges[q].j * g.pitch + edges[q].i] = kGeneral;
}

__global__ void k_class_nodes(uint8_t* cls, DeviceGrid g, const int4* nodes, int n, uint8_t value) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) cls[(long long)nodes[q].z * g.plane + (long long)nodes[q].y * g.pitch + nodes[q].x] = value;
}

cudaError_t launch_class_nodes(const DeviceGrid& g, const int4* nodes, int n, int value, uint8_t* cls, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_class_nodes<<<(n + 127) / 128, 128, 0, st>>>(cls, g, nodes, n, (uint8_t)value);
    return cudaGetLastError();
}

cudaError_t launch_node_class(const DeviceGrid& g, const uint8_t* mat, const LumpedEdge* edges, int n_edges,
                              const int* design_box, uint8_t* cls, cudaStream_t st) {
    const int4 dlo = design_box ? make_int4(design_box[0], design_box[1], design_box[2], 0) : make_int4(1, 1, 1, 0);
    const int4 dhi = design_box ? make_int4(design_box[3], design_box[4], design_box[5], 0) : make_int4(0, 0, 0, 0);
    dim3 block(32, 8, 1);
    dim3 grid((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + kSetupPlanes - 1) / kSetupPlanes);
    k_node_class<<<grid, block, 0, st>>>(mat, cls, g, dlo, dhi);
    if (n_edges > 0) k_class_lumped<<<(n_edges + 127) / 128, 128, 0, st>>>(cls, g, edges, n_edges);
    return cudaGetLastError();
}

}  // namespace fdtd

namespace fdtd {

// Interface rows. Every kInterfaceNode and kGeneral node is keyed by its seven cell materials,
// packed one byte each in the order (i,j,k) (i-1,j,k) (i,j-1,k) (i,j,k-1) (i-1,j-1,k) (i-1,j,k-1)
// (i,j-1,k-1), cells outside the grid as material 0 (as the general path reads them). The
// distinct keys are collected in a hash set on the device (open addressing, linear probing), only
// they are sorted on the host, and each of the first kMaxInterfaceRows gets the coefficient row
// the general path would build for such a node (e_coef / h_coef: table entries where an edge's
// cells agree, the reference's averages otherwise), so an interior node's update is the table
// form with the same bits. Interior nodes whose key has no row take the general path, with the
// same bits too. The rows of nodes in CPML slabs or on boundary planes (classes kGeneral and
// kUniformGeneral + m) serve the CPML sweep, which divides the curl coefficients by the CPML
// kappa and applies the boundary rules itself; the per-node kernels keep their general path for
// those nodes. Lumped edges get no row (launch_rec_general).
namespace {
__device__ __forceinline__ unsigned long long cell_key(const uint8_t* mat, const DeviceGrid& g, int i, int j, int k) {
    const long long R = g.pitch, P = g.plane, n = (long long)k * P + (long long)j * R + i;
    const unsigned long long m0 = mat[n], mi = i > 0 ? mat[n - 1] : 0, mj = j > 0 ? mat[n - R] : 0;
    const unsigned long long mk = k > 0 ? mat[n - P] : 0, mij = (i > 0 && j > 0) ? mat[n - 1 - R] : 0;
    const unsigned long long mik = (i > 0 && k > 0) ? mat[n - 1 - P] : 0, mjk = (j > 0 && k > 0) ? mat[n - R - P] : 0;
    return m0 | mi << 8 | mj << 16 | mk << 24 | mij << 32 | mik << 40 | mjk << 48;
}
constexpr unsigned long long kEmptyKey = ~0ull;  // keys use 56 bits
constexpr int kMaxProbes = 64;
__device__ __forceinline__ unsigned slot_of(unsigned long long key) {
    return (unsigned)((key * 0x9E3779B97F4A7C15ull) >> (64 - kIfaceTableBits));
}
// Slot of `key` in the set, or -1.
__device__ __forceinline__ int find_slot(const unsigned long long* __restrict__ table, unsigned long long key) {
    unsigned s = slot_of(key);
    for (int q = 0; q < kMaxProbes; ++q, s = (s + 1) & (kIfaceTableSize - 1)) {
        const unsigned long long v = table[s];
        if (v == key) return (int)s;
        if (v == kEmptyKey) return -1;
    }
    return -1;
}
}  // namespace

// Insert the key of every kInterfaceNode or kGeneral node into the set while it holds fewer than
// kIfaceTableSize / 2 keys (*filled counts them, a few more may land while it reaches that); a key
// that finds no room stays out (its nodes take the general path).
__device__ __forceinline__ void iface_insert(unsigned long long* table, int* filled, unsigned long long key) {
    unsigned s = slot_of(key);
    for (int q = 0; q < kMaxProbes; ++q, s = (s + 1) & (kIfaceTableSize - 1)) {
        const unsigned long long v = *(volatile unsigned long long*)(table + s);
        if (v == key) return;
        if (v != kEmptyKey) continue;
        if (*(volatile int*)filled >= kIfaceTableSize / 2) return;
        const unsigned long long old = atomicCAS(table + s, kEmptyKey, key);
        if (old == kEmptyKey) {
            atomicAdd(filled, 1);
            return;
        }
        if (old == key) return;
    }
}
__global__ void k_iface_insert(const uint8_t* __restrict__ cls, const uint8_t* __restrict__ mat, DeviceGrid g,
                               unsigned long long* table, int* filled) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nx || j >= g.ny) return;
    for (int k = blockIdx.z * kSetupPlanes, k1 = min(g.nz, k + kSetupPlanes); k < k1; ++k) {
        const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
        if (cls[n] == kInterfaceNode || cls[n] == kGeneral) iface_insert(table, filled, cell_key(mat, g, i, j, k));
    }
}

// The keys held in the set, in slot order, to keys[atomicAdd(count)].
__global__ void k_iface_compact(const unsigned long long* __restrict__ table, unsigned long long* keys, int* count) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= kIfaceTableSize) return;
    const unsigned long long v = table[s];
    if (v != kEmptyKey) keys[atomicAdd(count, 1)] = v;
}

// slot_row[slot of sorted key q] = q for the rows kept.
__global__ void k_iface_slot_rows(const unsigned long long* __restrict__ table, const unsigned long long* __restrict__ keys,
                                  int n_keys, int* slot_row) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_keys) return;
    const int s = find_slot(table, keys[q]);
    if (s >= 0) slot_row[s] = q;
}

// Coefficient rows of every node (StepParams::rec): the material id of fast-path nodes and of
// kUniformGeneral + m nodes (m), the interface row of kInterfaceNode and kGeneral nodes whose key
// has one, and kRecGeneral | class for the rest. kInterfaceNode nodes without a row become
// kGeneral.
__device__ __forceinline__ void iface_row(uint8_t* __restrict__ cls, const uint8_t* __restrict__ mat, const DeviceGrid& g,
                                          const unsigned long long* __restrict__ table, const int* __restrict__ slot_row,
                                          uint16_t* __restrict__ rec, int i, int j, int k);
__global__ void k_iface_rows(uint8_t* __restrict__ cls, const uint8_t* __restrict__ mat, DeviceGrid g,
                             const unsigned long long* __restrict__ table, const int* __restrict__ slot_row,
                             uint16_t* __restrict__ rec) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nx || j >= g.ny) return;
    for (int k = blockIdx.z * kSetupPlanes, k1 = min(g.nz, k + kSetupPlanes); k < k1; ++k)
        iface_row(cls, mat, g, table, slot_row, rec, i, j, k);
}
__device__ __forceinline__ void iface_row(uint8_t* __restrict__ cls, const uint8_t* __restrict__ mat, const DeviceGrid& g,
                                          const unsigned long long* __restrict__ table, const int* __restrict__ slot_row,
                                          uint16_t* __restrict__ rec, int i, int j, int k) {
    const long long n = (long long)k * g.plane + (long long)j * g.pitch + i;
    int c = cls[n];
    int r = kRecGeneral | c;
    if (c < kUniformGeneral) {
        r = c;
    } else if (c < kInterfaceNode) {
        r = c - kUniformGeneral;
    } else if (c == kInterfaceNode || c == kGeneral) {
        const int s = find_slot(table, cell_key(mat, g, i, j, k));
        const int row = s >= 0 ? slot_row[s] : -1;
        if (row >= 0) {
            r = kFirstInterfaceRow + row;
        } else if (c == kInterfaceNode) {
            cls[n] = kGeneral;
            r = kRecGeneral | kGeneral;
        }
    }
    rec[n] = (uint16_t)r;
}

// Lumped edges keep the general path in every schedule (their E update is the lumped override).
__global__ void k_rec_general(uint16_t* rec, DeviceGrid g, const LumpedEdge* edges, int n_edges) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n_edges)
        rec[(long long)edges[q].k * g.plane + (long long)edges[q].j * g.pitch + edges[q].i] = (uint16_t)(kRecGeneral | kGeneral);
}

cudaError_t launch_rec_general(const DeviceGrid& g, const LumpedEdge* edges, int n_edges, uint16_t* rec, cudaStream_t st) {
    if (n_edges <= 0) return cudaSuccess;
    k_rec_general<<<(n_edges + 127) / 128, 128, 0, st>>>(rec, g, edges, n_edges);
    return cudaGetLastError();
}

// Coefficient row kFirstInterfaceRow + q of unique key q, from the material rows and properties.
__global__ void k_iface_coefs(const __grid_constant__ StepParams p, const unsigned long long* __restrict__ keys,
                              int n_keys, MatCoef* coef) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_keys) return;
    const unsigned long long key = keys[q];
    const int m0 = (int)(key & 0xff), mi = (int)((key >> 8) & 0xff), mj = (int)((key >> 16) & 0xff);
    const int mk = (int)((key >> 24) & 0xff), mij = (int)((key >> 32) & 0xff), mik = (int)((key >> 40) & 0xff);
    const int mjk = (int)((key >> 48) & 0xff);
    // position-free coefficients: no design cells (those nodes are kDesignNode); CPML kappa and
    // boundary faces are the CPML sweep's
    const Coef3 ex = e_coef(p, 0, m0 == mj && m0 == mk && m0 == mjk, m0, mj, mk, mjk, 1, 1, 1);
    const Coef3 ey = e_coef(p, 1, m0 == mi && m0 == mk && m0 == mik, m0, mi, mk, mik, 1, 1, 1);
    const Coef3 ez = e_coef(p, 2, m0 == mi && m0 == mj && m0 == mij, m0, mi, mj, mij, 1, 1, 1);
    const Coef3 hx = h_coef(p, 0, false, m0 == mi, m0, mi);
    const Coef3 hy = h_coef(p, 1, false, m0 == mj, m0, mj);
    const Coef3 hz = h_coef(p, 2, false, m0 == mk, m0, mk);
    MatCoef c;
    c.e[0] = make_float4(ex.a, ex.bp, ex.bm, 0.f);
    c.e[1] = make_float4(ey.a, ey.bp, ey.bm, 0.f);
    c.e[2] = make_float4(ez.a, ez.bp, ez.bm, 0.f);
    c.h[0] = make_float4(hx.a, hx.bp, hx.bm, 0.f);
    c.h[1] = make_float4(hy.a, hy.bp, hy.bm, 0.f);
    c.h[2] = make_float4(hz.a, hz.bp, hz.bm, 0.f);
    coef[kFirstInterfaceRow + q] = c;
}

cudaError_t launch_iface_set(const DeviceGrid& g, const uint8_t* cls, const uint8_t* mat, unsigned long long* table,
                             int* counters, unsigned long long* keys, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(table, 0xff, sizeof(unsigned long long) * kIfaceTableSize, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, 2 * sizeof(int), st);
    if (e != cudaSuccess) return e;
    const dim3 block(32, 8, 1), grid((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + kSetupPlanes - 1) / kSetupPlanes);
    k_iface_insert<<<grid, block, 0, st>>>(cls, mat, g, table, counters);
    k_iface_compact<<<kIfaceTableSize / 256, 256, 0, st>>>(table, keys, counters + 1);
    return cudaGetLastError();
}

cudaError_t launch_iface_rows(const DeviceGrid& g, uint8_t* cls, const uint8_t* mat, const unsigned long long* table,
                              const unsigned long long* keys, int n_keys, int* slot_row, uint16_t* rec, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(slot_row, 0xff, sizeof(int) * kIfaceTableSize, st);
    if (e != cudaSuccess) return e;
    if (n_keys > 0) k_iface_slot_rows<<<(n_keys + 127) / 128, 128, 0, st>>>(table, keys, n_keys, slot_row);
    const dim3 block(32, 8, 1), grid((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + kSetupPlanes - 1) / kSetupPlanes);
    k_iface_rows<<<grid, block, 0, st>>>(cls, mat, g, table, slot_row, rec);
    return cudaGetLastError();
}

cudaError_t launch_iface_coefs(const StepParams& p, const unsigned long long* keys, int n_keys, MatCoef* coef,
                               cudaStream_t st) {
    if (n_keys <= 0) return cudaSuccess;
    k_iface_coefs<<<(n_keys + 127) / 128, 128, 0, st>>>(p, keys, n_keys, coef);
    return cudaGetLastError();
}

}  // namespace fdtd
