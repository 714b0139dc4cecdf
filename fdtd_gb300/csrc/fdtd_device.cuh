// Device-side data layout and arithmetic shared by every update kernel.
//
// Field arrays are FP32 SoA, (nz, ny, pitch) with pitch = nx rounded up to 32 floats, x fastest.
// The per-cell material is a uint8 index into a material table; the per-edge coefficients the
// reference stores in 24 arrays (setSigmaEpsSigmaMu + setCoefficients + setABCPML,
// fdtdrav.h:1097-1308, 1747-2160) are rebuilt in registers from that index: a table lookup when
// the cells around an edge share one material, the reference's averaging formula otherwise.
// CPML memory (psi) lives in slabs on the six faces only.
//
// Floating-point forms: every expression that the reference evaluates with FMA contraction is
// written here with explicit __fmaf_rn / __fmul_rn / __fdiv_rn so that the rounding sequence is
// fixed by the source and not by the optimiser, and the CPU oracle can restate it exactly.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fdtd {

constexpr float kTiny = 1.2e-38f;  // setZero's initial value for fields, psi and conductivities
constexpr int kMaxMaterials = 256;
constexpr int kDefaultEntry = kMaxMaterials;  // H coefficient of faces the reference never averages
constexpr int kGeneral = 255;                 // node class of nodes that take the general path
constexpr int kUniformGeneral = 128;         // classes below: fast-path nodes (the material id);
                                             // kUniformGeneral + m: general nodes whose seven cells
                                             // all hold material m (m < kInterfaceNode - kUniformGeneral)
constexpr int kInterfaceNode = 252;          // node class of interior nodes at a material interface
                                             // (no lumped edge): the table-coefficient update with
                                             // the coefficient row StepParams::rec gives
constexpr int kPlateNode = 254;              // node class of nodes with a plate-covered E edge
constexpr int kDesignNode = 253;              // node class of the design region's edge box; classes
                                              // below it are fast-path material ids
constexpr int kDesign = 255;                  // material index of design-region cells (per-cell eps_r)
// Coefficient rows: StepParams::coef holds the material rows 0 .. kMaxMaterials (the last one is
// kDefaultEntry), then one row per distinct seven-cell material combination of the interface
// nodes, from kFirstInterfaceRow. StepParams::rec holds per node its row, or kRecGeneral | class
// for nodes on the general path.
constexpr int kFirstInterfaceRow = kMaxMaterials + 1;
constexpr int kRecGeneral = 0x8000;
constexpr int kMaxInterfaceRows = kRecGeneral - kFirstInterfaceRow;

// Per-material coefficients for an edge whose surrounding cells all hold the same material.
// e[c] = {Ca, Cb_plus, Cb_minus, 0} for Ex, Ey, Ez; h[c] = {Ch, Cb_plus, Cb_minus, 0} for Hx, Hy,
// Hz (one 16-byte load per component).
struct MatCoef {
    float4 e[3];
    float4 h[3];
};

// Cell material of one axis: eps_r, sigma_e, mu_r, sigma_m. A component of E or H averages the
// values of its own axis (setSigmaEpsSigmaMu, fdtdrav.h:1097-1220: Ex from the x values, ...).
struct MatAxis {
    float eps, sig, mu, sigm;
};
struct MatProps {
    MatAxis a[3];  // x, y, z
};

// One face slab of CPML memory per axis side: two E and two H psi arrays.
//   x faces: e = {psi_eyx, psi_ezx}, h = {psi_hyx, psi_hzx}, layout (nz, ny, P)
//   y faces: e = {psi_exy, psi_ezy}, h = {psi_hxy, psi_hzy}, layout (nz, P, pitch)
//   z faces: e = {psi_exz, psi_eyz}, h = {psi_hxz, psi_hyz}, layout (P, ny, pitch)
struct PsiFace {
    float* e[2];
    float* h[2];
};

// A lumped element edge (source or resistor) with its coefficient override.
// An Ez edge (comp 2) holds Ceze, Cezhy, Cezhx, Cezj of defineSourceZ / defineResistor; an Ex edge
// (comp 0, defineSourceX) holds Cexe, Cexhz, Cexhy in the same slots and never injects.
struct LumpedEdge {
    int i, j, k;
    int comp;           // 0: Ex, 2: Ez
    int source;         // index of the driving waveform, -1 for a resistor or an Ex edge
    float ceze, cezhy, cezhx, cezj;
};

// E edges of one component that a zero-thickness plate covers in the planes it is bucketed under
// (definePlateX / Y / Z, fdtdrav.h:1574-1679): i in [i0, i1], j in [j0, j1]; their sigma_e is
// replaced by the plate's.
struct PlateEdges {
    int comp;
    int i0, i1, j0, j1;
    float sigma;
};

struct Probe {
    int comp, i, j, k;
};

struct DeviceGrid {
    int nx, ny, nz, pitch;
    long long plane;  // pitch * ny
    int pxn, pxp, pyn, pyp, pzn, pzp;
    float dx, dy, dz, dt, eps0, mu0;
};

// Curl coefficients of one material (the CPML background) divided by the CPML stretching kappa
// at every node of each axis, the value setABCPML leaves in the per-edge arrays
// (fdtdrav.h:1893-1906); outside the slabs kappa = 1 and the entries equal the undivided
// coefficient. Index [axis][slot] with the slots
//   x: {Ey minus, Ez plus}   y: {Ex plus, Ez minus}   z: {Ex minus, Ey plus}
// for E and
//   x: {Hy plus, Hz minus}   y: {Hx minus, Hz plus}   z: {Hx plus, Hy minus}
// for H.
struct BgCurl {
    int mat;
    const float* e[3][2];
    const float* h[3][2];
};

// Everything an update kernel reads besides the fields.
struct StepParams {
    DeviceGrid g;
    const uint8_t* mat;          // (nz, ny, pitch)
    // Node class (nz, ny, pitch): the material id when the node takes the fast path (every
    // component updated, outside the CPML slabs, no lumped edge, the seven cells of its three E
    // edge averages all of that material), kInterfaceNode, kUniformGeneral + m, kDesignNode,
    // kPlateNode or kGeneral otherwise. Built by launch_node_class.
    const uint8_t* cls;
    // Coefficient row of each node (nz, ny, pitch): the material id for fast-path nodes, the
    // interface row for kInterfaceNode nodes, kRecGeneral | class otherwise. Built with cls.
    const uint16_t* rec;
    const MatProps* props;       // kMaxMaterials entries
    // kMaxMaterials + 1 material rows (the last = reference default for H faces), then the
    // interface rows (kFirstInterfaceRow + q)
    const MatCoef* coef;
    // 1-D CPML profiles per axis (length nx, ny, nz): b/a for E and H, kappa for E and H
    const float *bex, *aex, *bmx, *amx, *kex, *kmx;
    const float *bey, *aey, *bmy, *amy, *key, *kmy;
    const float *bez, *aez, *bmz, *amz, *kez, *kmz;
    // lumped edges and probes, bucketed by plane k (CSR offsets, nz + 1 entries)
    const LumpedEdge* lumped;
    const int* lumped_k;
    const Probe* probes;
    const int* probe_k;
    int* probe_ids;              // probe id of each bucketed entry
    const float* const* waves;   // per source: per-edge signal by step
    const long long* wave_len;
    float* probe_ring;           // (capacity, n_probes)
    int n_probes;
    long long ring_cap;
    int* status;                 // device error word
    BgCurl bg;                   // kappa-divided curl coefficients of the CPML background material
    // design region: cells of material kDesign inside dbox = [d0,d3) x [d1,d4) x [d2,d5) take eps_r
    // from deps ((d5-d2), (d4-d1), (d3-d0), x fastest); NULL when the handle has none
    const float* deps;
    int dbox[6];
    // plate edges bucketed by plane k (CSR offsets, nz + 1 entries, in the order the plates were
    // added); NULL when the handle has none
    const PlateEdges* plates;
    const int* plate_k;
    const int4* plate_nodes;     // nodes of class kPlateNode {i, j, k, 0} (updated by k_plate_e)
    int n_plate_nodes;
    // records of an adjoint run that k_design_e takes in two-pass steps (NULL otherwise): the new
    // E of the design edge box into design_snap (three arrays of the box volume, x fastest), and
    // the FoM sample Ez into *fom_sample, from the design node fom_node when the probe is one
    // (else -1) or read at node fom_read by the kernel's first thread (else -1)
    float* design_snap;
    float* fom_sample;
    long long fom_node, fom_read;
};

// ------------------------------------------------------------------------------------------
// Arithmetic forms
// ------------------------------------------------------------------------------------------

// c1*v + c2*d2 + c3*d3 (calc_e fdtdrav.h:674, 705, 731; calc_h fdtdrav.h:338, 366, 385)
__device__ __forceinline__ float upd3(float c1, float v, float c2, float d2, float c3, float d3) {
    return __fmaf_rn(c3, d3, __fmaf_rn(c1, v, __fmul_rn(c2, d2)));
}
// The reference's Hx statement (fdtdrav.h:331-338) sits in two branches that share Chxh*Hx; it is
// contracted with that product as the addend: c3*d3 + (c2*d2 + c1*v).
__device__ __forceinline__ float upd3_hx(float c1, float v, float c2, float d2, float c3, float d3) {
    return __fmaf_rn(c3, d3, __fmaf_rn(c2, d2, __fmul_rn(c1, v)));
}
// with the lumped-source term c4*s (fdtdrav.h:728)
__device__ __forceinline__ float upd4(float c1, float v, float c2, float d2, float c3, float d3,
                                      float c4, float s) {
    return __fmaf_rn(c4, s, __fmaf_rn(c3, d3, __fmaf_rn(c1, v, __fmul_rn(c2, d2))));
}
// psi = b*psi + a*d (e.g. fdtdrav.h:404)
__device__ __forceinline__ float psi_upd(float b, float psi, float a, float d) {
    return __fmaf_rn(b, psi, __fmul_rn(a, d));
}
// The reference's Psi_hyz statement (fdtdrav.h:537) is contracted with b*psi as the addend.
__device__ __forceinline__ float psi_upd_hyz(float b, float psi, float a, float d) {
    return __fmaf_rn(a, d, __fmul_rn(b, psi));
}
// f = f + cpsi*psi (e.g. fdtdrav.h:410)
__device__ __forceinline__ float psi_add(float f, float cpsi, float psi) {
    return __fmaf_rn(cpsi, psi, f);
}

// Edge average of four cell values, ((a+b)+c)+d scaled by 0.25 (fdtdrav.h:1135, 1153, 1170).
__host__ __device__ __forceinline__ float avg4(float a, float b, float c, float d) {
    return (((a + b) + c) + d) * 0.25f;
}
// Harmonic mean of two cell values, (2*a*b)/(a+b) (fdtdrav.h:1183-1213).
__device__ __forceinline__ float harm2(float a, float b) {
    return __fdiv_rn(__fmul_rn(2.0f * a, b), __fadd_rn(a, b));
}

// Update coefficients of setCoefficients (fdtdrav.h:1250-1303) from an averaged relative
// material value `rel` and conductivity `cond` (c0 = eps0 for E, mu0 for H).
struct Coef3 {
    float a, bp, bm;
};
__device__ __forceinline__ Coef3 coef3(float rel, float cond, float dt, float c0, float dplus, float dminus) {
    const float two_r = 2.0f * rel;
    const float dts = __fmul_rn(dt, cond);
    const float num = __fmaf_rn(two_r, c0, -dts);
    const float den = __fmaf_rn(two_r, c0, dts);
    Coef3 r;
    r.a = __fdiv_rn(num, den);
    r.bp = __fdiv_rn(2.0f * dt, __fmul_rn(den, dplus));
    r.bm = __fdiv_rn(-2.0f * dt, __fmul_rn(den, dminus));
    return r;
}

__device__ __forceinline__ void atomic_flag(int* status, int code) {
    if (status) atomicCAS(status, 0, code);
}

}  // namespace fdtd
