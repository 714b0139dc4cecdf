// Launch interface of the update kernels (host-visible declarations).
#pragma once

#include <cuda.h>

#include <vector>

#include "fdtd_device.cuh"

namespace fdtd {

struct FieldPtrs {
    float *ex, *ey, *ez, *hx, *hy, *hz;
};

// Six CPML faces in the order x_n, x_p, y_n, y_p, z_n, z_p.
struct PsiSet {
    PsiFace f[6];
};

// One time step m with the two-pass schedule (E pass then H pass, in place).
cudaError_t launch_two_pass(const StepParams& p, const FieldPtrs& f, const PsiSet& ps, long long m,
                            cudaStream_t st);

// A box of nodes [x0, x1) x [y0, y1) x [z0, z1).
struct NodeBox {
    int x0, y0, z0, x1, y1, z1;
};

// One two-pass step m over the nodes of box b only (inside the grid; the design region's E and
// the plate nodes as in launch_two_pass). Nodes outside b keep their values.
cudaError_t launch_two_pass_box(const StepParams& p, const FieldPtrs& f, const PsiSet& ps, const NodeBox& b, long long m,
                                cudaStream_t st);

// One two-pass step whose step index is *base + s (device counter), for graph replay; handles
// without a design region or plates only.
cudaError_t launch_two_pass_rel(const StepParams& p, const FieldPtrs& f, const PsiSet& ps, const long long* base, int s,
                                cudaStream_t st);

// E of the design region's nodes, fi/pin -> fo/pout, after a schedule's E kernels; nothing
// without a design region.
cudaError_t launch_design_e(const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo, const PsiSet& pin,
                            const PsiSet& pout, long long m, cudaStream_t st);

// E of the plate nodes (StepParams::plate_nodes), fi/pin -> fo/pout, after a schedule's E kernels.
cudaError_t launch_plate_e(const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo, const PsiSet& pin,
                           const PsiSet& pout, long long m, cudaStream_t st);

// Shell items of the fused schedule (planner.h), one list per set of CPML slabs their nodes may
// lie in: kShellZ (z slabs only: planes outside the interior z range within the interior's x / y
// range, and tiles around a design region), kShellYZ (the y bands beside the interior), kShellX
// (the x bands beside the swept rows, inside the interior z range), kShellAny (the rest of the x
// bands, corners included, and whole grids without interior tiles).
enum { kShellZ = 0, kShellYZ = 1, kShellX = 2, kShellAny = 3, kShellLists = 4 };
struct ShellWork {
    const int4* items[kShellLists];
    int n[kShellLists];
};

// Shell passes of the fused schedule (yee_two_pass.cu): E (e_pass) or H of the nodes of the shell
// items, reading fi / pin (buffer A) and writing fo / pout (buffer B). The lists must lie one after
// the other in device memory (one launch covers them).
cudaError_t launch_shell(bool e_pass, const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo, const PsiSet& pin,
                         const PsiSet& pout, const ShellWork& w, long long m, cudaStream_t st);

// Fused schedule (yee_fused.cu): per step the shell E pass, the z-marching interior sweep (TMA
// tiles of buffer A: H with halo, old E, coefficient rows) and the shell H pass; fields A -> B, CPML
// memory psi_in -> psi_out. The items come from plan_fused (planner.h).
struct FusedMaps {
    CUtensorMap h[3];
    CUtensorMap e[3];
    CUtensorMap rec;  // coefficient rows (StepParams::rec)
};
// Tensor maps of the CPML sweep: the sweep's own, plus the CPML memory of buffer A's y and z faces
// per side (0: n face, 1: p face) and array (the two E, the two H arrays of the face): E arrays in
// E-tile boxes (the halo nodes' E needs its old psi too), H arrays in boxes of the tile's own nodes.
// Faces without CPML cells have no maps: bit s of `faces` is set for y side s, bit 2 + s for z
// side s, and the sweep loads through no other map.
struct CpmlMaps {
    FusedMaps base;
    CUtensorMap ye[2][2], yh[2][2];
    CUtensorMap ze[2][2], zh[2][2];
    int faces;
};
// Work items of one step (device arrays of int4 in the formats of planner.h).
struct FusedWork {
    const int4* interior;
    int n_interior;
    ShellWork shell;
    const int4* cpml;  // CPML items (CPML sweep), run after the interior sweep on its stream
    int n_cpml;
};
cudaError_t fused_configure();
int fused_smem_bytes();
int cpml_smem_bytes();
// fork (optional): a second stream and two events; the interior sweep then runs on `aux`,
// concurrently with the shell E pass on `st` (they read buffer A and write disjoint nodes of B),
// and `st` waits for it before the shell H pass.
struct FusedFork {
    cudaStream_t aux;
    cudaEvent_t fork, join;
};
// cmaps: the CPML sweep's maps (buffer A), needed when w.n_cpml > 0.
cudaError_t launch_fused(const FusedMaps& maps, const StepParams& p, const FieldPtrs& fi, const FieldPtrs& fo,
                         const PsiSet& psi_in, const PsiSet& psi_out, long long m, const FusedWork& w, cudaStream_t st,
                         const FusedFork* fork = nullptr, const CpmlMaps* cmaps = nullptr);
// encode_fn: the driver's cuTensorMapEncodeTiled. Returns 0 on success.
int encode_fused_maps(FusedMaps* out, const DeviceGrid& g, float* const h[3], float* const e[3], const uint16_t* rec,
                      void* encode_fn);
// The CPML sweep's maps of a buffer (fields h, e, CPML memory psi) into out.
int encode_cpml_maps(CpmlMaps* out, const DeviceGrid& g, float* const h[3], float* const e[3], const uint16_t* rec,
                     const PsiSet& psi, void* encode_fn);

// Setup kernels (setup_kernels.cu).
// r0 = 0: the reference's grading (sigma_opt); r0 > 0: sigma_max from that reflection coefficient.
cudaError_t launch_cpml_profiles(const DeviceGrid& g, float pi, float r0, float* const prof[18], cudaStream_t st);
cudaError_t launch_material_tables(const DeviceGrid& g, const MatProps* props, int n, MatCoef* coef,
                                   cudaStream_t st);
cudaError_t launch_lumped_coefs(const DeviceGrid& g, const uint8_t* mat, const MatProps* props,
                                LumpedEdge* edges, const int* boxes, const float* resist, const int* owner,
                                int n_edges, cudaStream_t st);
// kappa_dev: device array of 6 pointers {kappa_e x, kappa_m x, kappa_e y, kappa_m y, kappa_e z,
// kappa_m z}; out_dev: device array of 12 pointers, per axis {E slot 0, E slot 1, H slot 0, H slot 1}.
cudaError_t launch_bg_curl(const DeviceGrid& g, const MatCoef* coef, int bg, const float* const* kappa_dev,
                           float* const* out_dev, cudaStream_t st);
cudaError_t launch_fill(float* p, long long n, float v, cudaStream_t st);
// Columns nx .. pitch-1 of every row of a field array set to v.
cudaError_t launch_fill_padding(float* p, const DeviceGrid& g, float v, cudaStream_t st);
// Node classes (StepParams::cls) from the material index and the lumped edges.
// design_box: the design region's cells or NULL (its edge box gets class kDesignNode).
// Set the node class of the listed nodes ({i, j, k, -}) to `value`.
cudaError_t launch_class_nodes(const DeviceGrid& g, const int4* nodes, int n, int value, uint8_t* cls, cudaStream_t st);
cudaError_t launch_node_class(const DeviceGrid& g, const uint8_t* mat, const LumpedEdge* edges, int n_edges,
                              const int* design_box, uint8_t* cls, cudaStream_t st);
// Largest material index of the grid's cells into *out (device int).
cudaError_t launch_index_max(const uint8_t* mat, const DeviceGrid& g, int* out, cudaStream_t st);
cudaError_t launch_paint(uint8_t* mat, const DeviceGrid& g, const int box[6], uint8_t value, cudaStream_t st);
// Interface rows (setup_kernels.cu). launch_iface_set collects the distinct seven-cell keys of the
// kInterfaceNode nodes in a device hash set (table: kIfaceTableSize slots; counters: 2 ints) and
// lists them, unsorted, in keys (kIfaceTableSize entries; counters[1] = their number).
// launch_iface_rows, given the n_keys sorted keys that get rows, writes the per-node coefficient
// rows (StepParams::rec; nodes without a row become kGeneral; slot_row: kIfaceTableSize ints of
// scratch). launch_iface_coefs computes the rows themselves (p: the handle's parameters with the
// material rows in place).
constexpr int kIfaceTableBits = 17;
constexpr int kIfaceTableSize = 1 << kIfaceTableBits;
cudaError_t launch_iface_set(const DeviceGrid& g, const uint8_t* cls, const uint8_t* mat, unsigned long long* table,
                             int* counters, unsigned long long* keys, cudaStream_t st);
cudaError_t launch_iface_rows(const DeviceGrid& g, uint8_t* cls, const uint8_t* mat, const unsigned long long* table,
                              const unsigned long long* keys, int n_keys, int* slot_row, uint16_t* rec, cudaStream_t st);
cudaError_t launch_iface_coefs(const StepParams& p, const unsigned long long* keys, int n_keys, MatCoef* coef,
                               cudaStream_t st);
// The lumped edges' nodes back to kRecGeneral | kGeneral in rec (after launch_iface_rows).
cudaError_t launch_rec_general(const DeviceGrid& g, const LumpedEdge* edges, int n_edges, uint16_t* rec, cudaStream_t st);

}  // namespace fdtd
