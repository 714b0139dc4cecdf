// Work planner of the fused schedule (host only, no CUDA types: also compiled on its own by the
// CPU tests, which check that the items cover every node exactly once).
//
// A fused step reads buffer A and writes buffer B. Its nodes are split into
//   * interior items {x0, y0, k0, k1}: a kTileX x kTileY column over planes [k0, k1) whose nodes
//     and E halo are all interior (no CPML slab, no boundary plane), for the TMA sweep;
//   * shell items {x0, y0, k, code} for the per-node shell passes: blocks of up to 256 nodes of
//     planes k .. k + nk - 1, shape s = code & 15 (widths 32, 16, 64, 128, 256, 8, 4, 2, 1),
//     columns (code >> 4) & 511, rows (code >> 13) & 511, nk - 1 = (code >> 22) & 15; in four
//     lists by the CPML slabs their nodes may lie in (kPlanShellZ: z slabs only; kPlanShellYZ: y
//     and z; kPlanShellX: x only; kPlanShellAny: any), so that each list's kernel leaves the
//     impossible slab tests out;
//   * CPML items {x0, y0, k0, k1} (when asked for): kTileX x kTileY columns over planes [k0, k1)
//     whose x range (E halo included) is interior, for the CPML sweep (z and y slabs, boundary
//     planes and rows): the planes outside the interior z range above and below every interior
//     tile, and the y bands beside the swept rectangle over all planes. A band tile's rows may
//     reach outside the grid (rows below 0 or from ny on: the sweep leaves them out); its rows
//     inside the grid are all outside the swept rectangle. They replace the kPlanShellZ and
//     kPlanShellYZ items of those nodes.
#pragma once

#include <vector>

namespace fdtd {

constexpr int kTileX = 32, kTileY = 16;  // interior sweep tiles
constexpr int kMaxItemPlanes = 512;      // planes one sweep item streams (chunk + 2)
constexpr int kShellPlanes = 4;          // planes per shell item
enum { kPlanShellZ = 0, kPlanShellYZ = 1, kPlanShellX = 2, kPlanShellAny = 3, kPlanShellLists = 4 };

struct PlanItem {
    int x, y, z, w;  // same layout as int4
};

struct PlanGrid {
    int nx, ny, nz;
    int pxn, pxp, pyn, pyp, pzn, pzp;
};

struct FusedPlan {
    std::vector<PlanItem> interior;
    std::vector<PlanItem> shell[kPlanShellLists];
    std::vector<PlanItem> cpml;
};

// Thickest CPML slab (cells) the CPML sweep takes: a slab then fits in one tile row band.
constexpr int kCpmlMaxSlab = kTileY - 1;

// Planes per interior item (see plan_chunk in planner.cpp).
int plan_chunk(const PlanGrid& g);

// design_box: the design region's cells {i0, j0, k0, i1, j1, k1} (edge box: nodes i0..i1,
// j0..j1, k0..k1) or NULL; interior tiles whose E positions reach it go to the shell.
// cpml_tiles: plan CPML items where the grid allows them (no design region, every y and z slab
// at most kCpmlMaxSlab cells, interior tiles present); otherwise those nodes stay in the shell.
void plan_fused(const PlanGrid& g, int kc, const int* design_box, FusedPlan& out, bool cpml_tiles = false);

}  // namespace fdtd
