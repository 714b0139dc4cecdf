// Work planner of the fused schedule (host only, no CUDA types: also compiled on its own by the
// CPU tests, which check that the items cover every node exactly once).
//
// A fused step reads buffer A and writes buffer B. Its nodes are split into work items of three
// z-marching sweeps and one per-node pass:
//   * interior items {x0, y0, k0, k1}: a kTileX x kTileY column over planes [k0, k1) whose nodes
//     and E halo are all interior (no CPML slab, no boundary plane): the interior sweep;
//   * wide items {x0 | w << 16, y0 | h << 16, k0, k1}: a kTileX x kTileY column of which the
//     first w columns and h rows are the item's, over planes [k0, k1), anywhere in the grid: the
//     general sweep, which carries the CPML recurrences (z caps of the interior columns, the y
//     bands, and whole grids without interior tiles);
//   * narrow items, the same for kNarrowX x kNarrowY columns (the x bands beside the interior);
//   * shell items {x0, y0, k, code}: blocks of up to 256 nodes of planes k .. k + nk - 1 for the
//     per-node kernels (tiles that reach a design region's edge box, whose E needs the per-cell
//     eps_r): shape s = code & 15 (widths 32, 16, 64, 128, 256, 8, 4, 2, 1), columns
//     (code >> 4) & 511, rows (code >> 13) & 511, nk - 1 = (code >> 22) & 15.
#pragma once

#include <vector>

namespace fdtd {

constexpr int kTileX = 32, kTileY = 16;      // interior and wide sweep tiles
constexpr int kNarrowX = 16, kNarrowY = 32;  // narrow sweep tiles
constexpr int kMaxItemPlanes = 512;          // planes one sweep item streams (chunk + 2)
constexpr int kShellPlanes = 4;              // planes per shell item

struct PlanItem {
    int x, y, z, w;  // same layout as int4
};

struct PlanGrid {
    int nx, ny, nz;
    int pxn, pxp, pyn, pyp, pzn, pzp;
};

struct FusedPlan {
    std::vector<PlanItem> interior, wide, narrow, shell;
};

// Planes per sweep item (see plan_chunk in planner.cpp).
int plan_chunk(const PlanGrid& g);

// design_box: the design region's cells {i0, j0, k0, i1, j1, k1} (edge box: nodes i0..i1,
// j0..j1, k0..k1) or NULL; sweep items whose E positions reach it become shell items.
void plan_fused(const PlanGrid& g, int kc, const int* design_box, FusedPlan& out);

}  // namespace fdtd
