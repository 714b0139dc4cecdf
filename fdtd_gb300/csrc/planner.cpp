// Work planner of the fused schedule (host only). See planner.h for the item formats.
#include "planner.h"

#include <algorithm>

namespace fdtd {

namespace {

// Shell item block shapes of 256 nodes (the shell kernels' block is 256 threads): widths. Shapes
// narrower than 16 serve only rectangles narrower than 16, since their warps load short row pieces.
constexpr int kShapes = 9;
constexpr int kShapeW[kShapes] = {32, 16, 64, 128, 256, 8, 4, 2, 1};

// Shell items of the rectangle [x0, x0+w) x [y0, y0+h) of planes k .. k+nk-1: the block shape
// with the fewest items.
void shell_rect(std::vector<PlanItem>& out, int x0, int y0, int w, int h, int k, int nk) {
    if (w <= 0 || h <= 0 || nk <= 0) return;
    int best = 0, narrowest = 1;
    while (narrowest < w && narrowest < 16) narrowest *= 2;
    long long best_n = -1;
    for (int sh = 0; sh < kShapes; ++sh) {
        const int bw = kShapeW[sh], bh = 256 / bw;
        if (bw < narrowest) continue;
        const long long n = (long long)((w + bw - 1) / bw) * ((h + bh - 1) / bh);
        if (best_n < 0 || n < best_n) { best_n = n; best = sh; }
    }
    const int bw = kShapeW[best], bh = 256 / bw;
    for (int y = 0; y < h; y += bh)
        for (int x = 0; x < w; x += bw) {
            const int cw = std::min(bw, w - x), ch = std::min(bh, h - y);
            out.push_back(PlanItem{x0 + x, y0 + y, k, best | cw << 4 | ch << 13 | (nk - 1) << 22});
        }
}

// Tile starts along an axis: from lo (rounded up to `align`) while the tile's far E positions
// (start + size) stay <= hi, plus, when `overlap`, one tile ending on hi (it overlaps its
// neighbour, which writes the same values there).
std::vector<int> starts(int lo, int hi, int size, int align, bool overlap) {
    std::vector<int> v;
    const int a0 = (lo + align - 1) / align * align;
    for (int q = a0; q + size <= hi; q += size) v.push_back(q);
    if (overlap && !v.empty() && v.back() + size < hi) {
        const int last = (hi - size) / align * align;
        if (last > v.back()) v.push_back(last);
    }
    return v;
}

}  // namespace

// Planes per interior item: chunks are halved until the grid has at least kMinItems of them, and
// no chunk is longer than kMaxChunk planes (an item also streams the plane below and recomputes
// the one above). 8192 items measured best at 512^3 against 2048, 4096 and 16384 (32 planes
// there). The cap matters on larger grids: at 1024 x 1024 x 896 the item count alone gives
// 224-plane chunks, and capping them at 32 planes took the fused step from 13.31 to 9.95 ms
// (70.6 -> 94.4 Gcell-updates/s; 16, 24, 40 and 56 planes: 10.27, 10.05, 9.92, 10.14 ms). Short
// chunks keep the CTAs in flight on neighbouring planes, so the halo rows one CTA loads are still
// in L2 when its neighbours load them.
int plan_chunk(const PlanGrid& g) {
    constexpr long long kMinItems = 8192;
    constexpr int kMaxChunk = 32;
    const long long tiles = (long long)((g.nx + kTileX - 1) / kTileX) * ((g.ny + kTileY - 1) / kTileY);
    int kc = g.nz;
    while (kc > 16 && tiles * ((g.nz + kc - 1) / kc) < kMinItems) kc = (kc + 1) / 2;
    return std::max(1, std::min(kc, kMaxChunk));
}

// Interior tiles (32 x 16 columns whose E positions x0..x0+TX, y0..y0+TY all lie in the x / y
// interior) get their interior planes as interior items (chunks of at most kc planes; the E
// positions of an item's top plane are recomputed, so a chunk keeps its top plane in the interior
// range). Tiles start at the first interior node (x0 rounded up to a multiple of 8: every TMA box
// then starts on a 16-byte boundary and every warp's row of stores on a 32-byte sector; origins
// off the sector grid left sectors half written by two CTAs, which measured up to 30 % slower) and
// step by the tile size; one more tile per axis ends on the last interior node. With a design
// region, tiles that reach its edge box stay out of the sweep and no overlapping tiles are added.
// Everything else is the shell: per run of planes a few rectangles, cut into items of 256 nodes
// in the block shape that wastes the fewest threads, in the list of the slabs they may touch:
// planes outside the interior z range split into the part over the interior's x / y range (z
// slabs only), the y bands beside it (y and z) and the x bands (any); inside the interior z range
// the y bands over the interior's x range (y and z), the x bands (x only over the swept rows, any
// beside them) and left-out design tiles (no slab: the z list). Grids without interior tiles are
// one rectangle per plane (any).
// With CPML items, the planes outside the interior z range over the swept rectangle and the y
// bands over its x range are CPML items instead of shell rectangles: per interior tile one item
// below and one above the interior planes, and per band tile (rows from 0, and from the end of
// the swept rectangle, the last one ending on the grid's last row) the whole column in chunks of
// kc planes.
void plan_fused(const PlanGrid& g, int kc, const int* design_box, FusedPlan& out, bool cpml_tiles) {
    out.interior.clear();
    for (auto& s : out.shell) s.clear();
    out.cpml.clear();
    const int xlo = std::max(g.pxn, 1), xhi = std::min(g.nx - 1 - g.pxp, g.nx - 2);  // interior nodes, inclusive
    const int ylo = std::max(g.pyn, 1), yhi = std::min(g.ny - 1 - g.pyp, g.ny - 2);
    const int zlo = std::max(g.pzn, 1), zhi = std::min(g.nz - 1 - g.pzp, g.nz - 2);
    const bool overlap = design_box == nullptr;
    std::vector<int> xs, ys;
    if (zhi > zlo) {
        xs = starts(xlo, xhi, kTileX, 8, overlap);
        ys = starts(ylo, yhi, kTileY, 1, overlap);
    }
    const int* d = design_box;
    std::vector<PlanItem> left_out;  // tiles inside the swept rectangle that reach the design edge box
    std::vector<PlanItem> swept_tiles;
    for (int y0 : ys)
        for (int x0 : xs) {
            if (d && x0 <= d[3] && d[0] <= x0 + kTileX && y0 <= d[4] && d[1] <= y0 + kTileY) left_out.push_back(PlanItem{x0, y0, 0, 0});
            else swept_tiles.push_back(PlanItem{x0, y0, 0, 0});
        }
    // plane-major order (see the end): chunks outer, tiles in row order inner
    out.interior.reserve(swept_tiles.size() * (size_t)std::max(1, (zhi - zlo + kc - 1) / kc));
    for (int k = zlo; k < zhi; k += kc)
        for (const PlanItem& t : swept_tiles) out.interior.push_back(PlanItem{t.x, t.y, k, std::min(k + kc, zhi)});
    const bool swept = !xs.empty() && !ys.empty();
    const int X0 = swept ? xs.front() : 0, X1 = swept ? xs.back() + kTileX : 0;
    const int Y0 = swept ? ys.front() : 0, Y1 = swept ? ys.back() + kTileY : 0;
    const bool cpml = cpml_tiles && swept && design_box == nullptr && g.ny >= kTileY &&
                      std::max(std::max(g.pyn, g.pyp), std::max(g.pzn, g.pzp)) <= kCpmlMaxSlab;
    if (cpml) {
        for (int y0 : ys)
            for (int x0 : xs) {
                out.cpml.push_back(PlanItem{x0, y0, 0, zlo});
                out.cpml.push_back(PlanItem{x0, y0, zhi, g.nz});
            }
        std::vector<int> bands;  // the low band's last tile ends on row Y0, the high band's first starts on Y1
        for (int y1 = Y0; y1 > 0; y1 -= kTileY) bands.push_back(y1 - kTileY);
        for (int y0 = Y1; y0 < g.ny; y0 += kTileY) bands.push_back(y0);
        for (int y0 : bands)
            for (int x0 : xs)
                for (int k = 0; k < g.nz; k += kc) out.cpml.push_back(PlanItem{x0, y0, k, std::min(k + kc, g.nz)});
    }
    std::vector<PlanItem>& sz = out.shell[kPlanShellZ];
    std::vector<PlanItem>& syz = out.shell[kPlanShellYZ];
    std::vector<PlanItem>& sx = out.shell[kPlanShellX];
    std::vector<PlanItem>& sany = out.shell[kPlanShellAny];
    // runs of up to kShellPlanes planes with the same rectangles share items
    for (int k = 0; k < g.nz;) {
        const bool caps = swept && (k < zlo || k >= zhi);
        const int end = !swept ? g.nz : k < zlo ? zlo : k < zhi ? zhi : g.nz;
        const int nk = std::min(kShellPlanes, end - k);
        if (!swept) {
            shell_rect(sany, 0, 0, g.nx, g.ny, k, nk);
        } else {
            if (caps && !cpml) shell_rect(sz, X0, Y0, X1 - X0, Y1 - Y0, k, nk);
            if (!cpml) {
                shell_rect(syz, X0, 0, X1 - X0, Y0, k, nk);
                shell_rect(syz, X0, Y1, X1 - X0, g.ny - Y1, k, nk);
            }
            if (caps) {
                shell_rect(sany, 0, 0, X0, g.ny, k, nk);
                shell_rect(sany, X1, 0, g.nx - X1, g.ny, k, nk);
            } else {  // the swept rows lie outside the y slabs, the planes outside the z slabs
                for (int x0 : {0, X1}) {
                    const int w = x0 == 0 ? X0 : g.nx - X1;
                    shell_rect(sany, x0, 0, w, Y0, k, nk);
                    shell_rect(sx, x0, Y0, w, Y1 - Y0, k, nk);
                    shell_rect(sany, x0, Y1, w, g.ny - Y1, k, nk);
                }
            }
            if (!caps)
                for (const PlanItem& t : left_out) shell_rect(sz, t.x, t.y, kTileX, kTileY, k, nk);
        }
        k += nk;
    }
    // plane-major order: CTAs run in item order, so the CTAs in flight then work on neighbouring
    // planes of many tiles instead of many planes of a few tiles, which keeps the pages they touch
    // few on large grids
    // (the interior and shell lists are generated in that order; a stable sort by plane, done only
    // where a list is out of order, keeps the order of items of one plane)
    auto by_plane = [](const PlanItem& a, const PlanItem& b) { return a.z < b.z; };
    auto order = [&](std::vector<PlanItem>& v) {
        if (!std::is_sorted(v.begin(), v.end(), by_plane)) std::stable_sort(v.begin(), v.end(), by_plane);
    };
    order(out.interior);
    order(out.cpml);
    for (auto& s : out.shell) order(s);
}

}  // namespace fdtd
