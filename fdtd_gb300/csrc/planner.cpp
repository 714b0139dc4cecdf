// Work planner of the fused schedule (host only). See planner.h for the item formats.
#include "planner.h"

#include <algorithm>

namespace fdtd {

namespace {

// Shell item block shapes of 256 nodes (the shell kernels' block is 256 threads): widths. Shapes
// narrower than 16 serve only rectangles narrower than 16, since their warps load short row pieces.
constexpr int kShapes = 9;
constexpr int kShapeW[kShapes] = {32, 16, 64, 128, 256, 8, 4, 2, 1};

int round_up(int v, int a) { return (v + a - 1) / a * a; }

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

// Shell items of a column [x0, x0+w) x [y0, y0+h) over planes [k0, k1).
void shell_column(std::vector<PlanItem>& out, int x0, int y0, int w, int h, int k0, int k1) {
    for (int k = k0; k < k1; k += kShellPlanes) shell_rect(out, x0, y0, w, h, k, std::min(kShellPlanes, k1 - k));
}

// The E positions a sweep item computes, nodes [x0, x0+tx] x [y0, y0+ty] x [k0, k1], reach the
// design region's edge box.
bool touches(const int* d, int x0, int y0, int k0, int tx, int ty, int k1) {
    return d && x0 <= d[3] && d[0] <= x0 + tx && y0 <= d[4] && d[1] <= y0 + ty && k0 <= d[5] && d[2] <= k1;
}

// General sweep items over [xa, xb) x [ya, yb) x [za, zb): tiles of tx x ty from (xa, ya), chunks
// of kc planes; items whose E positions reach the design edge box go to the shell instead.
void sweep_rect(std::vector<PlanItem>& out, std::vector<PlanItem>& shell, int xa, int xb, int ya, int yb, int za,
                int zb, int tx, int ty, int kc, const int* design) {
    if (xa >= xb || ya >= yb || za >= zb) return;
    for (int y = ya; y < yb; y += ty)
        for (int x = xa; x < xb; x += tx) {
            const int w = std::min(tx, xb - x), h = std::min(ty, yb - y);
            for (int k = za; k < zb; k += kc) {
                const int k1 = std::min(k + kc, zb);
                if (touches(design, x, y, k, tx, ty, k1)) {
                    shell_column(shell, x, y, w, h, k, k1);
                    continue;
                }
                out.push_back(PlanItem{x | w << 16, y | h << 16, k, k1});
            }
        }
}

}  // namespace

// Planes per sweep item: whole columns unless that leaves too few CTAs to fill the GPU, and at
// most kMaxItemPlanes - 2 (an item also streams the plane below and recomputes the one above).
// Chunks are halved until the grid has at least kMinItems of them; 8192 measured best at 512^3 and
// 1024 x 1024 x 896 against 2048, 4096 and 16384 (shorter chunks keep the CTAs in flight on fewer
// planes; each chunk re-reads two planes).
int plan_chunk(const PlanGrid& g) {
    constexpr long long kMinItems = 8192;
    const long long tiles = (long long)((g.nx + kTileX - 1) / kTileX) * ((g.ny + kTileY - 1) / kTileY);
    int kc = g.nz;
    while (kc > 16 && tiles * ((g.nz + kc - 1) / kc) < kMinItems) kc = (kc + 1) / 2;
    return std::max(1, std::min(kc, kMaxItemPlanes - 2));
}

// Interior tiles start at the first interior node rounded up to a multiple of 16 in x and y (the
// TMA boxes of every sweep then start on 16-byte boundaries, every warp's row of stores on a
// 32-byte sector, and the bands beside the interior are whole narrow / wide tiles when the CPML
// is at most 16 cells thick) and step by the tile size while the tile's far E positions stay
// interior. The rest of the grid goes to the general sweep: the z caps of the interior columns
// (planes outside the interior z range), the y bands over the interior's x range (wide tiles),
// and the x bands over the whole y range (narrow tiles). Without interior tiles the whole grid is
// one general sweep of wide tiles. Tiles that reach a design region's edge box go to the shell.
void plan_fused(const PlanGrid& g, int kc, const int* design_box, FusedPlan& out) {
    out.interior.clear();
    out.wide.clear();
    out.narrow.clear();
    out.shell.clear();
    const int xlo = std::max(g.pxn, 1), xhi = std::min(g.nx - 1 - g.pxp, g.nx - 2);  // interior nodes, inclusive
    const int ylo = std::max(g.pyn, 1), yhi = std::min(g.ny - 1 - g.pyp, g.ny - 2);
    const int zlo = std::max(g.pzn, 1), zhi = std::min(g.nz - 1 - g.pzp, g.nz - 2);
    std::vector<int> xs, ys;
    if (zhi > zlo) {
        for (int x = round_up(xlo, 16); x + kTileX <= xhi; x += kTileX) xs.push_back(x);
        for (int y = round_up(ylo, 16); y + kTileY <= yhi; y += kTileY) ys.push_back(y);
    }
    const int* d = design_box;
    // general items stream half as many planes as interior ones: they are fewer, and the shorter
    // marches spread them over more CTAs
    const int kg = std::min(kc, std::max(8, kc / 2));
    if (xs.empty() || ys.empty()) {
        sweep_rect(out.wide, out.shell, 0, g.nx, 0, g.ny, 0, g.nz, kTileX, kTileY, kg, d);
    } else {
        const int X0 = xs.front(), X1 = xs.back() + kTileX, Y0 = ys.front(), Y1 = ys.back() + kTileY;
        for (int y0 : ys)
            for (int x0 : xs) {
                if (touches(d, x0, y0, zlo, kTileX, kTileY, zhi)) {
                    shell_column(out.shell, x0, y0, kTileX, kTileY, zlo, zhi);
                    continue;
                }
                for (int k = zlo; k < zhi; k += kc) out.interior.push_back(PlanItem{x0, y0, k, std::min(k + kc, zhi)});
            }
        // z caps of the interior rectangle
        sweep_rect(out.wide, out.shell, X0, X1, Y0, Y1, 0, zlo, kTileX, kTileY, kg, d);
        sweep_rect(out.wide, out.shell, X0, X1, Y0, Y1, zhi, g.nz, kTileX, kTileY, kg, d);
        // y bands over the interior's x range, x bands over the whole y range
        sweep_rect(out.wide, out.shell, X0, X1, 0, Y0, 0, g.nz, kTileX, kTileY, kg, d);
        sweep_rect(out.wide, out.shell, X0, X1, Y1, g.ny, 0, g.nz, kTileX, kTileY, kg, d);
        sweep_rect(out.narrow, out.shell, 0, X0, 0, g.ny, 0, g.nz, kNarrowX, kNarrowY, kg, d);
        sweep_rect(out.narrow, out.shell, X1, g.nx, 0, g.ny, 0, g.nz, kNarrowX, kNarrowY, kg, d);
    }
    // plane-major order: CTAs run in item order, so the CTAs in flight then work on neighbouring
    // planes of many tiles instead of many planes of a few tiles, which keeps the pages they touch
    // few on large grids
    auto by_plane = [](const PlanItem& a, const PlanItem& b) { return a.z < b.z; };
    std::stable_sort(out.interior.begin(), out.interior.end(), by_plane);
    std::stable_sort(out.wide.begin(), out.wide.end(), by_plane);
    std::stable_sort(out.narrow.begin(), out.narrow.end(), by_plane);
    std::stable_sort(out.shell.begin(), out.shell.end(), by_plane);
}

}  // namespace fdtd
