"""CPU tests of the fused schedule's work planner (fdtd_gb300/csrc/planner.cpp), compiled here with
g++ into a host-only library: the items of every list together store each node exactly once
(overlapping tiles write the same values), interior items keep the TMA alignment and the plane
limit and hold only interior nodes (E halo included) away from a design region's edge box, CPML
items lie inside the grid with an interior x range (E halo included), and no shell list holds
nodes of a CPML slab its kernel leaves out."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fdtd_gb300", "csrc")
BUILD = os.path.join(ROOT, "tests", "_build")
LIB = os.path.join(BUILD, "libplan_probe.so")
SRCS = [os.path.join(CSRC, "planner.cpp"), os.path.join(ROOT, "tests", "plan_probe.cpp")]

TILE_X, TILE_Y, MAX_ITEM_PLANES, SHELL_PLANES = 32, 16, 512, 4
SHAPE_W = [32, 16, 64, 128, 256, 8, 4, 2, 1]
# shell lists and the CPML slabs (bit 0 x, 1 y, 2 z) their kernels test for
SHELL_LISTS = (("shell_z", 4), ("shell_yz", 6), ("shell_x", 1), ("shell_any", 7))
LISTS = ("interior",) + tuple(n for n, _ in SHELL_LISTS) + ("cpml",)
CPML_MAX_SLAB = TILE_Y - 1


@pytest.fixture(scope="module")
def lib():
    os.makedirs(BUILD, exist_ok=True)
    if not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB)
                                      for s in SRCS + [os.path.join(CSRC, "planner.h")]):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I" + CSRC, "-o", LIB] + SRCS)
    L = ctypes.CDLL(LIB)
    L.plan_probe.restype = ctypes.c_int
    return L


def plan(lib, dims, pml, design=None, cpml=False):
    g = (ctypes.c_int * 9)(*dims, *pml)
    d = None if design is None else (ctypes.c_int * 6)(*design)
    counts = (ctypes.c_int * len(LISTS))()
    lib.plan_probe(g, d, int(cpml), counts, None, 0)
    n = sum(counts)
    items = np.zeros((max(n, 1), 4), dtype=np.int32)
    kc = lib.plan_probe(g, d, int(cpml), counts, items.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n)
    lists, o = {}, 0
    for q, name in enumerate(LISTS):
        lists[name] = items[o:o + counts[q]]
        o += counts[q]
    return kc, lists


def interior_range(n, pn, pp):
    return max(pn, 1), min(n - 1 - pp, n - 2)


def in_slab(q, n, pn, pp):
    return q < pn or q >= n - pp


def check(lib, dims, pml, design=None, cpml=False):
    nx, ny, nz = dims
    kc, L = plan(lib, dims, pml, design, cpml)
    xlo, xhi = interior_range(nx, pml[0], pml[1])
    ylo, yhi = interior_range(ny, pml[2], pml[3])
    zlo, zhi = interior_range(nz, pml[4], pml[5])
    owned = np.zeros((nz, ny, nx), dtype=np.int32)
    for x0, y0, k0, k1 in L["interior"]:
        assert x0 % 8 == 0 and 0 < k1 - k0 <= MAX_ITEM_PLANES - 2
        assert xlo <= x0 and x0 + TILE_X <= xhi and ylo <= y0 and y0 + TILE_Y <= yhi and zlo <= k0 and k1 <= zhi
        if design is not None:
            d = design
            assert not (x0 <= d[3] and d[0] <= x0 + TILE_X and y0 <= d[4] and d[1] <= y0 + TILE_Y), \
                "an interior tile reaches the design edge box"
        owned[k0:k1, y0:y0 + TILE_Y, x0:x0 + TILE_X] = 1  # overlapping tiles store the same values
    swept_plane = owned[min(zlo, nz - 1)].copy()  # nodes of the interior tiles in one interior plane
    cp = np.zeros_like(owned)  # overlapping CPML tiles store the same values
    for x0, y0, k0, k1 in L["cpml"]:
        assert x0 % 8 == 0 and 0 <= k0 < k1 <= nz and k1 - k0 <= MAX_ITEM_PLANES - 2
        assert xlo <= x0 and x0 + TILE_X <= xhi and -TILE_Y < y0 < ny
        ya, yb = max(y0, 0), min(y0 + TILE_Y, ny)
        if k0 >= zlo and k1 <= zhi:  # a band tile: its rows in the grid lie outside the swept rows
            swept = swept_plane[:, x0:x0 + TILE_X].any(axis=1)
            assert not swept[ya:yb].any(), "a band tile recomputes swept rows"
        cp[k0:k1, ya:yb, x0:x0 + TILE_X] = 1
    cover = owned + cp
    for name, slabs in SHELL_LISTS:
        for x0, y0, k, code in L[name]:
            s, cols, rows, nk = code & 15, (code >> 4) & 511, (code >> 13) & 511, ((code >> 22) & 15) + 1
            bw = SHAPE_W[s]
            assert cols <= bw and rows <= 256 // bw and nk <= SHELL_PLANES
            assert x0 + cols <= nx and y0 + rows <= ny and k + nk <= nz
            # the slabs the list's kernel leaves out hold none of its nodes
            if not slabs & 1:
                assert not any(in_slab(x, nx, pml[0], pml[1]) for x in range(x0, x0 + cols)), name
            if not slabs & 2:
                assert not any(in_slab(y, ny, pml[2], pml[3]) for y in range(y0, y0 + rows)), name
            if not slabs & 4:
                assert not any(in_slab(z, nz, pml[4], pml[5]) for z in range(k, k + nk)), name
            cover[k:k + nk, y0:y0 + rows, x0:x0 + cols] += 1
    assert cover.min() == 1 and cover.max() == 1, (int(cover.min()), int(cover.max()))
    return kc, L


@pytest.mark.parametrize("dims,pml", [
    ((512, 512, 512), (10,) * 6),
    ((256, 256, 256), (10,) * 6),
    ((128, 128, 128), (10,) * 6),
    ((64, 64, 64), (10,) * 6),
    ((80, 56, 40), (6,) * 6),
    ((96, 61, 47), (8,) * 6),
    ((33, 45, 70), (8,) * 6),
    ((17, 13, 11), (3, 2, 2, 3, 1, 2)),
    ((70, 45, 80), (0,) * 6),
    ((61, 50, 30), (1,) * 6),
    ((90, 37, 33), (2,) * 6),
    ((100, 17, 16), (3,) * 6),
    ((1024, 1024, 64), (10,) * 6),
    ((300, 200, 100), (0, 16, 12, 5, 20, 1)),
])
def test_plan_covers_every_node_once(lib, dims, pml):
    check(lib, dims, pml)


def test_bench_grid_lists(lib):
    """512^3 with 10-cell CPML: most nodes interior, every shell list in use."""
    _, L = check(lib, (512, 512, 512), (10,) * 6)
    assert len(L["interior"]) > 0 and all(len(L[n]) > 0 for n, _ in SHELL_LISTS)


@pytest.mark.parametrize("dims,kc_want", [((512, 512, 512), 32), ((1024, 1024, 896), 32), ((256, 256, 256), 16),
                                          ((1024, 1024, 128), 32)])
def test_interior_chunks_capped_and_plane_major(lib, dims, kc_want):
    """Interior items are at most 32 planes long (the cap that keeps the CTAs in flight on
    neighbouring planes; the 1024 x 1024 x 896 grid alone would give 224-plane chunks) and every
    list runs in plane-major order, tiles in row order within a plane."""
    kc, L = plan(lib, dims, (10,) * 6)
    assert kc == kc_want
    it = L["interior"]
    assert (it[:, 3] - it[:, 2] <= kc).all() and (it[:, 3] > it[:, 2]).all()
    for name in LISTS:
        z = L[name][:, 2]
        assert (np.diff(z) >= 0).all(), name
    # within one plane of the interior list: y outer, x inner
    first = it[it[:, 2] == it[0, 2]]
    order = np.lexsort((first[:, 0], first[:, 1]))
    assert (order == np.arange(len(first))).all()


@pytest.mark.parametrize("dims,pml,design", [
    ((128, 128, 128), (10,) * 6, (48, 48, 56, 80, 80, 72)),
    ((40, 40, 40), (6,) * 6, (16, 16, 17, 24, 24, 23)),
    ((96, 80, 64), (8,) * 6, (9, 10, 9, 30, 20, 18)),   # reaching into the CPML corner
])
def test_plan_with_design_region(lib, dims, pml, design):
    _, L = check(lib, dims, pml, design)
    assert sum(len(L[n]) for n, _ in SHELL_LISTS) > 0


@pytest.mark.parametrize("dims,pml", [
    ((512, 512, 512), (10,) * 6),
    ((256, 256, 256), (10,) * 6),
    ((128, 128, 128), (10,) * 6),
    ((80, 56, 40), (6,) * 6),
    ((96, 61, 47), (8,) * 6),
    ((33, 45, 70), (8,) * 6),
    ((70, 45, 80), (0,) * 6),
    ((61, 50, 30), (1,) * 6),
    ((100, 17, 16), (3,) * 6),
    ((1024, 1024, 64), (10,) * 6),
    ((300, 200, 100), (0, 16, 12, 5, 15, 1)),
    ((96, 90, 64), (8, 8, 15, 15, 15, 15)),
])
def test_plan_with_cpml_items(lib, dims, pml):
    """With CPML items every node is still stored once; where the grid has interior tiles and
    slabs of at most 15 cells, the z and y shell lists are empty."""
    _, L = check(lib, dims, pml, cpml=True)
    if len(L["interior"]) and max(pml[2:]) <= CPML_MAX_SLAB:
        assert len(L["cpml"]) > 0 and len(L["shell_z"]) == 0 and len(L["shell_yz"]) == 0
    if max(pml[2:]) > CPML_MAX_SLAB:
        assert len(L["cpml"]) == 0


def test_no_cpml_items_with_design(lib):
    _, L = check(lib, (128, 128, 128), (10,) * 6, (48, 48, 56, 80, 80, 72), cpml=True)
    assert len(L["cpml"]) == 0 and len(L["shell_z"]) > 0
