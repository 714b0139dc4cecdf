"""CPU tests of the fused schedule's work planner (fdtd_gb300/csrc/planner.cpp), compiled here with
g++ into a host-only library: the items of every list together store each node exactly once, sweep
items keep the TMA alignment and the plane limit, interior items hold only interior nodes (E halo
included), and no sweep item reaches a design region's edge box."""
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

TILE_X, TILE_Y, NARROW_X, NARROW_Y, MAX_ITEM_PLANES, SHELL_PLANES = 32, 16, 16, 32, 512, 4
SHAPE_W = [32, 16, 64, 128, 256, 8, 4, 2, 1]


@pytest.fixture(scope="module")
def lib():
    os.makedirs(BUILD, exist_ok=True)
    if not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB)
                                      for s in SRCS + [os.path.join(CSRC, "planner.h")]):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I" + CSRC, "-o", LIB] + SRCS)
    L = ctypes.CDLL(LIB)
    L.plan_probe.restype = ctypes.c_int
    return L


def plan(lib, dims, pml, design=None):
    g = (ctypes.c_int * 9)(*dims, *pml)
    d = None if design is None else (ctypes.c_int * 6)(*design)
    counts = (ctypes.c_int * 4)()
    lib.plan_probe(g, d, counts, None, 0)
    n = sum(counts)
    items = np.zeros((max(n, 1), 4), dtype=np.int32)
    kc = lib.plan_probe(g, d, counts, items.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n)
    lists, o = [], 0
    for q in range(4):
        lists.append(items[o:o + counts[q]])
        o += counts[q]
    return kc, lists


def interior_range(n, pn, pp):
    return max(pn, 1), min(n - 1 - pp, n - 2)


def check(lib, dims, pml, design=None):
    nx, ny, nz = dims
    kc, (interior, wide, narrow, shell) = plan(lib, dims, pml, design)
    cover = np.zeros((nz, ny, nx), dtype=np.int32)
    xlo, xhi = interior_range(nx, pml[0], pml[1])
    ylo, yhi = interior_range(ny, pml[2], pml[3])
    zlo, zhi = interior_range(nz, pml[4], pml[5])
    for x0, y0, k0, k1 in interior:
        assert x0 % 8 == 0 and 0 < k1 - k0 <= MAX_ITEM_PLANES - 2
        assert xlo <= x0 and x0 + TILE_X <= xhi and ylo <= y0 and y0 + TILE_Y <= yhi and zlo <= k0 and k1 <= zhi
        cover[k0:k1, y0:y0 + TILE_Y, x0:x0 + TILE_X] += 1
    for lst, tx, ty in ((wide, TILE_X, TILE_Y), (narrow, NARROW_X, NARROW_Y)):
        for xw, yh, k0, k1 in lst:
            x0, w, y0, h = xw & 0xffff, xw >> 16, yh & 0xffff, yh >> 16
            assert x0 % 4 == 0 and 0 < w <= tx and 0 < h <= ty and 0 < k1 - k0 <= MAX_ITEM_PLANES - 2
            assert x0 + w <= nx and y0 + h <= ny and 0 <= k0 and k1 <= nz
            if design is not None:
                d = design
                assert not (x0 <= d[3] and d[0] <= x0 + tx and y0 <= d[4] and d[1] <= y0 + ty and k0 <= d[5]
                            and d[2] <= k1), "a sweep item reaches the design edge box"
            cover[k0:k1, y0:y0 + h, x0:x0 + w] += 1
    for x0, y0, k, code in shell:
        s, cols, rows, nk = code & 15, (code >> 4) & 511, (code >> 13) & 511, ((code >> 22) & 15) + 1
        bw = SHAPE_W[s]
        assert cols <= bw and rows <= 256 // bw and nk <= SHELL_PLANES
        cover[k:k + nk, y0:y0 + rows, x0:x0 + cols] += 1
    assert cover.min() == 1 and cover.max() == 1, (int(cover.min()), int(cover.max()))
    return kc, interior, wide, narrow, shell


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


def test_bench_grid_uses_whole_band_tiles(lib):
    """512^3 with 10-cell CPML: the x bands are whole narrow tiles, the y bands whole wide tiles, and
    no shell items remain."""
    _, interior, wide, narrow, shell = check(lib, (512, 512, 512), (10,) * 6)
    assert len(shell) == 0 and len(interior) > 0
    assert all((it[0] >> 16) == NARROW_X and (it[1] >> 16) == NARROW_Y for it in narrow)
    assert all((it[0] >> 16) == TILE_X and (it[1] >> 16) == TILE_Y for it in wide)


@pytest.mark.parametrize("dims,pml,design", [
    ((128, 128, 128), (10,) * 6, (48, 48, 56, 80, 80, 72)),
    ((40, 40, 40), (6,) * 6, (16, 16, 17, 24, 24, 23)),
    ((96, 80, 64), (8,) * 6, (9, 10, 9, 30, 20, 18)),   # reaching into the CPML corner
])
def test_plan_with_design_region(lib, dims, pml, design):
    _, _, _, _, shell = check(lib, dims, pml, design)
    assert len(shell) > 0
