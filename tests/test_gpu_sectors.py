"""Sector plates (fdtd_add_sector; the reference's defineSec / tricheck, fdtdrav.h:1681-1744,
56-128): the edges they cover against the reference's own defineSec on the reference-kernel
harness, and runs against the same edges given as plates and against the oracle, bit for bit."""
import dataclasses

import numpy as np
import pytest

import oracle
from conftest import bitwise_equal
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu

# (tri = px0, py0, px1, py1, px2, py2 with apex (px1, py1), pz0, radius in m, max_x, max_y):
# sides through grid nodes, an apex on a node, a radius cutting the wedge, bounds cutting it
SECTORS = [((6, 26, 18, 12, 30, 26), 9, 0.0105, 34, 30),
           ((20, 4, 20, 16, 33, 16), 11, 0.02, 28, 30),
           ((3, 5, 15, 15, 27, 5), 7, 0.0125, 36, 17)]


def scenario(steps=120):
    sc = S.vacuum_cube(40, steps, pml=4, name="sectors")
    sc.nx, sc.ny, sc.nz = 40, 34, 24
    sc.materials.append(S.Material(eps_r=4.4, sigma_e=0.002))
    sc.bricks.append(S.Brick((4, 4, 4, 36, 30, 9), 1))
    sc.sources = [S.LumpedSource((20, 17, 9, 20, 17, 12), 50.0, S.gaussian_derivative(steps, sc.dt, 20e9, 1e-3))]
    sc.probes = [S.Probe(c, 14 + c, 15, 10) for c in range(6)] + [S.Probe(S.EX, 19, 13, 9), S.Probe(S.EY, 17, 10, 11)]
    return sc


def plates_of(sc, q):
    tri, pz0, r, mx, my = SECTORS[q]
    return S.sector_plates(tri, pz0, r, mx, my, 5.8e7, 3e7, sc.dx, sc.dy, sc.nx, sc.ny)


def test_sector_edges_vs_reference_defineSec(gpu_lib):
    """sigma_e_x / sigma_e_y after the reference's defineSec on its own averaged arrays equal the
    oracle's with the sector given as plates (plates write the same arrays)."""
    import refharness
    if not refharness.available():
        pytest.skip("reference-kernel harness not built")
    sc = scenario()
    for q, (tri, pz0, r, mx, my) in enumerate(SECTORS):
        h = refharness.RefHarness()
        try:
            h.setup(sc)
            h.sector(tri, pz0, r, mx, my, 5.8e7, 3e7)
            ref_x, ref_y = h.get("sigma_e_x"), h.get("sigma_e_y")
        finally:
            h.close()
        sc_q = dataclasses.replace(sc, plates=plates_of(sc, q))
        ex, ey = S.sector_edges(tri, pz0, r, mx, my, sc.dx, sc.dy, sc.nx, sc.ny)
        assert ex.sum() > 20 and ey.sum() > 20
        assert bitwise_equal(oracle.coef(sc_q, "sig_x"), ref_x), q
        assert bitwise_equal(oracle.coef(sc_q, "sig_y"), ref_y), q


@pytest.mark.parametrize("schedule", [1, 2])
def test_sector_runs(gpu_lib, schedule):
    """add_sector equals the same edges given as plates, and the oracle (GPU CPML profiles)."""
    from fdtd_gb300 import solver
    sc = scenario()
    plates = [p for q in range(len(SECTORS)) for p in plates_of(sc, q)]
    with solver.Simulation.from_scenario(sc, schedule, probe_capacity=sc.steps) as sim:
        for tri, pz0, r, mx, my in SECTORS:
            sim.add_sector(tri, pz0, r, mx, my, 5.8e7, 3e7)
        sim.step(sc.steps)
        sim.synchronize()
        p1, f1, prof = sim.read_probes(0, sc.steps), sim.fields(), sim.cpml_profiles()
    sc_p = dataclasses.replace(sc, plates=plates)
    with solver.Simulation.from_scenario(sc_p, schedule, probe_capacity=sc.steps) as sim:
        sim.step(sc.steps)
        sim.synchronize()
        p2, f2 = sim.read_probes(0, sc.steps), sim.fields()
    assert bitwise_equal(p1, p2) and bitwise_equal(f1, f2)
    po, fo = oracle.run(sc_p, profile_override=prof)
    assert bitwise_equal(p1, po) and bitwise_equal(f1, fo)


def test_sector_validation(gpu_lib):
    from fdtd_gb300 import solver
    sc = scenario()
    with solver.Simulation.from_scenario(sc) as sim:
        for args in [((6, 26, 18, 12, 30, 26), 24, 0.01, 30, 30, 1.0, 1.0),   # plane outside
                     ((6, 26, 18, 12, 30, 26), 9, 0.01, -1, 30, 1.0, 1.0),    # negative bound
                     ((6, 26, 18, 12, 30, 26), 9, 0.01, 30, 30, -1.0, 1.0)]:  # negative sigma
            with pytest.raises(solver.FDTDError):
                sim.add_sector(*args)
