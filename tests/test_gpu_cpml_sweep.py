"""The CPML sweep (schedule FUSED_CPML: the fused schedule with its z-march also over the planes
below and above the interior and over the y bands, with the z and y CPML recurrences, boundary
planes and rows) against the two-pass schedule, bit for bit: probes of every step and all six
final fields.

The grids have interior tiles and y / z slabs of at most 15 cells, so the planner gives the z caps
and y bands to the CPML sweep. They put materials, lumped edges, plates and probes inside those
regions and on the boundary planes and rows, so the sweep's table path, its out-of-line general
path (lumped edges, plates) and its masks all run.
"""
import dataclasses

import numpy as np
import pytest

from conftest import bitwise_equal, rel_l2
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu


def run(sc, schedule, steps):
    from fdtd_gb300 import solver
    with solver.Simulation.from_scenario(sc, schedule, probe_capacity=steps) as sim:
        sim.step(steps)
        sim.synchronize()
        return sim.read_probes(0, steps), sim.fields()


FUSED_CPML = 3


def check(sc, steps):
    p1, f1 = run(sc, 1, steps)
    p2, f2 = run(sc, FUSED_CPML, steps)
    assert np.isfinite(p1).all() and np.abs(p1).max() > 0
    assert bitwise_equal(p2, p1), rel_l2(p2, p1)
    for c in range(6):
        assert bitwise_equal(f2[c], f1[c]), (c, rel_l2(f2[c], f1[c]))


def slab_probes(sc):
    """Probes of every component in the z caps, the y bands, on the boundary plane k = 0 and the
    boundary row j = 0, over the interior x range."""
    nx, ny, nz = sc.nx, sc.ny, sc.nz
    i = nx // 2
    pts = [(i, ny // 2, 1), (i + 3, ny // 3, nz - 2), (i, 1, nz // 2), (i - 5, ny - 2, nz // 3),
           (i, ny // 2, 0), (i + 1, 0, nz // 2), (i + 2, 2, 2), (i, ny - 3, nz - 3)]
    return [S.Probe(c, *pt) for pt in pts for c in range(6)]


def cpml_case(nx=96, ny=72, nz=48, pml=(6, 7, 8, 5, 7, 6), steps=40, seed=12):
    sc = S.scaled_boxes(nx, ny, nz, steps, seed=seed, pml=4, n_boxes=10, n_sources=1, n_probes=4, name="cpml_sweep")
    sc = dataclasses.replace(sc, pml=pml)
    py0, pz0 = pml[2], pml[4]
    # a magnetic lossy box across the low z cap and the low y band, a dielectric one in the high cap
    sc.materials.append(S.Material(eps_r=3.0, sigma_e=0.02, mu_r=1.7, sigma_m=2e3))
    sc.bricks.append(S.Brick((20, 0, 0, 60, py0 + 6, pz0 + 3), len(sc.materials) - 1))
    sc.materials.append(S.Material(eps_r=7.5, sigma_e=0.01))
    sc.bricks.append(S.Brick((30, 20, nz - 5, 70, 50, nz), len(sc.materials) - 1))
    wave = sc.sources[0].waveform
    # a source in the low z cap, a resistor in the high y band and one in the high z cap
    sc.sources = sc.sources + [S.LumpedSource((44, ny // 2, 1, 44, ny // 2, 4), 50.0, wave)]
    sc.resistors = [S.Resistor((50, ny - 3, 10, 50, ny - 3, 14), 75.0),
                    S.Resistor((40, 30, nz - 5, 40, 30, nz - 2), 100.0)]
    # plates: z-normal in the low cap, y-normal in the low band, x-normal crossing the high band
    sc.plates = [S.Plate(2, (24, 10, 3, 56, 40, 3), 5.8e7, 5.8e7),
                 S.Plate(1, (30, 2, 10, 50, 2, 20), 1e7, 2e7),
                 S.Plate(0, (64, ny - 12, 8, 64, ny - 1, 30), 3e5, 4e5)]
    sc.probes = list(sc.probes) + slab_probes(sc)
    return sc


def test_cpml_sweep_equals_two_pass(gpu_lib):
    check(cpml_case(), 40)


@pytest.mark.parametrize("pml", [(4, 4, 3, 2, 0, 7), (6, 6, 15, 15, 15, 15), (5, 5, 16, 4, 16, 3), (2, 9, 1, 1, 1, 0)])
def test_cpml_sweep_slab_thicknesses(gpu_lib, pml):
    """Asymmetric slabs, a face without CPML (boundary plane only), the thickest slab the sweep
    takes (15 cells) and one above it (16: those nodes stay in the shell)."""
    sc = cpml_case(nx=96, ny=80, nz=64, pml=pml, steps=30, seed=sum(pml))
    check(sc, 30)


def test_cpml_sweep_many_chunks(gpu_lib):
    """Several z chunks per y-band column (a tall grid), ragged y bands."""
    sc = cpml_case(nx=80, ny=61, nz=300, pml=(6, 6, 9, 11, 8, 8), steps=20, seed=3)
    check(sc, 20)


def test_switching_between_fused_forms(gpu_lib):
    """FUSED and FUSED_CPML alternate mid-run (the work is planned again at each switch): the
    result equals the two-pass schedule's."""
    from fdtd_gb300 import solver
    sc = cpml_case(steps=30)
    p1, f1 = run(sc, 1, 30)
    with solver.Simulation.from_scenario(sc, 2, probe_capacity=30) as sim:
        for n, s in ((7, FUSED_CPML), (9, 2), (5, FUSED_CPML), (9, 1)):
            sim.step(n)
            sim.set_schedule(s)
        sim.synchronize()
        assert bitwise_equal(sim.read_probes(0, 30), p1)
        assert bitwise_equal(sim.fields(), f1)
