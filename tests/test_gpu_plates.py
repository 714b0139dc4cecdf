"""Zero-thickness plates on the GPU: both schedules against the oracle on edge-case grids, the
fixture of the reference's own plate kernels (tests/test_gpu_parity.py), and the host checks.

The edge cases: plates inside the CPML corners, on the low boundary planes, overlapping plates
(the later one wins), x-, y- and z-normal plates crossing each other, a plate next to a lumped
source, ragged grids (sizes that are not multiples of the tile), and the static-scratch entry.
"""
import numpy as np
import pytest

import oracle
from conftest import bitwise_equal
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu

FDTD_ERR_INVALID, FDTD_ERR_STATE = 1, 4


def plate_case(nx=37, ny=29, nz=23, steps=120, pml=(4, 3, 5, 4, 3, 4)):
    sc = S.vacuum_cube(nx, steps, pml=4, name="plates_edge")
    sc.nx, sc.ny, sc.nz = nx, ny, nz
    sc.pml = pml
    sc.materials.append(S.Material(eps_r=3.0, sigma_e=0.01))
    sc.bricks.append(S.Brick((6, 5, 4, 30, 24, 9), 1))
    sc.plates = [S.Plate(2, (0, 0, 4, nx - 1, ny - 1, 4), 1e10, 1e10),    # ground over the whole plane
                 S.Plate(2, (9, 10, 9, 27, 15, 9), 5.8e7, 5.8e7),
                 S.Plate(2, (20, 12, 9, 33, 18, 9), 1e4, 2e4),              # overlaps the strip, into the CPML
                 S.Plate(0, (2, 2, 2, 2, 20, 15), 1e6, 2e6),                # inside the x CPML
                 S.Plate(0, (0, 4, 5, 0, 9, 11), 7e5, 8e5),                 # on the boundary plane i = 0
                 S.Plate(1, (10, 20, 5, 26, 20, 14), 3e5, 4e5),             # crosses the z plates
                 S.Plate(1, (12, 0, 3, 18, 0, 8), 5e5, 6e5)]                # on the boundary plane j = 0
    sc.sources = [S.LumpedSource((14, 12, 4, 14, 12, 9), 50.0, S.gaussian_derivative(steps, sc.dt, 25e9, 1e-3))]
    sc.resistors = [S.Resistor((24, 13, 4, 24, 13, 9), 75.0)]
    sc.probes = [S.Probe(S.EZ, 18, 12, 6), S.Probe(S.EX, 15, 12, 9), S.Probe(S.EY, 2, 10, 8),
                 S.Probe(S.HX, 18, 13, 7), S.Probe(S.EZ, 15, 20, 8), S.Probe(S.EX, 1, 1, 4)]
    return sc


def run(sc, schedule, static=False):
    from fdtd_gb300 import solver
    with solver.Simulation.from_scenario(sc, schedule, probe_capacity=sc.steps) as sim:
        if static:
            sim.prepare()
            sim.step_static_scratch(sc.steps)
        else:
            sim.step(sc.steps)
        sim.synchronize()
        return sim.read_probes(0, sc.steps), sim.fields(), sim.cpml_profiles()


@pytest.mark.parametrize("schedule", [1, 2])
@pytest.mark.parametrize("dims", [(37, 29, 23), (64, 40, 33)])
def test_plates_vs_oracle_bitwise(gpu_lib, schedule, dims):
    sc = plate_case(*dims)
    p, f, prof = run(sc, schedule)
    po, fo = oracle.run(sc, profile_override=prof)
    assert bitwise_equal(p, po)
    assert bitwise_equal(f, fo)
    # the plates change the result
    sc0 = plate_case(*dims)
    sc0.plates = []
    p0, _ = oracle.run(sc0, profile_override=prof)
    assert not np.array_equal(p0, po)


def test_plates_static_scratch(gpu_lib):
    sc = plate_case(30, 26, 20, steps=40, pml=(3, 3, 3, 3, 3, 3))
    sc.plates[0] = S.Plate(2, (0, 0, 4, 29, 25, 4), 1e10, 1e10)
    p1, f1, _ = run(sc, 2)
    p2, f2, _ = run(sc, 0, static=True)
    assert bitwise_equal(p1, p2) and bitwise_equal(f1, f2)


def test_plate_validation(gpu_lib):
    from fdtd_gb300 import solver
    sc = plate_case()
    with solver.Simulation.from_scenario(sc) as sim:
        for axis, box in [(3, (1, 1, 1, 2, 2, 2)), (2, (1, 1, 1, 0, 2, 2)), (2, (1, 1, 40, 2, 2, 40))]:
            with pytest.raises(solver.FDTDError) as e:
                sim.add_plate(axis, box, 1.0, 1.0)
            assert e.value.code == FDTD_ERR_INVALID
        with pytest.raises(solver.FDTDError) as e:
            sim.add_plate(2, (1, 1, 1, 2, 2, 1), -1.0, 1.0)
        assert e.value.code == FDTD_ERR_INVALID
        # an x plate covering the lumped source's Ez edges
        sim.add_plate(0, (14, 10, 4, 14, 14, 9), 1e6, 1e6)
        with pytest.raises(solver.FDTDError) as e:
            sim.prepare()
        assert "lumped" in str(e.value)
    with solver.Simulation.from_scenario(plate_case()) as sim:
        with pytest.raises(solver.FDTDError) as e:
            sim.set_design_region((16, 16, 12, 20, 20, 15), np.ones((3, 4, 4), np.float32))
        assert e.value.code == FDTD_ERR_STATE
        with pytest.raises(solver.FDTDError):
            solver.Batch([sim])
