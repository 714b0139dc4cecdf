"""x-directed lumped elements (fdtd_add_lumped_source with axis 0; the reference's defineSourceX,
fdtdrav.h:1311-1365): Ex edges i in [is,ie), j in [js,ie] (its j bound is the box's ie), k in
[ks,ke] take its load coefficients; the reference never injects them (calc_e, fdtdrav.h:681). A run
with such elements (one inside a CPML slab, one over a dielectric boundary) against the reference's
own kernels on the harness and against the oracle, bit for bit."""
import dataclasses

import numpy as np
import pytest

import oracle
from conftest import bitwise_equal, rel_l2
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu

FIELDS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def scenario(steps=150):
    sc = S.vacuum_cube(36, steps, pml=4, name="xsource")
    sc.nx, sc.ny, sc.nz = 36, 32, 28
    sc.materials.append(S.Material(eps_r=4.0, sigma_e=0.01))
    sc.bricks.append(S.Brick((4, 4, 4, 32, 16, 12), 1))
    sc.sources = [S.LumpedSource((18, 16, 12, 18, 16, 15), 50.0, S.gaussian_derivative(steps, sc.dt, 20e9, 1e-3))]
    # (is, js, ks, ie, je, ke): Ex i in [is, ie), j in [js, ie], k in [ks, ke]
    sc.x_sources = [S.LumpedSource((10, 14, 10, 15, 15, 12), 50.0, np.zeros(0, np.float32)),
                    S.LumpedSource((20, 2, 2, 23, 3, 3), 75.0, np.zeros(0, np.float32))]
    # probes outside the CPML slabs (the harness samples after the whole step, the solver's
    # probes before the CPML correction, as sampleField does); the element inside the slabs is
    # checked through the final fields
    sc.probes = [S.Probe(S.EX, 12, 14, 11), S.Probe(S.EX, 21, 10, 5), S.Probe(S.EZ, 14, 16, 12),
                 S.Probe(S.HY, 12, 15, 11), S.Probe(S.EY, 11, 14, 10)]
    return sc


def test_xsource_coefficients_vs_reference(gpu_lib):
    """Cexe / Cexhz / Cexhy after the reference's setup with defineSourceX equal the oracle's."""
    import refharness
    if not refharness.available():
        pytest.skip("reference-kernel harness not built")
    sc = scenario()
    h = refharness.RefHarness()
    try:
        h.setup(sc)
        ref = {n: h.get(n) for n in ("Cexe", "Cexhz", "Cexhy")}
    finally:
        h.close()
    for n, r in ref.items():
        assert bitwise_equal(oracle.coef(sc, n), r), n


@pytest.mark.parametrize("schedule", [1, 2])
def test_xsource_run_vs_reference_and_oracle(gpu_lib, schedule):
    import refharness
    from fdtd_gb300 import solver
    sc = scenario()
    with solver.Simulation.from_scenario(sc, schedule, probe_capacity=sc.steps) as sim:
        sim.step(sc.steps)
        sim.synchronize()
        p, f, prof = sim.read_probes(0, sc.steps), sim.fields(), sim.cpml_profiles()
    assert np.abs(p).max() > 0
    po, fo = oracle.run(sc, profile_override=prof)
    assert bitwise_equal(p, po), rel_l2(p, po)
    assert bitwise_equal(f, fo)
    if not refharness.available():
        pytest.skip("reference-kernel harness not built")
    h = refharness.RefHarness()
    try:
        h.setup(sc)
        p_ref, _ = h.run(sc.steps, src_slot=0, signal=sc.signal_per_node(0), probes=sc.probes)
        f_ref = h.fields()
    finally:
        h.close()
    assert bitwise_equal(p, p_ref), rel_l2(p, p_ref)
    for c, n in enumerate(FIELDS):
        assert bitwise_equal(f[c], f_ref[n]), (n, rel_l2(f[c], f_ref[n]))


def test_xsource_validation(gpu_lib):
    from fdtd_gb300 import solver
    sc = scenario()
    with solver.Simulation.from_scenario(sc) as sim:
        for box in [(10, 14, 10, 10, 15, 12),    # empty i range
                    (10, 0, 10, 15, 15, 12),     # j = 0 (boundary row)
                    (10, 14, 0, 15, 15, 12),     # k = 0
                    (30, 14, 10, 35, 15, 12)]:   # j bound ie beyond the updated rows
            with pytest.raises(solver.FDTDError):
                sim.add_source(box, 50.0, np.zeros(0, np.float32), axis=0)
        with pytest.raises(solver.FDTDError):  # shares Ex edges with the first one
            sim.add_source((12, 14, 11, 16, 15, 11), 50.0, np.zeros(0, np.float32), axis=0)
        with pytest.raises(solver.FDTDError):  # no x-directed resistor in the reference
            sim.add_resistor((10, 14, 10, 15, 15, 12), 50.0, axis=0)
