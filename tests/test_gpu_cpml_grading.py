"""CPML grading from a reflection coefficient (fdtd_set_cpml_grading).

- the profiles follow sigma_max = -(m + 1) ln(r0) / (2 eta0 P delta) with the reference's kappa and
  alpha profiles and recurrence coefficients, checked against the formulas in FP64, per slab
  thickness (asymmetric slabs get their own sigma_max);
- a run with that grading equals the oracle run on the same profiles bit for bit, so the update
  takes the new profiles everywhere (fused and two-pass alike);
- r0 = 0 restores the reference's profiles exactly; invalid r0 is rejected;
- a pulse leaving the grid through either grading leaves a small residue behind.
"""
import numpy as np
import pytest

import oracle
from conftest import bitwise_equal
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu


def grading_fp64(n, pn, pp, delta, dt, eps0, mu0, r0):
    """The six profiles of one axis in FP64: b_e, a_e, b_m, a_m, kappa_e, kappa_m."""
    m = 3.0
    out = {k: np.full(n, np.nan) for k in ("b_e", "a_e", "b_m", "a_m", "k_e", "k_m")}
    eta0 = np.sqrt(mu0 / eps0)
    for q in range(n):
        if q < pn:
            P, roe, rom = pn, (pn - q - 0.75) / pn, (pn - q - 0.25) / pn
        elif q >= n - pp:
            P, roe, rom = pp, (q - (n - pp - 1) - 0.75) / pp, (q - (n - pp - 1) - 0.25) / pp
        else:
            continue
        smax = -(m + 1) * np.log(r0) / (2 * eta0 * P * delta)
        se, sm = smax * roe ** m, smax * rom ** m * (mu0 / eps0)
        ke, km = 1 + 4 * roe ** m, 1 + 4 * rom ** m
        ae_, am_ = 0.05 * (1 - roe), 0.05 * (1 - rom) * (mu0 / eps0)
        be = np.exp(-(dt / eps0) * (se / ke + ae_))
        bm = np.exp(-(dt / mu0) * (sm / km + am_))
        out["b_e"][q], out["b_m"][q] = be, bm
        out["a_e"][q] = (be - 1) * se / (delta * ke * (se + ke * ae_))
        out["a_m"][q] = (bm - 1) * sm / (delta * km * (sm + km * am_))
        out["k_e"][q], out["k_m"][q] = ke, km
    return out


def case(r0, schedule=1):
    sc = S.scaled_boxes(64, 56, 48, 40, seed=21, pml=6, n_boxes=6, n_sources=1, n_probes=6, name="grading")
    sc.pml = (6, 9, 5, 8, 7, 4)
    sc.cpml_r0 = r0
    return sc


@pytest.mark.parametrize("r0", [1e-6, 1e-3])
def test_profiles_follow_reflection_coefficient(gpu_lib, r0):
    from fdtd_gb300 import solver
    sc = case(r0)
    with solver.Simulation.from_scenario(sc) as sim:
        prof = sim.cpml_profiles()
    dims = {"x": (sc.nx, sc.pml[0], sc.pml[1], sc.dx), "y": (sc.ny, sc.pml[2], sc.pml[3], sc.dy),
            "z": (sc.nz, sc.pml[4], sc.pml[5], sc.dz)}
    for ax, (n, pn, pp, d) in dims.items():
        ref = grading_fp64(n, pn, pp, d, np.float32(sc.dt), np.float32(sc.eps0), np.float32(sc.mu0), r0)
        slab = ~np.isnan(ref["b_e"])
        for k in ("b_e", "b_m", "k_e", "k_m"):
            np.testing.assert_allclose(prof[k + ax][slab], ref[k][slab], rtol=2e-6, err_msg=k + ax)
        for k in ("a_e", "a_m"):  # (b - 1) cancels: a few FP32 ulps of b become 1e-4 of a
            np.testing.assert_allclose(prof[k + ax][slab], ref[k][slab], rtol=5e-4, err_msg=k + ax)


@pytest.mark.parametrize("schedule", [1, 2])
def test_run_equals_oracle_on_the_same_profiles(gpu_lib, schedule):
    from fdtd_gb300 import solver
    sc = case(1e-6)
    with solver.Simulation.from_scenario(sc, schedule, probe_capacity=sc.steps) as sim:
        sim.step(sc.steps)
        sim.synchronize()
        p, f, prof = sim.read_probes(0, sc.steps), sim.fields(), sim.cpml_profiles()
    po, fo = oracle.run(sc, profile_override=prof)
    assert bitwise_equal(p, po) and bitwise_equal(f, fo)


def test_reference_grading_restored_and_validation(gpu_lib):
    from fdtd_gb300 import solver
    sc = case(0.0)
    with solver.Simulation.from_scenario(sc) as a, solver.Simulation.from_scenario(sc) as b:
        ref = a.cpml_profiles()
        b.set_cpml_grading(1e-6)
        graded = b.cpml_profiles()
        assert not np.array_equal(graded["b_ez"], ref["b_ez"])
        b.set_cpml_grading(0.0)
        back = b.cpml_profiles()
        for k in ref:
            assert np.array_equal(back[k].view(np.uint32), ref[k].view(np.uint32)), k
        for bad in (-1.0, 1.0, 2.5, float("nan")):
            with pytest.raises(solver.FDTDError):
                b.set_cpml_grading(bad)


def test_pulse_absorbed_with_either_grading(gpu_lib):
    """A pulse from the centre of a 48^3 vacuum grid: after it has crossed into the CPML (300 steps),
    the field energy left in the interior is a small fraction of its peak, with either grading."""
    from fdtd_gb300 import solver
    for r0 in (0.0, 1e-6):
        sc = S.vacuum_cube(48, 300, pml=10, name="absorb")
        sc.cpml_r0 = r0
        sc.probes = []
        with solver.Simulation.from_scenario(sc) as sim:
            energies = []
            for _ in range(15):
                sim.step(20)
                f = sim.fields()[:, 12:36, 12:36, 12:36].astype(np.float64)
                energies.append(float((f[:3] ** 2).sum() * sc.eps0 + (f[3:] ** 2).sum() * sc.mu0))
        assert energies[-1] < 1e-2 * max(energies), (r0, energies[-1] / max(energies))
