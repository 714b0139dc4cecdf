"""fdtd_step_static_scratch: the fused sweep with a static device scratch, allocating nothing.

Collected last (file name) so that it also runs after every other GPU test has used the library
in this process; it must pass alone as well. Each case compares two calls in a row against
fdtd_step under the fused schedule on a second handle built from the same scenario, and checks
that the device's free memory (cudaMemGetInfo) and the handle's own allocation counter do not
move across the static calls.
"""
import dataclasses

import numpy as np
import pytest

import golden_scenarios as gs
from conftest import bitwise_equal
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu

FDTD_ERR_STATE, FDTD_ERR_RANGE = 4, 5


def scenario():
    return S.scaled_boxes(40, 36, 32, 40, seed=5, pml=6, n_boxes=6, n_sources=2, n_probes=6, name="static_scratch")


def other_layout():
    """Different dimensions and CPML thicknesses from scenario(): its field and CPML pieces sit at
    other offsets of the scratch, so a later call would see stale data if it relied on any."""
    sc = S.scaled_boxes(52, 30, 28, 20, seed=9, pml=4, n_boxes=5, n_sources=1, n_probes=3, name="other_layout")
    return dataclasses.replace(sc, pml=(3, 5, 4, 2, 5, 3))


def state(sim):
    import torch
    buf = torch.empty(sim.state_bytes(), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    sim.save_state(buf.data_ptr())
    return buf.cpu().numpy()


def compare(ref, sim):
    ref.synchronize()
    sim.synchronize()
    assert ref.current_step == sim.current_step
    assert bitwise_equal(ref.fields(), sim.fields())
    n = ref.current_step
    assert bitwise_equal(ref.read_probes(0, n), sim.read_probes(0, n))
    assert np.array_equal(state(ref), state(sim))


def free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def static_calls(ref, sim, calls):
    """fdtd_step on ref and fdtd_step_static_scratch on sim for each count; the device's free
    memory and sim's allocation counter must not move across the static calls."""
    before = sim.device_bytes()
    for n in calls:
        ref.step(n)  # first: any module the step kernels live in is loaded before measuring
        free0 = free_bytes()
        sim.step_static_scratch(n)
        sim.synchronize()
        assert free_bytes() == free0, "device memory changed across fdtd_step_static_scratch"
        compare(ref, sim)
    assert sim.device_bytes() == before


def dirty_scratch():
    """Leave data of another grid layout in the scratch (odd count: the result is copied back out
    of it, so the scratch keeps that grid's fields and CPML memory)."""
    from fdtd_gb300 import solver
    with solver.Simulation.from_scenario(other_layout(), probe_capacity=16) as sim:
        sim.prepare()
        sim.step_static_scratch(5)
        sim.synchronize()


@pytest.mark.parametrize("calls", [(3, 4), (2, 5)])
def test_two_calls_match_fused_step(gpu_lib, calls):
    from fdtd_gb300 import solver
    dirty_scratch()
    sc = scenario()
    with solver.Simulation.from_scenario(sc, solver.SCHEDULE_FUSED, probe_capacity=64) as ref, \
            solver.Simulation.from_scenario(sc, probe_capacity=64) as sim:
        sim.prepare()
        sim.step_static_scratch(0)  # per-device set-up only
        static_calls(ref, sim, calls)


def test_after_fused_steps_on_the_second_buffer(gpu_lib):
    # one fdtd_step under the fused schedule leaves the state in the handle's second buffer
    from fdtd_gb300 import solver
    sc = scenario()
    with solver.Simulation.from_scenario(sc, solver.SCHEDULE_FUSED, probe_capacity=64) as ref, \
            solver.Simulation.from_scenario(sc, solver.SCHEDULE_FUSED, probe_capacity=64) as sim:
        ref.step(1)
        sim.step(1)
        static_calls(ref, sim, (3, 3))


def test_plates_and_lumped_elements(gpu_lib):
    """Plates (k_plate_e), a lumped source and a resistor, CPML on every face."""
    from fdtd_gb300 import solver
    dirty_scratch()
    sc = gs.plates_scenario()
    with solver.Simulation.from_scenario(sc, solver.SCHEDULE_FUSED, probe_capacity=64) as ref, \
            solver.Simulation.from_scenario(sc, probe_capacity=64) as sim:
        sim.prepare()
        sim.step_static_scratch(0)
        static_calls(ref, sim, (5, 6))


def test_design_region(gpu_lib):
    """A design region (k_design_e and the tiles left out of the sweep around it)."""
    from fdtd_gb300 import solver
    dirty_scratch()
    prob = S.design_problem(n=40, steps=40, design=(8, 8, 6), pml=6)
    sims = []
    try:
        for schedule in (solver.SCHEDULE_FUSED, solver.SCHEDULE_AUTO):
            sim = solver.Simulation.from_scenario(prob.scenario, schedule, probe_capacity=64)
            sim.add_probe(S.EZ, *prob.probe)
            sim.set_design_region(prob.box, prob.eps)
            sims.append(sim)
        ref, sim = sims
        sim.prepare()
        sim.step_static_scratch(0)
        static_calls(ref, sim, (7, 4))
    finally:
        for s in sims:
            s.close()


def test_rejects_unprepared_and_oversize(gpu_lib):
    from fdtd_gb300 import solver
    sc = scenario()
    with solver.Simulation.from_scenario(sc) as sim:
        sim.add_probe(2, 5, 5, 5)  # a change after preparation
        with pytest.raises(solver.FDTDError) as e:
            sim.step_static_scratch(1)
        assert e.value.code == FDTD_ERR_STATE
    big = S.vacuum_cube(128, 4, pml=10, name="big")
    with solver.Simulation.from_scenario(big) as sim:
        sim.prepare()
        with pytest.raises(solver.FDTDError) as e:
            sim.step_static_scratch(1)
        assert e.value.code == FDTD_ERR_RANGE
        assert "static scratch" in str(e.value)
