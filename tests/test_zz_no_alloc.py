"""fdtd_step_static_scratch: the fused sweep with a static device scratch, allocating nothing.

Collected last (file name) so that it also runs after every other GPU test has used the library
in this process; it must pass alone as well. Each case compares two calls in a row against
fdtd_step under the fused schedule on a second handle built from the same scenario.
"""
import numpy as np
import pytest

from conftest import bitwise_equal
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu

FDTD_ERR_STATE, FDTD_ERR_RANGE = 4, 5


def scenario():
    return S.scaled_boxes(40, 36, 32, 40, seed=5, pml=6, n_boxes=6, n_sources=2, n_probes=6, name="static_scratch")


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


@pytest.mark.parametrize("calls", [(3, 4), (2, 5)])
def test_two_calls_match_fused_step(gpu_lib, calls):
    from fdtd_gb300 import solver
    sc = scenario()
    with solver.Simulation.from_scenario(sc, solver.SCHEDULE_FUSED, probe_capacity=64) as ref, \
            solver.Simulation.from_scenario(sc, probe_capacity=64) as sim:
        sim.prepare()
        before = sim.device_bytes()
        sim.step_static_scratch(0)  # per-device set-up only
        for n in calls:
            ref.step(n)
            sim.step_static_scratch(n)
            compare(ref, sim)
        assert sim.device_bytes() == before


def test_after_fused_steps_on_the_second_buffer(gpu_lib):
    # one fdtd_step under the fused schedule leaves the state in the handle's second buffer
    from fdtd_gb300 import solver
    sc = scenario()
    with solver.Simulation.from_scenario(sc, solver.SCHEDULE_FUSED, probe_capacity=64) as ref, \
            solver.Simulation.from_scenario(sc, solver.SCHEDULE_FUSED, probe_capacity=64) as sim:
        ref.step(1)
        sim.step(1)
        for n in (3, 3):
            ref.step(n)
            sim.step_static_scratch(n)
            compare(ref, sim)


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
