"""GPU behaviour of the C ABI: checkpoint/resume, the probe ring buffer, streams, errors."""
import ctypes

import numpy as np
import pytest

import golden_scenarios as gs
from conftest import bitwise_equal
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu


def small():
    sc = S.scaled_boxes(28, 24, 20, 60, seed=21, pml=4, n_boxes=5, n_sources=1, n_probes=4, name="api")
    return sc


def test_save_load_state_roundtrip(gpu_lib):
    import torch
    from fdtd_gb300 import solver
    sc = small()
    with solver.Simulation.from_scenario(sc) as sim:
        sim.step(20)
        buf = torch.empty(sim.state_bytes(), dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        sim.save_state(buf.data_ptr())
        sim.step(25)
        sim.synchronize()
        a = sim.fields()
        pa = sim.read_probes(20, 25)
        sim.load_state(buf.data_ptr())
        assert sim.current_step == 20
        sim.step(25)
        sim.synchronize()
        b = sim.fields()
        pb = sim.read_probes(20, 25)
    assert bitwise_equal(a, b) and bitwise_equal(pa, pb)


def test_probe_ring_wraps(gpu_lib):
    from fdtd_gb300 import solver
    sc = small()
    with solver.Simulation.from_scenario(sc, probe_capacity=7) as sim:
        sim.step(30)
        sim.synchronize()
        last = sim.read_probes(23, 7)
        with pytest.raises(solver.FDTDError) as e:
            sim.read_probes(10, 5)
        assert e.value.code == 5  # FDTD_ERR_RANGE
    with solver.Simulation.from_scenario(sc, probe_capacity=64) as sim:
        sim.step(30)
        sim.synchronize()
        full = sim.read_probes(0, 30)
    assert bitwise_equal(last, full[23:30])


def test_device_bytes_follow_reallocation(gpu_lib):
    """Buffers rebuilt with another size (the probe ring here) leave fdtd_device_bytes counting
    what the handle holds now, not what it ever allocated."""
    from fdtd_gb300 import solver
    sc = small()
    with solver.Simulation.from_scenario(sc, probe_capacity=16) as sim:
        sim.prepare()
        base = sim.device_bytes()
        sim.set_probe_capacity(1 << 16)
        sim.prepare()
        big = sim.device_bytes()
        assert big > base
        sim.set_probe_capacity(16)
        sim.prepare()
        assert sim.device_bytes() == base


def test_steps_in_chunks_equal_one_call(gpu_lib):
    from fdtd_gb300 import solver
    sc = small()
    with solver.Simulation.from_scenario(sc) as sim:
        for _ in range(6):
            sim.step(5)
        sim.synchronize()
        a = sim.fields()
    with solver.Simulation.from_scenario(sc) as sim:
        sim.step(30)
        sim.synchronize()
        b = sim.fields()
    assert bitwise_equal(a, b)


def test_caller_stream(gpu_lib):
    import torch
    from fdtd_gb300 import solver
    sc = small()
    s = torch.cuda.Stream()
    with solver.Simulation.from_scenario(sc) as sim:
        sim.set_stream(s.cuda_stream)
        sim.step(30)
        sim.synchronize()
        a = sim.fields()
    with solver.Simulation.from_scenario(sc) as sim:
        sim.step(30)
        sim.synchronize()
        b = sim.fields()
    assert bitwise_equal(a, b)


def test_device_field_copies(gpu_lib):
    import torch
    from fdtd_gb300 import solver
    sc = small()
    with solver.Simulation.from_scenario(sc) as sim:
        sim.step(12)
        t = torch.empty(sim.shape, dtype=torch.float32, device="cuda")
        sim.get_field_device(2, t.data_ptr())
        sim.synchronize()
        assert bitwise_equal(t.cpu().numpy(), sim.get_field(2))
        t.mul_(0.5)
        torch.cuda.synchronize()
        sim.set_field_device(2, t.data_ptr())
        sim.synchronize()
        assert bitwise_equal(sim.get_field(2), t.cpu().numpy())


def test_argument_errors(gpu_lib):
    from fdtd_gb300 import solver
    sc = small()
    with solver.Simulation.from_scenario(sc) as sim:
        with pytest.raises(solver.FDTDError):
            sim.add_source((0, 5, 5, 0, 5, 6), 50.0, np.zeros(4, np.float32))  # on the PEC wall
        with pytest.raises(solver.FDTDError):
            sim.add_source((5, 5, 5, 5, 5, 5), 50.0, np.zeros(4, np.float32))  # empty k range
        with pytest.raises(solver.FDTDError):
            sim.add_source(sc.sources[0].box, 50.0, np.zeros(4, np.float32))  # shares an edge
        with pytest.raises(solver.FDTDError):
            sim.add_probe(7, 1, 1, 1)
        with pytest.raises(solver.FDTDError):
            sim.set_materials(np.array([[1, 0, 1, 0]], np.float32))  # sigma_m = 0 gives 0/0
        bad = np.zeros(sim.shape, np.uint8)
        bad[0, 0, 0] = 200
        with pytest.raises(solver.FDTDError):
            sim.set_material_index(bad)


def test_no_source_keeps_initial_state(gpu_lib):
    """Without excitation every node stays at the scale of the reference's initial 1.2e-38."""
    from fdtd_gb300 import solver
    sc = small()
    sc.sources = []
    with solver.Simulation.from_scenario(sc) as sim:
        sim.step(10)
        sim.synchronize()
        f = sim.fields()
    assert np.all(np.abs(f) < np.float32(1e-36))


def test_auto_schedule_trial(gpu_lib):
    """AUTO on a grid above the trial size: the first long fdtd_step call times both schedules on
    real steps and keeps one; the state equals a two-pass run bit for bit. Below the trial size
    AUTO runs two-pass and allocates nothing more."""
    import torch
    from fdtd_gb300 import solver
    sc = S.random_boxes(224, 224, 176, 12, seed=9, n_boxes=16, edge=(8, 64), pml=10, n_sources=2, n_probes=4)
    states, probes = [], []
    for schedule, tune in ((solver.SCHEDULE_AUTO, False), (solver.SCHEDULE_AUTO, True), (solver.SCHEDULE_TWO_PASS, False)):
        with solver.Simulation.from_scenario(sc, schedule, probe_capacity=12) as sim:
            if tune:  # the trial up front, undone: the run then starts from step 0 with the choice made
                sim.step(3)
                sim.tune_schedule()
                assert sim.current_step == 3
                sim.step(9)
            else:
                sim.step(12)
            sim.synchronize()
            assert sim.current_step == 12
            if schedule == solver.SCHEDULE_AUTO:
                assert sim.active_schedule in (solver.SCHEDULE_TWO_PASS, solver.SCHEDULE_FUSED)
            buf = torch.empty(sim.state_bytes(), dtype=torch.uint8, device="cuda")
            torch.cuda.synchronize()
            sim.save_state(buf.data_ptr())
            torch.cuda.synchronize()
            states.append(buf)
            probes.append(sim.read_probes(0, 12))
    for q in (0, 1):
        assert torch.equal(states[q], states[2])
        assert bitwise_equal(probes[q], probes[2])
    small_sc = small()
    with solver.Simulation.from_scenario(small_sc, probe_capacity=40) as a, \
            solver.Simulation.from_scenario(small_sc, solver.SCHEDULE_TWO_PASS, probe_capacity=40) as b:
        a.step(40)
        b.step(40)
        a.synchronize()
        b.synchronize()
        assert a.active_schedule == solver.SCHEDULE_TWO_PASS
        assert a.device_bytes() == b.device_bytes()
        assert bitwise_equal(a.fields(), b.fields())


def test_auto_schedule_direct_on_large_grids(gpu_lib):
    """AUTO on a grid of at least 64 Mi cells whose interior tiles hold most nodes: fused without a
    trial (the first call's steps are all fused steps), the same bits as two-pass."""
    import torch
    from fdtd_gb300 import solver
    sc = S.random_boxes(408, 408, 408, 10, seed=4, n_boxes=24, edge=(16, 128), pml=10, n_sources=2, n_probes=6)
    mat = sc.material_index()
    out = []
    for schedule in (solver.SCHEDULE_AUTO, solver.SCHEDULE_TWO_PASS):
        with solver.Simulation.from_scenario(sc, schedule, material_index=mat, probe_capacity=10) as sim:
            sim.step(10)
            sim.synchronize()
            if schedule == solver.SCHEDULE_AUTO:
                assert sim.active_schedule == solver.SCHEDULE_FUSED
            buf = torch.empty(sim.state_bytes(), dtype=torch.uint8, device="cuda")
            torch.cuda.synchronize()
            sim.save_state(buf.data_ptr())
            torch.cuda.synchronize()
            out.append((buf.cpu(), sim.read_probes(0, 10)))
    assert torch.equal(out[0][0], out[1][0])
    assert bitwise_equal(out[0][1], out[1][1])
