"""GPU design region and discrete adjoint against the oracle.

- the forward with a design region equals the FP32 oracle bit for bit (GPU CPML profiles);
- the adjoint gradient (checkpointed and resident history) agrees with the oracle's FP64 adjoint
  and with central finite differences of the FP64 oracle forward (h = 1e-3) within 1e-3 relative;
- the checkpointed and the resident backward give identical bits;
- the torch.autograd.Function returns the same gradient through autograd.
"""
import numpy as np
import pytest

import oracle
from conftest import bitwise_equal
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-3  # relative, per the figure-of-merit gradient requirement


def design_case(seed=0, steps=160):
    sc = S.vacuum_cube(24, steps, pml=4, name="adjoint_gpu")
    sc.nx, sc.ny, sc.nz = 24, 22, 20
    sc.sources = [S.LumpedSource((7, 11, 9, 7, 11, 10), 50.0, S.gaussian_derivative(steps, sc.dt, 30e9, 1e-3))]
    sc.probes = [S.Probe(2, 18, 11, 9)]
    sc.materials.append(S.Material(eps_r=3.0, sigma_e=0.02))
    sc.bricks.append(S.Brick((17, 4, 5, 21, 9, 8), 1))  # a lossy dielectric next to the design region
    box = (10, 8, 7, 16, 14, 11)
    rng = np.random.default_rng(seed)
    eps = rng.uniform(1, 12, size=(box[5] - box[2], box[4] - box[1], box[3] - box[0])).astype(np.float32)
    return sc, box, eps, (18, 11, 9)


def gpu_grad(sc, box, eps, probe, K):
    from fdtd_gb300 import solver
    with solver.Simulation.from_scenario(sc, probe_capacity=sc.steps) as sim:
        sim.set_design_region(box, eps)
        J = sim.adjoint_forward(sc.steps, probe, K)
        g = sim.adjoint_backward()
        assert sim.current_step == sc.steps
    return J, g


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_design_forward_bitwise(gpu_lib):
    from fdtd_gb300 import solver
    sc, box, eps, probe = design_case()
    with solver.Simulation.from_scenario(sc, probe_capacity=sc.steps) as sim:
        sim.set_design_region(box, eps)
        sim.step(sc.steps)
        sim.synchronize()
        f = sim.fields()
        p = sim.read_probes(0, sc.steps)
        prof = sim.cpml_profiles()
    po, fo = oracle.run(sc, profile_override=prof, design=(box, eps.astype(np.float64)))
    assert bitwise_equal(p, po) and bitwise_equal(f, fo)


@pytest.mark.parametrize("schedule", [1, 2])
def test_design_forward_bitwise_swept(gpu_lib, schedule):
    """A grid with interior tiles: under the fused schedule the tiles that reach the design region's
    edge box stay out of the sweep, and the result still equals the oracle bit for bit."""
    from fdtd_gb300 import solver
    steps = 60
    sc = S.vacuum_cube(80, steps, pml=6, name="design_swept")
    sc.nx, sc.ny, sc.nz = 80, 56, 32
    sc.sources = [S.LumpedSource((20, 28, 15, 20, 28, 16), 50.0, S.gaussian_derivative(steps, sc.dt, 30e9, 1e-3))]
    sc.probes = [S.Probe(2, 50, 28, 15), S.Probe(3, 35, 25, 14)]
    sc.materials.append(S.Material(eps_r=4.0, sigma_e=0.01))
    sc.bricks.append(S.Brick((44, 10, 8, 60, 40, 24), 1))
    box = (30, 20, 10, 40, 30, 18)
    rng = np.random.default_rng(3)
    eps = rng.uniform(1, 12, size=(box[5] - box[2], box[4] - box[1], box[3] - box[0])).astype(np.float32)
    with solver.Simulation.from_scenario(sc, schedule, probe_capacity=steps) as sim:
        sim.set_design_region(box, eps)
        sim.step(steps)
        sim.synchronize()
        f = sim.fields()
        p = sim.read_probes(0, steps)
        prof = sim.cpml_profiles()
    po, fo = oracle.run(sc, profile_override=prof, design=(box, eps.astype(np.float64)))
    assert bitwise_equal(p, po) and bitwise_equal(f, fo)


@pytest.mark.parametrize("K", [0, 16])
def test_gradient_matches_fp64_adjoint(gpu_lib, K):
    sc, box, eps, probe = design_case()
    J, g = gpu_grad(sc, box, eps, probe, K)
    J64, g64 = oracle.fom_grad(sc, probe, box, eps.astype(np.float64), precision="f64")
    assert abs(J - J64) <= 1e-4 * abs(J64)
    assert rel(g, g64) < GRAD_TOL, rel(g, g64)


def test_checkpointed_equals_resident(gpu_lib):
    sc, box, eps, probe = design_case(2)
    J0, g0 = gpu_grad(sc, box, eps, probe, 0)
    J1, g1 = gpu_grad(sc, box, eps, probe, 7)  # segments of uneven length
    assert J0 == J1 and np.array_equal(g0, g1)


def test_gradient_matches_central_differences(gpu_lib):
    sc, box, eps, probe = design_case(1)
    _, g = gpu_grad(sc, box, eps, probe, 16)
    e64 = eps.astype(np.float64)
    rng = np.random.default_rng(5)
    h = 1e-3
    for _ in range(6):
        v = tuple(int(rng.integers(0, s)) for s in eps.shape)
        e1 = e64.copy(); e1[v] += h
        e2 = e64.copy(); e2[v] -= h
        fd = (oracle.fom_grad(sc, probe, box, e1, grad=False) - oracle.fom_grad(sc, probe, box, e2, grad=False)) / (2 * h)
        assert abs(g[v] - fd) <= GRAD_TOL * abs(fd), (v, g[v], fd)


def test_autograd_function(gpu_lib):
    import torch
    from fdtd_gb300.adjoint import probe_energy
    sc, box, eps, probe = design_case(3)
    x = torch.tensor(eps, dtype=torch.float32, requires_grad=True)
    J = probe_energy(x, sc, box, probe, sc.steps, checkpoint_every=32)
    (2.0 * J).backward()
    _, g = gpu_grad(sc, box, eps, probe, 32)
    assert np.array_equal(x.grad.numpy(), (2.0 * g).astype(np.float32))


def test_design_region_validation(gpu_lib):
    from fdtd_gb300 import solver
    sc, box, eps, probe = design_case()
    with solver.Simulation.from_scenario(sc) as sim:
        with pytest.raises(solver.FDTDError):
            sim.set_design_region((2, 8, 7, 8, 14, 11), np.ones((4, 6, 6), np.float32))  # reaches the CPML
        with pytest.raises(solver.FDTDError):
            sim.set_design_region((6, 9, 8, 9, 12, 11), np.ones((3, 3, 3), np.float32))  # touches the source edge
        with pytest.raises(solver.FDTDError):
            sim.adjoint_forward(10, probe, 4)  # no design region yet


def test_design_problem_sixteen_voxels(gpu_lib):
    """The 128^3 adjoint workload's structure at 48^3 / 600 steps: 16 seeded voxels against central
    differences of the FP64 oracle forward, h = 1e-3."""
    d = S.design_problem(48, 600, (12, 12, 6), seed=9)
    sc = d.scenario
    _, g = gpu_grad(sc, d.box, d.eps, d.probe, 64)
    e64 = d.eps.astype(np.float64)
    rng = np.random.default_rng(16)
    h = 1e-3
    worst = 0.0
    for _ in range(16):
        v = tuple(int(rng.integers(0, s)) for s in d.eps.shape)
        e1 = e64.copy(); e1[v] += h
        e2 = e64.copy(); e2[v] -= h
        fd = (oracle.fom_grad(sc, d.probe, d.box, e1, grad=False) -
              oracle.fom_grad(sc, d.probe, d.box, e2, grad=False)) / (2 * h)
        worst = max(worst, abs(g[v] - fd) / abs(fd))
    assert worst <= GRAD_TOL, worst


def test_full_size_workload_against_fp64_reference(gpu_lib):
    """The 128^3 / 4000-step workload itself (32 x 32 x 16 design region, checkpoints every 64
    steps): the GPU gradient against the FP64 oracle's adjoint gradient over the whole design region
    and against central differences of the FP64 oracle forward at 16 seeded voxels, both recorded
    in tests/golden/adjoint_c4.npz by tests/golden/make_adjoint_c4.py."""
    from conftest import GOLDEN
    import os
    path = os.path.join(GOLDEN, "adjoint_c4.npz")
    if not os.path.exists(path):
        pytest.skip("reference gradient not generated")
    ref = np.load(path)
    d = S.design_problem(128, int(ref["steps"]))
    assert tuple(ref["box"]) == tuple(d.box) and tuple(ref["probe"]) == tuple(d.probe)
    J, g = gpu_grad(d.scenario, d.box, d.eps, d.probe, 64)
    assert abs(J - float(ref["J"])) <= GRAD_TOL * float(ref["J"])
    g64 = ref["grad"]
    assert rel(g, g64) <= GRAD_TOL, rel(g, g64)
    for v, fd in zip(ref["voxels"], ref["fd"]):
        v = tuple(int(x) for x in v)
        assert abs(g[v] - fd) <= GRAD_TOL * abs(fd), (v, g[v], fd)


@pytest.mark.parametrize("K", [0, 16])
def test_batch_adjoint_equals_per_instance(gpu_lib, K):
    """fdtd_batch_adjoint over three designs (different eps_r, probes and design boxes; each
    simulation on its own stream) gives the J and gradients of per-instance forward + backward,
    bit for bit, and leaves every simulation at the forward's final step."""
    import torch
    from fdtd_gb300 import solver
    cases = []
    for seed, shift in ((1, 0), (2, 1), (5, -1)):
        sc, box, eps, probe = design_case(seed, steps=120)
        box = (box[0] + shift, box[1], box[2], box[3] + shift, box[4], box[5])
        probe = (probe[0], probe[1] + shift, probe[2])
        cases.append((sc, box, eps, probe))
    want = [gpu_grad(sc, box, eps, probe, K) for sc, box, eps, probe in cases]
    streams = [torch.cuda.Stream() for _ in cases]
    sims = []
    try:
        for (sc, box, eps, probe), st in zip(cases, streams):
            sim = solver.Simulation.from_scenario(sc, probe_capacity=sc.steps)
            sims.append(sim)
            sim.set_stream(st.cuda_stream)
            sim.set_design_region(box, eps)
        J, grads = solver.batch_adjoint(sims, 120, [c[3] for c in cases], K)
        for sim in sims:
            assert sim.current_step == 120
    finally:
        for sim in sims:
            sim.close()
    for (Jw, gw), Jb, gb in zip(want, J, grads):
        assert Jb == Jw
        assert np.array_equal(gb, gw)


def test_batch_adjoint_validation(gpu_lib):
    from fdtd_gb300 import solver
    sc, box, eps, probe = design_case(steps=20)
    with solver.Simulation.from_scenario(sc, probe_capacity=20) as a, \
            solver.Simulation.from_scenario(sc, probe_capacity=20) as b:
        a.set_design_region(box, eps)
        with pytest.raises(solver.FDTDError):
            solver.batch_adjoint([a, b], 20, [probe, probe])  # b has no design region
        with pytest.raises(solver.FDTDError):
            solver.batch_adjoint([a, a], 20, [probe, probe])  # a handle twice


@pytest.mark.parametrize("K", [0, 16])
def test_repeated_adjoint_reuses_buffers(gpu_lib, K):
    """A second forward + backward of the same length on one handle (its buffers kept from the
    first) equals a fresh handle's forward + backward started from the same state and step."""
    from fdtd_gb300 import solver
    sc, box, eps, probe = design_case(7, steps=80)
    with solver.Simulation.from_scenario(sc, probe_capacity=160) as a, \
            solver.Simulation.from_scenario(sc, probe_capacity=160) as b:
        for s in (a, b):
            s.set_design_region(box, eps)
        a.adjoint_forward(80, probe, K)
        a.adjoint_backward()
        J1 = a.adjoint_forward(80, probe, K)
        g1 = a.adjoint_backward()
        b.step(80)
        J2 = b.adjoint_forward(80, probe, K)
        g2 = b.adjoint_backward()
        assert a.current_step == b.current_step == 160
        assert J1 == J2 and np.array_equal(g1, g2)
        assert bitwise_equal(a.fields(), b.fields())


def test_backward_keeps_probe_ring(gpu_lib):
    """A probe ring shorter than the run: after forward + backward (K = 16, segments recomputed)
    the ring holds the forward's last samples, as after plain steps; the recompute samples nothing."""
    from fdtd_gb300 import solver
    sc, box, eps, probe = design_case(4, steps=96)
    with solver.Simulation.from_scenario(sc, probe_capacity=24) as a, \
            solver.Simulation.from_scenario(sc, probe_capacity=24) as b:
        for s in (a, b):
            s.set_design_region(box, eps)
        a.adjoint_forward(96, probe, 16)
        a.adjoint_backward()
        b.step(96)
        b.synchronize()
        assert bitwise_equal(a.read_probes(72, 24), b.read_probes(72, 24))
        assert bitwise_equal(a.fields(), b.fields())


def test_checkpointed_equals_resident_fused(gpu_lib):
    """Under the fused schedule the forward ping-pongs between two field buffers, and the segment
    recompute (two-pass, in place, over the shrinking box around the design region) starts from
    checkpoints of either buffer: the gradient equals the resident history's bit for bit."""
    from fdtd_gb300 import solver
    steps = 50
    sc = S.vacuum_cube(80, steps, pml=6, name="adjoint_fused")
    sc.nx, sc.ny, sc.nz = 80, 56, 40
    sc.sources = [S.LumpedSource((20, 28, 19, 20, 28, 20), 50.0, S.gaussian_derivative(steps, sc.dt, 30e9, 1e-3))]
    sc.probes = [S.Probe(2, 52, 28, 19), S.Probe(3, 34, 40, 20)]
    sc.materials.append(S.Material(eps_r=4.0, sigma_e=0.01))
    sc.bricks.append(S.Brick((44, 10, 8, 60, 40, 30), 1))
    box = (30, 22, 15, 38, 30, 23)
    eps = np.random.default_rng(8).uniform(1, 12, size=(8, 8, 8)).astype(np.float32)
    probe = (52, 28, 19)
    out = []
    for K in (0, 9, 20):  # K = 20: box checkpoints every 9 steps inside each segment
        with solver.Simulation.from_scenario(sc, 2, probe_capacity=steps) as sim:
            sim.set_design_region(box, eps)
            J = sim.adjoint_forward(steps, probe, K)
            g = sim.adjoint_backward()
            out.append((J, g, sim.fields()))
    for J, g, f in out[1:]:
        assert J == out[0][0] and np.array_equal(g, out[0][1])
        assert bitwise_equal(f, out[0][2])


@pytest.mark.parametrize("probe", [(12, 10, 9), (18, 11, 9)])
def test_fom_records_same_in_both_schedules(gpu_lib, probe):
    """The two-pass steps take the FoM sample and the design-region snapshots inside the design
    kernel (from the design node itself when the probe is one, first probe: inside the design
    edge box); the fused steps take them with a kernel of their own. J and the gradient agree bit
    for bit, and J matches the FP64 oracle."""
    from fdtd_gb300 import solver
    sc, box, eps, _ = design_case(6, steps=90)
    out = []
    for schedule, K in ((1, 0), (1, 16), (2, 0), (2, 16)):
        with solver.Simulation.from_scenario(sc, schedule, probe_capacity=sc.steps) as sim:
            sim.set_design_region(box, eps)
            J = sim.adjoint_forward(sc.steps, probe, K)
            out.append((J, sim.adjoint_backward()))
    for J, g in out[1:]:
        assert J == out[0][0] and np.array_equal(g, out[0][1])
    J64 = oracle.fom_grad(sc, probe, box, eps.astype(np.float64), precision="f64", grad=False)
    assert abs(out[0][0] - J64) <= 1e-4 * abs(J64)


def test_auto_adjoint_on_a_large_grid_takes_fused(gpu_lib):
    """On a grid where AUTO's direct rule chooses the fused schedule (64 Mi cells, mostly interior
    tiles), the adjoint forward applies that choice; J and the gradient equal the two-pass
    schedule's bit for bit."""
    from fdtd_gb300 import solver
    steps = 24
    sc = S.vacuum_cube(64, steps, pml=10, name="adjoint_large")
    sc.nx, sc.ny, sc.nz = 512, 512, 256
    sc.sources = [S.LumpedSource((246, 256, 128, 246, 256, 129), 50.0, S.gaussian_derivative(steps, sc.dt, 30e9, 1e-3))]
    sc.probes = []
    box, probe = (250, 248, 124, 266, 264, 132), (268, 256, 128)
    eps = np.random.default_rng(2).uniform(1, 12, size=(8, 16, 16)).astype(np.float32)
    out = []
    for schedule in (0, 1):
        with solver.Simulation.from_scenario(sc, schedule, probe_capacity=steps) as sim:
            sim.set_design_region(box, eps)
            J = sim.adjoint_forward(steps, probe, 4)
            g = sim.adjoint_backward()
            out.append((J, g, sim.active_schedule))
    assert out[0][2] == 2 and out[1][2] == 1
    assert out[0][0] == out[1][0] and np.array_equal(out[0][1], out[1][1])
    assert np.abs(out[0][1]).max() > 0


@pytest.mark.parametrize("K", [1, 2, 3, 64, 200])
def test_checkpoint_interval_edge_cases(gpu_lib, K):
    """Checkpoint intervals of one step (segments of one step: the recompute updates only the
    design edge box), two and three steps (at or below the box-checkpoint interval), and longer
    than the run (a single partial segment with box checkpoints): the gradient equals the resident
    history's bit for bit."""
    sc, box, eps, probe = design_case(9, steps=50)
    J0, g0 = gpu_grad(sc, box, eps, probe, 0)
    J1, g1 = gpu_grad(sc, box, eps, probe, K)
    assert J0 == J1 and np.array_equal(g0, g1)
