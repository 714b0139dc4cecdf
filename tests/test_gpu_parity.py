"""GPU parity: the CUDA solver against the reference's own kernels (golden fixtures) and against
the CPU oracle, through the C ABI."""
import os

import numpy as np
import pytest

import golden_scenarios as gs
import oracle
from conftest import GOLDEN, REL_L2_TOL, bitwise_equal, golden, rel_l2, rel_l2_group
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu

FIELDS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
SCHEDULES = [1, 2]  # two-pass, fused sweep


def run_gpu(sc, steps=None, schedule=0, material_index=False, fields=True):
    from fdtd_gb300 import solver
    steps = sc.steps if steps is None else steps
    mi = sc.material_index() if material_index else None
    with solver.Simulation.from_scenario(sc, schedule, material_index=mi, probe_capacity=max(steps, 1)) as sim:
        sim.step(steps)
        sim.synchronize()
        p = sim.read_probes(0, steps)
        f = sim.fields() if fields else None
        prof = sim.cpml_profiles()
    return p, f, prof


def scenarios():
    return dict((s.name, (s, full)) for s, full in gs.fixture_scenarios())


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("name", ["small_vacuum", "small_boxes", "vacuum64", "plates", "aniso"])
def test_matches_reference_kernels_bitwise(gpu_lib, name, schedule):
    """Single-source scenarios: probe series and final fields equal the reference's bit for bit."""
    sc, full = scenarios()[name]
    if not os.path.exists(os.path.join(GOLDEN, name + ".npz")):
        pytest.skip("fixture not generated")
    fix = golden(name)
    p, f, _ = run_gpu(sc, schedule=schedule)
    assert bitwise_equal(p, fix["probes"]), rel_l2(p, fix["probes"])
    for c, n in enumerate(FIELDS):
        if full:
            assert bitwise_equal(f[c], fix[n]), (n, rel_l2(f[c], fix[n]))
        else:
            assert bitwise_equal(f[c][sc.nz // 2], fix[n + "_zmid"]), n
            assert abs(np.linalg.norm(f[c].astype(np.float64)) - float(fix[n + "_l2"])) <= 1e-12 * float(fix[n + "_l2"])


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_two_sources_vs_reference(gpu_lib, schedule):
    """The reference injects one source per calc_e launch, so its two-source fixture is the sum of
    two runs; linear superposition holds to FP32 rounding."""
    sc, _ = scenarios()["two_sources"]
    fix = golden("two_sources")
    p, f, _ = run_gpu(sc, schedule=schedule)
    assert rel_l2(p, fix["probes"]) < REL_L2_TOL
    ref = [fix[n] for n in FIELDS]
    for c, n in enumerate(FIELDS):
        assert rel_l2_group(f, ref, c) < REL_L2_TOL, n


def test_cpml_profiles_equal_reference(gpu_lib):
    sc = gs.onestep_scenario()
    fix = golden("coefs_onestep")
    _, _, prof = run_gpu(sc, steps=0, fields=False)
    for a in oracle.PROFILE_NAMES:
        kind = a[:3]  # b_e / a_e / b_m / a_m
        got = prof[kind + a[-1]]
        assert bitwise_equal(got, fix["cpml_" + a][: got.size]), a


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_onestep_bitwise(gpu_lib, schedule):
    """One step from a seeded random state, with a large source signal: bit-exact against one
    reference calc_e + calc_h."""
    from fdtd_gb300 import solver
    sc = gs.onestep_scenario()
    fix = golden("onestep")
    sig = fix["signal"] if "signal" in fix.files else sc.signal_per_node(0)
    sc.sources[0].waveform = np.asarray(sig[gs.ONESTEP_M:], dtype=np.float32)  # step 0 injects sig[m]
    rng = np.random.default_rng(99)
    shape = (sc.nz, sc.ny, sc.nx)
    state = {n: rng.standard_normal(shape).astype(np.float32) for n in FIELDS}
    with solver.Simulation.from_scenario(sc, schedule) as sim:
        for c, n in enumerate(FIELDS):
            sim.set_field(c, state[n])
        sim.step(1)
        sim.synchronize()
        out = sim.fields()
    for c, n in enumerate(FIELDS):
        key = n + ("_after_e" if c < 3 else "_after_h")
        assert bitwise_equal(out[c], fix[key]), (key, rel_l2(out[c], fix[key]))


def edge_cases():
    """Small scenarios that exercise masks, padding, faces and lumped elements."""
    cases = []
    # odd sizes (row pitch > nx), asymmetric CPML, probes of every component incl. inside CPML
    sc = S.vacuum_cube(17, 45, pml=2, name="odd17")
    sc.nx, sc.ny, sc.nz = 17, 13, 11
    sc.pml = (3, 2, 2, 3, 1, 2)
    sc.sources = [S.LumpedSource((8, 6, 5, 8, 6, 6), 50.0, sc.sources[0].waveform)]
    sc.probes = [S.Probe(c, 8 + c % 2, 6, 5) for c in range(6)] + [S.Probe(S.EZ, 1, 6, 5), S.Probe(S.HY, 15, 1, 9)]
    cases.append(sc)
    # random boxes with magnetic material, two sources and two resistors, boxes reaching into CPML
    sc = S.scaled_boxes(40, 33, 29, 60, seed=3, pml=4, n_boxes=9, n_sources=2, n_probes=6, name="boxes40")
    sc.materials.append(S.Material(eps_r=4.0, sigma_e=0.03, mu_r=1.5, sigma_m=1e4))
    sc.bricks.append(S.Brick((0, 0, 10, 40, 12, 16), len(sc.materials) - 1))
    sc.resistors = [S.Resistor((20, 5, 3, 21, 5, 5), 100.0), S.Resistor((30, 25, 20, 30, 26, 22), 25.0)]
    cases.append(sc)
    # PEC walls (zero-thickness CPML on some faces), source inside a CPML slab
    sc = S.vacuum_cube(24, 30, pml=3, name="pec_faces")
    sc.pml = (0, 4, 0, 4, 3, 0)
    sc.sources = [S.LumpedSource((21, 12, 12, 21, 12, 13), 50.0, sc.sources[0].waveform)]
    sc.probes = [S.Probe(S.EZ, 5, 12, 12), S.Probe(S.HX, 20, 3, 2)]
    cases.append(sc)
    # x extent a multiple of the row pitch, multi-edge source box
    sc = S.vacuum_cube(32, 35, pml=4, name="pitch32")
    sc.sources = [S.LumpedSource((15, 15, 14, 16, 16, 17), 50.0, sc.sources[0].waveform)]
    sc.probes = [S.Probe(S.EZ, 22, 16, 15), S.Probe(S.HZ, 10, 10, 10)]
    cases.append(sc)
    return cases


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("case", range(4))
def test_vs_oracle(gpu_lib, case, schedule):
    """Bit-exact against the oracle when the oracle uses the GPU's CPML profiles; within the FP32
    parity bar with the oracle's own (host libm) profiles."""
    sc = edge_cases()[case]
    p, f, prof = run_gpu(sc, schedule=schedule)
    po, fo = oracle.run(sc, profile_override=prof)
    assert bitwise_equal(p, po), rel_l2(p, po)
    for c, n in enumerate(FIELDS):
        assert bitwise_equal(f[c], fo[c]), (n, rel_l2(f[c], fo[c]))
    po2, fo2 = oracle.run(sc)
    assert rel_l2(p, po2) < REL_L2_TOL


def test_material_index_equals_bricks(gpu_lib):
    sc = edge_cases()[1]
    p1, f1, _ = run_gpu(sc, steps=20)
    p2, f2, _ = run_gpu(sc, steps=20, material_index=True)
    assert bitwise_equal(p1, p2) and bitwise_equal(f1, f2)


def pack_state(sc, fields, psi, step):
    """State buffer of fdtd_save_state / fdtd_load_state built from dense arrays: 6 fields padded to
    the 32-float row pitch, then per CPML face (x_n, x_p, y_n, y_p, z_n, z_p) the slabs
    e0, e1, h0, h1, then an 8 x int64 header (step, nx, ny, nz)."""
    nz, ny, nx = sc.nz, sc.ny, sc.nx
    pitch = (nx + 31) // 32 * 32
    parts = []
    for c in range(6):
        a = np.zeros((nz, ny, pitch), np.float32)
        a[:, :, :nx] = fields[c]
        parts.append(a.ravel())
    P = sc.pml
    names = {0: ("Psi_eyx", "Psi_ezx", "Psi_hyx", "Psi_hzx"), 1: ("Psi_exy", "Psi_ezy", "Psi_hxy", "Psi_hzy"),
             2: ("Psi_exz", "Psi_eyz", "Psi_hxz", "Psi_hyz")}
    for f in range(6):
        ax, side = f // 2, f % 2
        n = P[f]
        for nm in names[ax]:
            v = psi[nm]
            if ax == 0:
                sl = v[:, :, :n] if side == 0 else v[:, :, nx - n:]
                parts.append(np.ascontiguousarray(sl).ravel())
            elif ax == 1:
                a = np.zeros((nz, n, pitch), np.float32)
                a[:, :, :nx] = v[:, :n, :] if side == 0 else v[:, ny - n:, :]
                parts.append(a.ravel())
            else:
                a = np.zeros((n, ny, pitch), np.float32)
                a[:, :, :nx] = v[:n] if side == 0 else v[nz - n:]
                parts.append(a.ravel())
    hdr = np.zeros(8, np.int64)
    hdr[:4] = (step, nx, ny, nz)
    return np.concatenate([np.concatenate(parts).view(np.uint8), hdr.view(np.uint8)])


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_onestep_random_psi_bitwise(gpu_lib, schedule):
    """One step from random fields and random CPML memory (loaded through the state API): fields
    bit-exact against one reference calc_e + calc_h, which pins every psi recurrence."""
    import torch
    from fdtd_gb300 import solver
    sc = gs.onestep_scenario()
    fix = golden("onestep_psi")
    sc.sources[0].waveform = gs.onestep_signal()  # single-edge source: per-edge signal = V
    rng = np.random.default_rng(77)
    shape = (sc.nz, sc.ny, sc.nx)
    names = FIELDS + tuple(oracle.PSI_NAMES)
    st = {n: rng.standard_normal(shape).astype(np.float32) for n in names}
    buf = pack_state(sc, [st[n] for n in FIELDS], st, gs.ONESTEP_M)
    with solver.Simulation.from_scenario(sc, schedule) as sim:
        assert buf.size == sim.state_bytes()
        dev = torch.from_numpy(buf).cuda()
        torch.cuda.synchronize()
        sim.load_state(dev.data_ptr())
        assert sim.current_step == gs.ONESTEP_M
        sim.step(1)
        sim.synchronize()
        out = sim.fields()
    for c, n in enumerate(FIELDS):
        key = n + ("_after_e" if c < 3 else "_after_h")
        assert bitwise_equal(out[c], fix[key]), (key, rel_l2(out[c], fix[key]))


@pytest.mark.parametrize("dims,pml", [((70, 45, 40), 0), ((61, 50, 30), 1), ((90, 37, 33), 2)])
def test_fused_thin_shell_equals_two_pass(gpu_lib, dims, pml):
    """Grids whose shell bands are 1 to 8 nodes wide (no or thin CPML): the fused schedule's shell
    items take the narrow block shapes, and the result equals the two-pass schedule bit for bit."""
    import dataclasses
    nx, ny, nz = dims
    sc = S.scaled_boxes(nx, ny, nz, 20, seed=nx + pml, pml=3, n_boxes=6, n_sources=1, n_probes=5, name="thin_shell")
    sc = dataclasses.replace(sc, pml=(pml,) * 6)
    p1, f1, _ = run_gpu(sc, schedule=1)
    p2, f2, _ = run_gpu(sc, schedule=2)
    assert bitwise_equal(p1, p2), rel_l2(p2, p1)
    assert bitwise_equal(f1, f2), rel_l2(f2, f1)


@pytest.mark.parametrize("dims", [(70, 45, 80), (33, 13, 40), (100, 17, 16)])
def test_fused_equals_two_pass(gpu_lib, dims):
    """Ragged tiles in x and y, several z-chunks per column: the fused sweep reproduces the two-pass
    schedule bit for bit (probes and all fields), and switching schedules mid-run changes nothing."""
    from fdtd_gb300 import solver
    nx, ny, nz = dims
    sc = S.scaled_boxes(nx, ny, nz, 30, seed=nx + ny, pml=3, n_boxes=8, n_sources=1, n_probes=6, name="ragged")
    p1, f1, _ = run_gpu(sc, schedule=1)
    p2, f2, _ = run_gpu(sc, schedule=2)
    assert bitwise_equal(p1, p2), rel_l2(p2, p1)
    assert bitwise_equal(f1, f2), rel_l2(f2, f1)
    with solver.Simulation.from_scenario(sc, 2, probe_capacity=30) as sim:
        sim.step(11)
        sim.set_schedule(1)
        sim.step(7)
        sim.set_schedule(2)
        sim.step(12)
        sim.synchronize()
        assert bitwise_equal(sim.read_probes(0, 30), p1)
        assert bitwise_equal(sim.fields(), f1)
