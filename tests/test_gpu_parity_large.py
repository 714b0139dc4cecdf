"""GPU parity at full size: the 512^3 random-box workload (64 boxes, 65 materials, 4 delayed
sources, 16 probes, 2000 steps) and a 1024 x 1024 x 128 slab of the 1024 x 1024 x 896 generator
(1000 steps), each run through the C ABI under the fused schedule (the one AUTO keeps at these
sizes) and through the reference's own calc_e / calc_h (fdtdrav.h:577-915, 249-573) on the same GPU.

The reference injects one source box per calc_e launch (fdtdrav.h:726), with every source box
defined as a resistive load (defineSourceZ, fdtdrav.h:1368-1426). So each source is run on its own:
the reference with that box injected, the solver with that source and the other three boxes as
50-ohm resistors (the same Ceze / Cezhy / Cezhx expressions, fdtdrav.h:1429-1483). Those runs must
agree bit for bit (probes of every step, all six final fields). The four-source run of the solver
is then compared with the sum of the reference's single-source runs at the FP32 parity bar (1e-5
relative L2): the two differ only by the rounding of the superposition.

Also here: a grid whose distinct seven-cell material combinations exceed the coefficient table's
interface rows, so interface nodes overflow to the general path inside the sweep, checked bit for
bit against the oracle under both schedules.
"""
import dataclasses
import gc

import numpy as np
import pytest

import oracle
from conftest import REL_L2_TOL, bitwise_equal, rel_l2, rel_l2_group
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu

FIELDS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
# interface rows of the coefficient table (kMaxInterfaceRows: 0x8000 - 257)
MAX_INTERFACE_ROWS = 0x8000 - 257


def _harness():
    import refharness
    if not refharness.available():
        pytest.skip("reference-kernel harness not built")
    return refharness


def _run_solver(sc, steps, schedule=2, material_index=None):
    from fdtd_gb300 import solver
    with solver.Simulation.from_scenario(sc, schedule, material_index=material_index,
                                         probe_capacity=steps) as sim:
        sim.step(steps)
        sim.synchronize()
        return sim.read_probes(0, steps), sim.fields()


def _single_source(sc, s):
    """The scenario with source s driven and the other source boxes as resistive loads."""
    others = [S.Resistor(x.box, x.resistance) for q, x in enumerate(sc.sources) if q != s]
    return dataclasses.replace(sc, sources=[sc.sources[s]], resistors=list(sc.resistors) + others)


def _check_against_reference(sc, steps):
    import torch
    rh = _harness()
    ref_p = None
    ref_f = None
    for s in range(len(sc.sources)):
        h = rh.RefHarness()
        try:
            h.setup(sc)
            p_ref, _ = h.run(steps, src_slot=s, signal=sc.signal_per_node(s), probes=sc.probes)
            f_ref = h.fields()
        finally:
            h.close()
        torch.cuda.synchronize()
        p, f = _run_solver(_single_source(sc, s), steps)
        assert bitwise_equal(p, p_ref), (s, rel_l2(p, p_ref))
        for c, n in enumerate(FIELDS):
            assert bitwise_equal(f[c], f_ref[n]), (s, n, rel_l2(f[c], f_ref[n]))
        del f
        if ref_p is None:
            ref_p = p_ref.astype(np.float64)
            ref_f = [f_ref[n].astype(np.float64) for n in FIELDS]
        else:
            ref_p += p_ref
            for c, n in enumerate(FIELDS):
                ref_f[c] += f_ref[n]
        del f_ref
        gc.collect()
    p, f = _run_solver(sc, steps)
    assert rel_l2(p, ref_p) < REL_L2_TOL, rel_l2(p, ref_p)
    for c, n in enumerate(FIELDS):
        e = rel_l2_group(f, ref_f, c)
        assert e < REL_L2_TOL, (n, e)


def test_boxes512_vs_reference_kernels(gpu_lib):
    """The 512^3 benchmark workload over its full 2000 steps."""
    sc = S.config_512()
    _check_against_reference(sc, sc.steps)


def test_slab1024_vs_reference_kernels(gpu_lib):
    """A 1024 x 1024 x 128 slab of the 1024 x 1024 x 896 generator (same seed and box sizes; the
    boxes are clipped to the slab), 1000 steps. The full domain needs 316 GB in the reference's
    336 B/cell layout, more than one GPU holds."""
    sc = S.random_boxes(1024, 1024, 128, 1000, seed=1024, edge=(32, 256), name="slab1024x1024x128")
    _check_against_reference(sc, sc.steps)


def _overflow_scenario():
    """80 x 56 x 40 nodes, 4-cell CPML, every interior cell a random one of 200 materials
    (eps_r 1-12, sigma 0-0.05, a few magnetic), one source, one resistor, 8 probes, 60 steps."""
    sc = S.scaled_boxes(80, 56, 40, 60, seed=31, pml=4, n_boxes=1, n_sources=1, n_probes=8, name="overflow")
    rng = np.random.default_rng(8)
    mats = [S.Material()]
    for q in range(200):
        magnetic = q % 25 == 0
        mats.append(S.Material(eps_r=float(rng.uniform(1, 12)), sigma_e=float(rng.uniform(0, 0.05)),
                               mu_r=1.5 if magnetic else 1.0, sigma_m=1e3 if magnetic else float(S.REF_TINY)))
    idx = rng.integers(1, len(mats), size=(sc.nz, sc.ny, sc.nx)).astype(np.uint8)
    s = sc.sources[0].box
    sc = dataclasses.replace(sc, materials=mats, bricks=[],
                             resistors=[S.Resistor((s[0] + 2, s[1], s[2], s[0] + 2, s[1], s[5]), 75.0)])
    return sc, idx


def _distinct_interface_keys(idx):
    """Distinct seven-cell combinations (cells (i,j,k) (i-1,j,k) (i,j-1,k) (i,j,k-1) (i-1,j-1,k)
    (i-1,j,k-1) (i,j-1,k-1)) over nodes 1..n-1 per axis whose seven cells are not all one material."""
    c = idx.astype(np.uint64)
    m0 = c[1:, 1:, 1:]
    cells = [m0, c[1:, 1:, :-1], c[1:, :-1, 1:], c[:-1, 1:, 1:], c[1:, :-1, :-1], c[:-1, 1:, :-1], c[:-1, :-1, 1:]]
    key = np.zeros_like(m0)
    for q, a in enumerate(cells):
        key |= a << np.uint64(8 * q)
    mixed = np.zeros(m0.shape, bool)
    for a in cells[1:]:
        mixed |= a != m0
    return np.unique(key[mixed]).size


@pytest.mark.parametrize("schedule", [1, 2])
def test_interface_row_overflow_vs_oracle(gpu_lib, schedule):
    """More distinct interface combinations than the table has rows: the nodes beyond it take the
    general path (inside the sweep under the fused schedule). Bit-exact against the oracle with the
    GPU's CPML profiles."""
    sc, idx = _overflow_scenario()
    assert _distinct_interface_keys(idx) > MAX_INTERFACE_ROWS
    from fdtd_gb300 import solver
    with solver.Simulation.from_scenario(sc, schedule, material_index=idx, probe_capacity=sc.steps) as sim:
        sim.step(sc.steps)
        sim.synchronize()
        p, f, prof = sim.read_probes(0, sc.steps), sim.fields(), sim.cpml_profiles()
    sc_o = dataclasses.replace(sc)
    sc_o.material_index = lambda: idx  # the oracle paints from the scenario's index
    po, fo = oracle.run(sc_o, profile_override=prof)
    assert bitwise_equal(p, po), rel_l2(p, po)
    for c, n in enumerate(FIELDS):
        assert bitwise_equal(f[c], fo[c]), (n, rel_l2(f[c], fo[c]))
