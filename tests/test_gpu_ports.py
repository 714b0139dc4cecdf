"""GPU port voltage / current and port spectra through the C ABI.

- V(t), I(t) before the time average and I(t) after it equal the reference's voltMgpu / currMgpu /
  correcI on its own samples bit for bit, under both schedules, and the oracle's restatement;
- fdtd_port_spectrum's spectra agree with an FP64 FFT of the same V(t), I(t) (relative L2 1e-5),
  and its s11 / zin with the FP64 formulas on the bins that carry the signal;
- fdtd_port_zin equals the reference's c_zinS11 on the fixture's spectra bit for bit, and on the
  solver's own spectra when the reference-kernel harness is present.
"""
import os

import numpy as np
import pytest

import golden_scenarios as gs
import oracle
from conftest import GOLDEN, bitwise_equal, golden

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "port.npz")),
                                 reason="port fixture not generated")]

FDTD_ERR_INVALID, FDTD_ERR_STATE = 1, 4
SPEC_TOL = 1e-5  # relative L2 of the FP32 spectra against an FP64 FFT of the same samples


def crel(a, b) -> float:
    """Relative L2 error of complex arrays."""
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run_port(schedule=0, steps=None):
    from fdtd_gb300 import solver
    sc = gs.port_scenario()
    steps = sc.steps if steps is None else steps
    with solver.Simulation.from_scenario(sc, schedule, probe_capacity=steps) as sim:
        pid = sim.add_port(gs.PORT_BOX, gs.PORT_BOX)
        sim.step(steps)
        sim.synchronize()
        V, Iraw = sim.read_port(pid, time_average=False)
        V2, Iavg = sim.read_port(pid)
        series = sim.read_probes(0, steps)
        spec = sim.port_spectrum(pid, 50.0)
    assert bitwise_equal(V, V2)
    return sc, V, Iraw, Iavg, series, spec


@pytest.mark.parametrize("schedule", [1, 2])
def test_port_vi_bitwise_vs_reference(gpu_lib, schedule):
    sc, V, Iraw, Iavg, series, _ = run_port(schedule)
    fix = golden("port")
    assert bitwise_equal(series[:, :len(sc.probes)], fix["probes"])
    assert bitwise_equal(V, fix["voltage"])
    assert bitwise_equal(Iraw, fix["current_raw"])
    assert bitwise_equal(Iavg, fix["current_avg"])
    Vo, Io = oracle.port_vi(series, gs.PORT_BOX, gs.PORT_BOX, sc, col0=len(sc.probes))
    assert bitwise_equal(Vo, V) and bitwise_equal(Io, Iavg)


@pytest.mark.parametrize("schedule", [1, 2])
def test_current_loops_bitwise_vs_reference(gpu_lib, schedule):
    """x, y and z current loops (currMgpu cases 1, 2, 3) on one run."""
    from fdtd_gb300 import solver
    sc = gs.port_scenario()
    fix = golden("port")
    with solver.Simulation.from_scenario(sc, schedule, probe_capacity=sc.steps) as sim:
        ids = [sim.add_port(gs.PORT_BOX, gs.PORT_CURRENT_BOX, current_axis=a) for a in (0, 1, 2)]
        sim.step(sc.steps)
        sim.synchronize()
        for a, pid in enumerate(ids):
            V, Iraw = sim.read_port(pid, time_average=False)
            _, Iavg = sim.read_port(pid)
            assert bitwise_equal(V, fix["voltage"])
            assert bitwise_equal(Iraw, fix[f"current_raw_d{a + 1}"]), a
            assert bitwise_equal(Iavg, fix[f"current_avg_d{a + 1}"]), a


@pytest.mark.parametrize("schedule", [1, 2])
def test_voltage_directions_bitwise_vs_reference(gpu_lib, schedule):
    """x, y and z port voltages (voltMgpu directions 1, 2, 3) on one run, against the reference's
    own reduction of its samples and against the oracle."""
    import os
    from conftest import GOLDEN
    from fdtd_gb300 import solver
    if not os.path.exists(os.path.join(GOLDEN, "port_xy.npz")):
        pytest.skip("port_xy fixture not generated")
    sc = gs.port_scenario()
    fix = golden("port_xy")
    with solver.Simulation.from_scenario(sc, schedule, probe_capacity=sc.steps) as sim:
        ids = [sim.add_port(gs.PORT_BOX, gs.PORT_BOX, voltage_axis=a) for a in (0, 1, 2)]
        sim.step(sc.steps)
        sim.synchronize()
        series = sim.read_probes(0, sc.steps)
        col = len(sc.probes)
        for a, pid in enumerate(ids):
            V, _ = sim.read_port(pid)
            assert bitwise_equal(V, fix[f"voltage_d{a + 1}"]), a
            Vo, _ = oracle.port_vi(series, gs.PORT_BOX, gs.PORT_BOX, sc, col0=col, voltage_axis=a)
            assert bitwise_equal(Vo, V), a
            col += len(oracle.port_probes(gs.PORT_BOX, gs.PORT_BOX, voltage_axis=a))


def test_port_columns_in_probe_series(gpu_lib):
    from fdtd_gb300 import solver
    sc = gs.port_scenario()
    with solver.Simulation.from_scenario(sc, probe_capacity=8) as sim:
        sim.add_port(gs.PORT_BOX, gs.PORT_BOX)
        assert sim.n_probes == len(sc.probes) + len(oracle.port_probes(gs.PORT_BOX, gs.PORT_BOX))


def test_port_spectrum(gpu_lib):
    sc, V, _, Iavg, _, spec = run_port()
    ref = oracle.port_spectra(V, Iavg, 50.0)
    assert crel(spec["v"], ref["v"]) < SPEC_TOL
    assert crel(spec["i"], ref["i"]) < SPEC_TOL
    assert spec["v"].size == sc.steps // 2 + 1
    assert np.isclose(spec["freq"][1], 1.0 / (sc.steps * np.float32(sc.dt)))
    # s11 / zin where the voltage spectrum carries the signal
    band = np.abs(ref["v"]) > 1e-2 * np.abs(ref["v"]).max()
    assert band.sum() > 20
    for k in ("s11", "zin"):
        err = np.abs(spec[k][band] - ref[k][band]) / np.abs(ref[k][band])
        assert err.max() < 1e-3, (k, err.max())


def test_port_zin_bitwise_vs_reference(gpu_lib):
    from fdtd_gb300 import solver
    fix = golden("port")
    for q, z0 in enumerate(fix["z0"]):
        s11, zin = solver.port_zin(fix["spec_v"], fix["spec_i"], complex(z0))
        assert bitwise_equal(s11.view(np.float32), fix["s11"][q].view(np.float32))
        assert bitwise_equal(zin.view(np.float32), fix["zin"][q].view(np.float32))


def test_port_spectrum_zin_vs_reference_kernel_live(gpu_lib):
    import refharness
    if not refharness.available():
        pytest.skip("reference-kernel harness not built")
    sc, _, _, _, _, spec = run_port()
    h = refharness.RefHarness()
    try:
        h.setup(sc)
        s11, zin = h.zin(sc.steps, spec["v"], spec["i"], 50.0)
    finally:
        h.close()
    assert bitwise_equal(s11.view(np.float32), spec["s11"].view(np.float32))
    assert bitwise_equal(zin.view(np.float32), spec["zin"].view(np.float32))


def test_port_validation(gpu_lib):
    from fdtd_gb300 import solver
    sc = gs.port_scenario()
    with solver.Simulation.from_scenario(sc, probe_capacity=16) as sim:
        for vbox, cbox in [((14, 13, 9, 15, 14, 9), gs.PORT_BOX),     # empty k range
                           (gs.PORT_BOX, (0, 13, 9, 15, 14, 12)),     # no node below the loop in x
                           ((14, 13, 9, 15, 40, 12), gs.PORT_BOX)]:   # outside the grid
            with pytest.raises(solver.FDTDError) as e:
                sim.add_port(vbox, cbox)
            assert e.value.code == FDTD_ERR_INVALID
        for vbox, axis in [(gs.PORT_BOX, 3), ((14, 13, 9, 14, 14, 12), 0), ((14, 13, 9, 15, 13, 12), 1)]:
            with pytest.raises(solver.FDTDError) as e:  # unknown axis; empty x range; empty y range
                sim.add_port(vbox, gs.PORT_BOX, voltage_axis=axis)
            assert e.value.code == FDTD_ERR_INVALID
        pid = sim.add_port(gs.PORT_BOX, gs.PORT_BOX)
        sim.step(4)
        with pytest.raises(solver.FDTDError) as e:
            sim.add_port(gs.PORT_BOX, gs.PORT_BOX)
        assert e.value.code == FDTD_ERR_STATE
        with pytest.raises(solver.FDTDError):
            sim.read_port(pid + 1)
        with pytest.raises(solver.FDTDError):
            sim.port_spectrum(pid, z0=-50.0)
