"""Scenarios behind the golden fixtures in this directory (shared by make_golden.py and the tests).

Every scenario is rebuilt deterministically from these definitions, so a fixture only stores the
reference's outputs. Sizes are small enough for the CPU oracle to finish in seconds, except the
64^3 vacuum case, whose fixture keeps probe series, field norms and a mid-plane slice only.
"""
from __future__ import annotations

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from fdtd_gb300 import scenario as S  # noqa: E402

ONESTEP_M = 7


def onestep_signal():
    """Per-edge source signal for the single-step fixture: large enough (|Cezj*s| ~ O(1)) that the
    rounding of the lumped-source term shows in the result."""
    import numpy as np
    return (np.random.default_rng(1234).standard_normal(ONESTEP_M + 1) * 1e-3).astype(np.float32)


def vacuum64():
    """64^3 vacuum workload with extra probes of every component (all outside the CPML)."""
    sc = S.vacuum_cube(64, 1000, name="vacuum64")
    sc.probes += [S.Probe(S.EZ, 32, 32, 40), S.Probe(S.HX, 32, 40, 32), S.Probe(S.HY, 40, 32, 32),
                  S.Probe(S.EX, 36, 36, 36), S.Probe(S.EY, 30, 34, 32), S.Probe(S.HZ, 28, 28, 33)]
    return sc


def small_vacuum():
    """32x28x24 vacuum, asymmetric CPML, one centred source, 80 steps (pulse still inside)."""
    sc = S.vacuum_cube(32, 80, pml=5, name="small_vacuum")
    sc.nx, sc.ny, sc.nz = 32, 28, 24
    sc.pml = (6, 5, 4, 6, 5, 4)
    wf = sc.sources[0].waveform
    sc.sources = [S.LumpedSource((15, 13, 11, 15, 13, 12), 50.0, wf)]
    sc.probes = [S.Probe(S.EZ, 20, 13, 11), S.Probe(S.HX, 15, 16, 12), S.Probe(S.HY, 12, 13, 14),
                 S.Probe(S.EX, 17, 15, 13), S.Probe(S.EY, 14, 11, 10), S.Probe(S.HZ, 16, 12, 9)]
    return sc


def boxes_scenario():
    """32x30x26 random dielectric boxes plus one magnetic box, one source, one resistor, 400 steps."""
    sc = S.scaled_boxes(32, 30, 26, 400, seed=11, pml=5, n_boxes=10, n_sources=1, n_probes=8,
                        name="small_boxes")
    sc.pml = (5, 6, 4, 5, 6, 4)
    sc.materials.append(S.Material(eps_r=3.0, sigma_e=0.01, mu_r=2.0, sigma_m=2e4))
    sc.bricks.append(S.Brick((9, 8, 9, 17, 14, 15), len(sc.materials) - 1))
    s = sc.sources[0].box
    sc.resistors = [S.Resistor((s[0] + 3, s[1] - 2, s[2], s[0] + 3, s[1] - 2, s[5] + 1), 75.0)]
    return sc


def two_sources():
    """32x28x24 vacuum with two delayed sources (reference runs once per source and sums), 90 steps."""
    sc = small_vacuum()
    sc.name = "two_sources"
    sc.steps = 90
    sc.sources[0].waveform = S.gaussian_derivative(sc.steps, sc.dt, 30e9, 1e-3)
    dt = sc.dt
    wf2 = S.gaussian_derivative(sc.steps, dt, 30e9, 1e-3, delay_steps=17.0, amp=0.5)
    sc.sources.append(S.LumpedSource((10, 16, 12, 10, 16, 14), 50.0, wf2))
    return sc


def aniso_scenario():
    """32x30x26 grid with per-axis (anisotropic) bricks as setBrick takes them (separate x / y / z
    eps_r, sigma_e, mu_r and sigma_m), overlapping so that edges average different axes' values,
    one reaching into the CPML; one source, one resistor, 300 steps."""
    sc = S.scaled_boxes(32, 30, 26, 300, seed=13, pml=5, n_boxes=0, n_sources=1, n_probes=8, name="aniso")
    sc.pml = (5, 6, 4, 5, 6, 4)
    sc.materials += [
        S.Material(eps_r=(2.0, 5.0, 9.0), sigma_e=(0.01, 0.0, 0.03)),
        S.Material(eps_r=(4.0, 4.0, 1.5), sigma_e=0.02, mu_r=(1.0, 2.5, 1.5), sigma_m=(1e3, 4e3, 2e4)),
        S.Material(eps_r=(7.0, 3.0, 3.0), sigma_e=(0.0, 0.05, 0.0)),
    ]
    sc.bricks = [S.Brick((7, 6, 6, 20, 18, 14), 1), S.Brick((14, 12, 9, 26, 24, 19), 2),
                 S.Brick((0, 3, 3, 11, 12, 10), 3)]
    s = sc.sources[0].box
    sc.resistors = [S.Resistor((s[0] + 2, s[1] + 1, s[2], s[0] + 2, s[1] + 1, s[5]), 60.0)]
    return sc


def onestep_scenario():
    """24x20x18 random boxes with a magnetic box, 4-cell CPML, one source: single-step checks."""
    sc = S.scaled_boxes(24, 20, 18, 16, seed=5, pml=4, n_boxes=6, n_sources=1, n_probes=2,
                        name="onestep")
    sc.pml = (4, 3, 4, 3, 4, 3)
    sc.materials.append(S.Material(eps_r=2.0, sigma_e=0.02, mu_r=3.0, sigma_m=5e3))
    sc.bricks.append(S.Brick((6, 5, 5, 12, 11, 10), len(sc.materials) - 1))
    return sc


def port_scenario():
    """30x28x24 grid with a dielectric slab under a 2x2-edge lumped port (source, voltage and
    current boxes on the same edges), 700 steps: more than one 512-thread block of the
    reference's time-series kernels."""
    steps = 700
    sc = S.vacuum_cube(30, steps, pml=5, name="port")
    sc.nx, sc.ny, sc.nz = 30, 28, 24
    sc.pml = (5, 6, 5, 6, 5, 4)
    sc.materials.append(S.Material(eps_r=4.4, sigma_e=0.005))
    sc.bricks.append(S.Brick((8, 7, 6, 22, 21, 9), len(sc.materials) - 1))
    sc.sources = [S.LumpedSource(PORT_BOX, 50.0, S.gaussian_derivative(steps, sc.dt, 20e9, 1e-3))]
    sc.probes = [S.Probe(S.EZ, 20, 14, 10), S.Probe(S.HY, 13, 14, 11)]
    return sc


def plates_scenario():
    """40x36x26 microstrip-like case: a substrate slab on a ground plate (reaching into the CPML),
    a strip plate with a second plate overlapping it (the later one wins), an x- and a y-normal
    plate, a lumped source and a resistor between ground and strip, 300 steps."""
    steps = 300
    sc = S.vacuum_cube(40, steps, pml=5, name="plates")
    sc.nx, sc.ny, sc.nz = 40, 36, 26
    sc.pml = (5, 6, 5, 6, 4, 5)
    sc.materials.append(S.Material(eps_r=4.4, sigma_e=0.002))
    sc.bricks.append(S.Brick((5, 6, 5, 35, 30, 9), len(sc.materials) - 1))
    sc.plates = [S.Plate(2, (3, 3, 5, 37, 33, 5), 1e10, 1e10),
                 S.Plate(2, (10, 14, 9, 30, 18, 9), 5.8e7, 5.8e7),
                 S.Plate(2, (25, 15, 9, 33, 20, 9), 5e6, 3e6),
                 S.Plate(0, (8, 10, 6, 8, 20, 12), 1e7, 2e7),
                 S.Plate(1, (12, 25, 7, 24, 25, 13), 3e5, 4e5)]
    sc.sources = [S.LumpedSource((12, 16, 5, 12, 16, 9), 50.0, S.gaussian_derivative(steps, sc.dt, 20e9, 1e-3))]
    sc.resistors = [S.Resistor((28, 16, 5, 28, 16, 9), 50.0)]
    sc.probes = [S.Probe(S.EZ, 20, 16, 7), S.Probe(S.EX, 18, 16, 10), S.Probe(S.EY, 20, 19, 9),
                 S.Probe(S.HX, 20, 17, 8), S.Probe(S.HY, 15, 16, 9), S.Probe(S.EZ, 8, 12, 8),
                 S.Probe(S.EX, 2, 10, 5), S.Probe(S.EZ, 16, 25, 9)]
    return sc


def marching_params(n_t_steps=500, current_direction=2, numdev=1, source_tp=1, resistor_opt=0, aniso=False):
    """marchingLoop's parameters for a reduced version of the reference driver's microstrip case
    (substrate brick on a ground plate, a feed strip and a wider patch plate, a Gaussian source at
    the feed, voltage and current sampled on the feed line): its cell sizes and constants,
    a 40 x 60 x 6-cell structure, 6-cell CPML, 4-cell air buffers. aniso: the substrate takes
    different eps_r, sigma_e, mu_r and sigma_m per axis."""
    import numpy as np
    f = np.float32
    eps_0 = f(8.854187817e-12)
    pi = f(3.1415)
    mu_0 = f(np.float64(f(4) * pi) * 1e-7)
    c = f(1) / np.sqrt(mu_0 * eps_0)
    dx, dy, dz = f(0.389e-3), f(0.4e-3), f(0.265e-3)
    dt = f(1 / (np.float64(c) * np.sqrt(1 / np.float64(dx) ** 2 + 1 / np.float64(dy) ** 2 + 1 / np.float64(dz) ** 2)))
    nc = f(20)
    tau = (nc * dy) / (f(2) * c)
    a = dict(NUMDEV=numdev, eps_0=eps_0, pi=pi, mu_0=mu_0, c=c, dx=dx, dy=dy, dz=dz, dt=dt, X=40, Y=60, Z=6,
             n_t_steps=n_t_steps, pml_x_n=6, pml_y_n=6, pml_z_n=6, pml_x_p=6, pml_y_p=6, pml_z_p=6,
             air_buff_x_n=4, air_buff_y_n=4, air_buff_z_n=4, air_buff_x_p=4, air_buff_y_p=4, air_buff_z_p=4,
             source_tp=source_tp, source_freq=f(2e9), source_amp=f(1),
             source_min_x=f(16) * dx, source_min_y=f(0), source_min_z=f(0),
             source_max_x=f(22) * dx, source_max_y=f(0), source_max_z=f(3) * dz,
             source_direction=3, rs=f(50), nc=nc, tau=tau, t_0=f(3) * tau)
    a.update(brick_min_x=[0.0], brick_min_y=[0.0], brick_min_z=[0.0], brick_max_x=[f(40) * dx],
             brick_max_y=[f(60) * dy], brick_max_z=[f(3) * dz], brick_sigma_e_x=[4e-4], brick_sigma_e_y=[4e-4],
             brick_sigma_e_z=[4e-4], brick_eps_r_x=[2.2], brick_eps_r_y=[2.2], brick_eps_r_z=[2.2],
             brick_sigma_m_x=[1.2e-38], brick_sigma_m_y=[1.2e-38], brick_sigma_m_z=[1.2e-38], brick_mu_r_x=[1.0],
             brick_mu_r_y=[1.0], brick_mu_r_z=[1.0], brick_opt=1, brick_num=1)
    a.update(pec_min_x=[0.0, f(16) * dx, f(10) * dx], pec_min_y=[0.0, 0.0, f(30) * dy],
             pec_min_z=[0.0, f(3) * dz, f(3) * dz], pec_max_x=[f(40) * dx, f(22) * dx, f(30) * dx],
             pec_max_y=[f(60) * dy, f(30) * dy, f(50) * dy], pec_max_z=[0.0, f(3) * dz, f(3) * dz],
             pec_sigma_e_x=[1e10] * 3, pec_sigma_e_y=[1e10] * 3, pec_sigma_e_z=[1e10] * 3, pec_opt=1, pec_num=3)
    a.update(resistor_min_x=f(30) * dx, resistor_min_y=f(50) * dy, resistor_min_z=f(0), resistor_max_x=f(30) * dx,
             resistor_max_y=f(50) * dy, resistor_max_z=f(3) * dz, resistor_resist=f(50), resistor_direction=3,
             resistor_opt=resistor_opt)
    a.update(sampled_voltage_min_x=f(16) * dx, sampled_voltage_min_y=f(10) * dy, sampled_voltage_min_z=f(0),
             sampled_voltage_max_x=f(22) * dx, sampled_voltage_max_y=f(10) * dy, sampled_voltage_max_z=f(3) * dz,
             voltage_direction=3)
    a.update(sampled_current_min_x=f(16) * dx, sampled_current_min_y=f(10) * dy, sampled_current_min_z=f(3) * dz,
             sampled_current_max_x=f(22) * dx, sampled_current_max_y=f(10) * dy, sampled_current_max_z=f(3) * dz,
             current_direction=current_direction)
    if current_direction == 3:  # a z loop needs ks < ke: around the feed's vertical edges
        a.update(sampled_current_min_z=f(0), sampled_current_max_z=f(3) * dz)
    if aniso:
        a.update(brick_eps_r_x=[2.2], brick_eps_r_y=[3.4], brick_eps_r_z=[6.1], brick_sigma_e_x=[4e-4],
                 brick_sigma_e_y=[1e-3], brick_sigma_e_z=[0.0], brick_mu_r_x=[1.0], brick_mu_r_y=[1.7],
                 brick_mu_r_z=[1.2], brick_sigma_m_x=[1.2e-38], brick_sigma_m_y=[5e2], brick_sigma_m_z=[1e3])
    return a


# voltage box: i, j closed, k half-open (voltMgpu case 3); current box: loop at plane ke - 1
PORT_BOX = (14, 13, 9, 15, 14, 12)
# a current box whose x, y and z loops (currMgpu cases 1, 2, 3) all lie inside the grid
PORT_CURRENT_BOX = (13, 12, 8, 16, 15, 11)


def fixture_scenarios():
    """(scenario, keep full fields?) for every run fixture."""
    return [(vacuum64(), False), (small_vacuum(), True), (boxes_scenario(), True), (two_sources(), True),
            (plates_scenario(), True), (aniso_scenario(), True)]
