"""The oracle's discrete adjoint (the checker of the GPU adjoint) against central finite differences.

Figure of merit J = sum_m dt * Ez(probe)^2; gradient with respect to eps_r of the cells of a design
region, through CPML and a resistive lumped port. In FP64 the adjoint is exact up to the FD
truncation error, so the agreement is far tighter than the 1e-3 bar the GPU adjoint is held to.
"""
import numpy as np
import pytest

import oracle
from fdtd_gb300 import scenario as S


def small_design_case(seed=0):
    sc = S.vacuum_cube(24, 160, pml=4, name="adjoint_small")
    sc.nx, sc.ny, sc.nz = 24, 22, 20
    sc.sources = [S.LumpedSource((7, 11, 9, 7, 11, 10), 50.0, S.gaussian_derivative(160, sc.dt, 30e9, 1e-3))]
    sc.probes = []
    sc.materials.append(S.Material(eps_r=3.0, sigma_e=0.02))
    sc.bricks.append(S.Brick((12, 5, 5, 20, 9, 8), 1))  # a lossy dielectric touching the design region
    box = (10, 8, 7, 16, 14, 11)
    rng = np.random.default_rng(seed)
    eps = rng.uniform(1, 12, size=(box[5] - box[2], box[4] - box[1], box[3] - box[0]))
    probe = (18, 11, 9)
    return sc, box, eps, probe


def central_fd(sc, probe, box, eps, v, h=1e-3):
    e1 = eps.copy(); e1[v] += h
    e2 = eps.copy(); e2[v] -= h
    return (oracle.fom_grad(sc, probe, box, e1, grad=False) - oracle.fom_grad(sc, probe, box, e2, grad=False)) / (2 * h)


def test_fp64_adjoint_matches_central_differences():
    sc, box, eps, probe = small_design_case()
    J, g = oracle.fom_grad(sc, probe, box, eps)
    assert J > 0 and np.all(np.isfinite(g))
    rng = np.random.default_rng(1)
    for _ in range(6):
        v = tuple(int(rng.integers(0, s)) for s in eps.shape)
        fd = central_fd(sc, probe, box, eps, v)
        assert abs(g[v] - fd) <= 1e-6 * abs(fd) + 1e-30, (v, g[v], fd)


def test_fp32_adjoint_close_to_fp64():
    sc, box, eps, probe = small_design_case(3)
    _, g64 = oracle.fom_grad(sc, probe, box, eps, precision="f64")
    _, g32 = oracle.fom_grad(sc, probe, box, eps, precision="f32")
    assert np.linalg.norm(g32 - g64) / np.linalg.norm(g64) < 1e-4


def test_box_history_form_equals_full_history():
    """The long-run form (only the design region's field history kept) gives the same J and
    gradient bits as the full-history form."""
    d = S.design_problem(24, 60, (6, 6, 4), pml=4, seed=2)
    e = d.eps.astype(np.float64)
    J1, g1 = oracle.fom_grad(d.scenario, d.probe, d.box, e)
    J2, g2 = oracle.fom_grad(d.scenario, d.probe, d.box, e, box_history=True)
    assert J1 == J2 and np.array_equal(g1, g2)
