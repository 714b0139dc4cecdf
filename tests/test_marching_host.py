"""Host-side restatement of marchingLoop's set-up (no GPU): grid size, NZ rounding for NUMDEV,
metre-to-index conversion and the scenario built from it."""
import numpy as np

import golden_scenarios as gs
from fdtd_gb300 import scenario as S


def test_indices_of_the_reduced_microstrip():
    a = gs.marching_params()
    ix = S.marching_indices(a)
    # 40 x 60 x 6 cells + 2 x (4 air + 6 CPML) per axis
    assert (ix["nx"], ix["ny"], ix["nz"]) == (60, 80, 26)
    o = 10
    assert ix["source"] == (o + 16, o, o, o + 22, o, o + 3)
    assert ix["voltage"] == (o + 16, o + 10, o, o + 22, o + 10, o + 3)
    assert ix["current"] == (o + 16, o + 10, o + 3, o + 22, o + 10, o + 3)
    assert ix["pecs"][0] == (o, o, o, o + 40, o + 60, o)
    assert ix["bricks"] == [(o, o, o, o + 40, o + 60, o + 3)]
    assert ix["resistor"] is None


def test_numdev_rounds_nz_up():
    for numdev, nz in ((1, 26), (2, 26), (3, 27), (4, 28), (8, 32)):
        assert S.marching_indices(gs.marching_params(numdev=numdev))["nz"] == nz


def test_calc_index_rounds_half_away_from_zero_in_float():
    d = np.float32(0.4e-3)
    assert S.calc_index(np.float32(10) * d, d) == 10
    assert S.calc_index(np.float32(2.5) * d, d) == 3
    assert S.calc_index(-np.float32(2.5) * d, d) == -3
    # 7.535e-3 / 0.389e-3 = 19.37 -> 19 (the reference driver's feed position)
    assert S.calc_index(7.535e-3, np.float32(0.389e-3)) == 19


def test_marching_scenario_structure():
    a = gs.marching_params(resistor_opt=1)
    wave = np.linspace(0, 1, a["n_t_steps"], dtype=np.float32)
    sc, vbox, cbox = S.marching_scenario(a, wave)
    assert len(sc.plates) == 3 and all(p.axis == 2 for p in sc.plates)
    assert sc.plates[0].sigma_1 == 1e10
    assert len(sc.materials) == 2 and np.allclose(sc.materials[1].axes()[:, 0], 2.2)
    assert len(sc.resistors) == 1 and sc.sources[0].resistance == 50.0
    assert sc.pml == (6, 6, 6, 6, 6, 6)
    assert vbox[2] < vbox[5]


def test_sector_plates_cover_the_sector_edges():
    """sector_plates decomposes the sector's Ex and Ey edges into plates that cover exactly them."""
    from fdtd_gb300 import scenario as S
    nx, ny, dx, dy = 40, 34, 1e-3, 1e-3
    tri, pz0, r, mx, my = (6, 26, 18, 12, 30, 26), 9, 0.0105, 34, 30
    ex, ey = S.sector_edges(tri, pz0, r, mx, my, dx, dy, nx, ny)
    cx, cy = np.zeros(ex.shape, np.int32), np.zeros(ey.shape, np.int32)
    for p in S.sector_plates(tri, pz0, r, mx, my, 1.0, 2.0, dx, dy, nx, ny):
        b = p.box
        assert b[2] == b[5] == pz0
        if p.axis == 2:  # Ex-only row run
            assert b[1] == b[4]
            cx[b[1], b[0]:b[3]] += 1
        else:            # Ey-only column run
            assert p.axis == 0 and b[0] == b[3]
            cy[b[1]:b[4], b[0]] += 1
    assert np.array_equal(cx, ex.astype(cx.dtype)) and np.array_equal(cy, ey.astype(cy.dtype))
    # the apex lies in the sector, a point beyond the radius does not
    assert ex[12, 18] and not ex[12, 33]


def test_material_tables_for_isotropic_and_per_axis_materials():
    """The scenario's material tables (the isotropic shortcut and the per-axis path) equal the
    values written out per axis in float32, for scalars, numpy scalars and per-axis sequences."""
    mats = [S.Material(), S.Material(eps_r=2.5, sigma_e=0.01), S.Material(eps_r=np.float64(3.3), mu_r=np.float32(1.7)),
            S.Material(eps_r=(2.0, 3.0, 4.0), sigma_e=0.02), S.Material(eps_r=[5.0, 5.0, 5.0], sigma_m=(1e3, 2e3, 3e3))]
    sc = S.Scenario("m", 8, 8, 8, 1e-3, 1e-3, 1e-3, 1e-12, (2,) * 6, 1, mats)

    def axes(m):
        out = np.zeros((3, 4), dtype=np.float32)
        for q, v in enumerate((m.eps_r, m.sigma_e, m.mu_r, m.sigma_m)):
            out[:, q] = np.broadcast_to(np.asarray(v, dtype=np.float32), (3,))
        return out

    want = np.stack([axes(m) for m in mats])
    assert np.array_equal(sc.material_table_axes().view(np.uint32), want.view(np.uint32))
    assert np.array_equal(sc.material_table().view(np.uint32), want[:, 0, :].view(np.uint32))
    assert [m.anisotropic for m in mats] == [False, False, False, True, True]
    assert sc.anisotropic
