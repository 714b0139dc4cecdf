"""Port voltage / current and port spectra of the oracle against the reference's own kernels.

The fixture ``port.npz`` holds what the reference computed on a GPU: its own sampling of the port
edges inside calc_e / calc_h, voltMgpu / currMgpu (V(t) and I(t) before correcI), correcI's output,
and c_zinS11 on seeded spectra for two reference impedances (tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest

import golden_scenarios as gs
import oracle
from conftest import GOLDEN, bitwise_equal, golden

pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "port.npz")),
                                reason="port fixture not generated")

PROFILE_KEYS = {"b_ex": "cpml_b_ex", "a_ex": "cpml_a_ex", "b_mx": "cpml_b_mx", "a_mx": "cpml_a_mx",
                "b_ey": "cpml_b_ey", "a_ey": "cpml_a_ey", "b_my": "cpml_b_my", "a_my": "cpml_a_my",
                "b_ez": "cpml_b_ez", "a_ez": "cpml_a_ez", "b_mz": "cpml_b_mz", "a_mz": "cpml_a_mz"}


def warp_edge(n: int) -> np.ndarray:
    """Steps whose correcI result depends on thread scheduling in the reference: it averages in
    place, one thread per step, and step t reads I(t+1), which lies in the next 32-thread warp
    when t % 32 == 31."""
    return (np.arange(n) % 32) == 31


def reference_average(raw: np.ndarray) -> np.ndarray:
    """correcI in the order the reference produced it: every step from its unaveraged successor,
    the last step from its averaged predecessor (the two branches diverge in one warp)."""
    r = raw.astype(np.float32)
    out = np.empty_like(r)
    out[:-1] = (r[:-1] + r[1:]) / np.float32(2)
    out[-1] = (r[-1] + out[-2]) / np.float32(2)
    return out


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "port_xy.npz")), reason="port_xy fixture not generated")
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_voltage_directions_bitwise(axis):
    """voltMgpu's x, y and z directions: the same Ez samples summed over the ranges each direction
    takes, times its scale."""
    sc = gs.port_scenario()
    fix = golden("port")
    prof = {k: fix[v] for k, v in PROFILE_KEYS.items()}
    probes = list(sc.probes) + oracle.port_probes(gs.PORT_BOX, gs.PORT_BOX, voltage_axis=axis)
    series, _ = oracle.run(sc, profile_override=prof, probes=probes)
    V, _ = oracle.port_vi(series, gs.PORT_BOX, gs.PORT_BOX, sc, col0=len(sc.probes), voltage_axis=axis)
    assert bitwise_equal(V, golden("port_xy")[f"voltage_d{axis + 1}"])


def oracle_port(time_average=True):
    sc = gs.port_scenario()
    fix = golden("port")
    prof = {k: fix[v] for k, v in PROFILE_KEYS.items()}
    probes = list(sc.probes) + oracle.port_probes(gs.PORT_BOX, gs.PORT_BOX)
    series, _ = oracle.run(sc, profile_override=prof, probes=probes)
    V, I = oracle.port_vi(series, gs.PORT_BOX, gs.PORT_BOX, sc, col0=len(sc.probes), time_average=time_average)
    return sc, fix, series, V, I


def test_port_probe_layout():
    p = oracle.port_probes(gs.PORT_BOX, gs.PORT_BOX)
    is_, js, ks, ie, je, ke = gs.PORT_BOX
    nv = (ie - is_ + 1) * (je - js + 1) * (ke - ks)
    assert len(p) == nv + 2 * (ie - is_ + 1) + 2 * (je - js + 1)
    assert (p[0].i, p[0].j, p[0].k) == (is_, js, ks) and (p[1].i, p[1].j, p[1].k) == (is_ + 1, js, ks)
    # z loop: Hy(ie, j) first, Hx(i, je) last, at plane ke - 1
    assert (p[nv].component, p[nv].i, p[nv].j, p[nv].k) == (4, ie, js, ke - 1)
    assert (p[-1].component, p[-1].i, p[-1].j, p[-1].k) == (3, ie, je, ke - 1)
    # y loop (source.cu's current direction): Hz(is-1, je-1, k) first, Hx(i, je-1, ks-1) last
    q = oracle.port_probes(gs.PORT_BOX, (14, 13, 9, 15, 13, 11), current_axis=1)
    assert (q[nv].component, q[nv].i, q[nv].j, q[nv].k) == (5, 13, 12, 9)
    assert (q[-1].component, q[-1].i, q[-1].j, q[-1].k) == (3, 15, 12, 8)
    assert len(q) == nv + 2 * 3 + 2 * 2


def test_oracle_port_vi_equals_reference():
    sc, fix, series, V, I = oracle_port(time_average=False)
    assert bitwise_equal(series[:, :len(sc.probes)], fix["probes"])
    assert bitwise_equal(V, fix["voltage"])
    assert bitwise_equal(I, fix["current_raw"])
    assert np.abs(V).max() > 0 and np.abs(I).max() > 0


def test_oracle_time_average_equals_correcI():
    _, fix, _, _, I = oracle_port(time_average=True)
    assert bitwise_equal(I, reference_average(fix["current_raw"]))
    # the fixture's own correcI output, including the steps where it raced
    assert bitwise_equal(I, fix["current_avg"])
    # at the racy steps the other order would have given a different value, so the check bites
    raw = fix["current_raw"].astype(np.float32)
    t = np.flatnonzero(warp_edge(raw.size))
    t = t[t + 1 < raw.size]
    alt = (raw[t] + (raw[t + 1] + raw[np.minimum(t + 2, raw.size - 1)]) / np.float32(2)) / np.float32(2)
    assert np.any(alt != fix["current_avg"][t])


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_oracle_current_loops_equal_reference(axis):
    """currMgpu's x, y and z loops (cases 1, 2, 3) on the reference's own samples."""
    sc = gs.port_scenario()
    fix = golden("port")
    key = f"current_raw_d{axis + 1}"
    if key not in fix.files:
        pytest.skip("fixture predates the three loop directions")
    prof = {k: fix[v] for k, v in PROFILE_KEYS.items()}
    probes = list(sc.probes) + oracle.port_probes(gs.PORT_BOX, gs.PORT_CURRENT_BOX, axis)
    series, _ = oracle.run(sc, profile_override=prof, probes=probes)
    for avg, name in ((False, key), (True, f"current_avg_d{axis + 1}")):
        V, I = oracle.port_vi(series, gs.PORT_BOX, gs.PORT_CURRENT_BOX, sc, col0=len(sc.probes),
                              time_average=avg, current_axis=axis)
        assert bitwise_equal(V, fix["voltage"])
        assert bitwise_equal(I, fix[name]), name
        assert np.abs(I).max() > 0


def test_zin_s11_formulas_against_reference():
    fix = golden("port")
    for q, z0 in enumerate(fix["z0"]):
        ref = oracle.zin_s11(fix["spec_v"].astype(np.complex128), fix["spec_i"].astype(np.complex128), complex(z0))
        for k in ("s11", "zin"):
            got = fix[k][q].astype(np.complex128)
            err = np.abs(got - ref[k]) / np.maximum(np.abs(ref[k]), 1e-30)
            assert np.median(err) < 1e-6 and np.max(err) < 1e-4, (k, q, err.max())


def test_port_spectra_of_a_known_signal():
    """A pure matched load: with I = V / z0 the reflection b vanishes and zin equals z0."""
    n, z0 = 256, 50.0
    t = np.arange(n)
    V = np.exp(-((t - 40) / 9.0) ** 2)
    out = oracle.port_spectra(V, V / z0, z0)
    assert np.allclose(out["s11"], 0, atol=1e-12 * np.abs(out["v"]).max() / np.abs(out["v"]).min())
    assert np.abs(out["s11"][:20]).max() < 1e-12
    assert np.allclose(out["zin"], z0)
    assert np.allclose(out["v"], np.fft.rfft(V))
