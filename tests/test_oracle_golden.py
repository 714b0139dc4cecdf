"""The CPU oracle against the golden fixtures produced by the reference's own kernels.

These pin the oracle: coefficient arrays and single steps must be bit-exact, full runs within the
FP32 parity bar, and the FP64 build states the FP32 error of the reference itself.
"""
import os

import numpy as np
import pytest

import golden_scenarios as gs
import oracle
from conftest import GOLDEN, REL_L2_TOL, bitwise_equal, golden, rel_l2, rel_l2_group

COEF_MAP = {"eps_r_x": "eps_x", "sigma_e_x": "sig_x", "eps_r_y": "eps_y", "sigma_e_y": "sig_y",
            "eps_r_z": "eps_z", "sigma_e_z": "sig_z", "mu_r_x": "mu_x", "sigma_m_x": "sm_x",
            "mu_r_y": "mu_y", "sigma_m_y": "sm_y", "mu_r_z": "mu_z", "sigma_m_z": "sm_z"}
FIELDS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def ref_profiles(fix):
    return {a: fix["cpml_" + a] for a in oracle.PROFILE_NAMES}


@pytest.fixture(scope="module")
def coefs():
    return golden("coefs_onestep")


def test_coefficients_bitwise(coefs):
    """Every per-edge array of setSigmaEpsSigmaMu / setCoefficients / setABCPML / defineSourceZ."""
    sc = gs.onestep_scenario()
    for name in coefs.files:
        if name.startswith("cpml_"):
            continue
        o = oracle.coef(sc, COEF_MAP.get(name, name))
        assert bitwise_equal(o, coefs[name]), name


def test_cpml_profiles_close(coefs):
    """1-D CPML profiles: the oracle uses the host libm's powf/expf, the reference CUDA's; the b
    values agree to a few ulp and a = (b-1)*... inherits that through the cancellation in b-1."""
    sc = gs.onestep_scenario()
    for name in oracle.PROFILE_NAMES:
        r = coefs["cpml_" + name]
        o = oracle.coef(sc, name)[: r.size]
        ulp = np.abs(r.view(np.int32).astype(np.int64) - o.view(np.int32).astype(np.int64)).max()
        assert ulp <= (2 if name.startswith("b") else 64), (name, ulp)


def test_onestep_bitwise():
    """calc_e then calc_h from a seeded random state, with the reference's own 1-D profiles."""
    sc = gs.onestep_scenario()
    fix = golden("onestep")
    if "signal" in fix.files:
        sig = fix["signal"]
        sc.sources[0].waveform = np.asarray(sig, dtype=np.float32) * np.float32(sc.sources[0].box[5] - sc.sources[0].box[2])
        sc.steps = sig.size
    rng = np.random.default_rng(99)
    shape = (sc.nz, sc.ny, sc.nx)
    state = {n: rng.standard_normal(shape).astype(np.float32) for n in FIELDS}
    init = np.stack([state[n] for n in FIELDS])
    out = oracle.onestep(sc, gs.ONESTEP_M, init, profile_override=ref_profiles(golden("coefs_onestep")))
    for c, n in enumerate(FIELDS):
        key = n + ("_after_e" if c < 3 else "_after_h")
        assert bitwise_equal(out[c], fix[key]), key


@pytest.mark.parametrize("name", ["small_vacuum", "small_boxes", "two_sources", "vacuum64"])
def test_full_runs(name):
    sc = dict((s.name, s) for s, _ in gs.fixture_scenarios())[name]
    fix = golden(name)
    probes, fields = oracle.run(sc)
    assert rel_l2(probes, fix["probes"]) < REL_L2_TOL
    if name != "vacuum64":
        ref = [fix[n] for n in FIELDS]
        for c, n in enumerate(FIELDS):
            assert rel_l2_group(fields, ref, c) < REL_L2_TOL, n


@pytest.mark.parametrize("name", ["small_vacuum", "small_boxes", "plates", "aniso"])
def test_full_runs_bitwise_with_reference_profiles(name):
    """With the reference's own 1-D CPML b / a profiles (CUDA expf), single-source runs are
    bit-exact: probes of every step and the final fields. The CPML stretching kappa is still the
    oracle's (host powf); for these thin CPMLs it equals CUDA's, so the runs match exactly."""
    sc = dict((s.name, s) for s, _ in gs.fixture_scenarios())[name]
    if not os.path.exists(os.path.join(GOLDEN, name + ".npz")):
        pytest.skip("fixture not generated")
    fix = golden(name)
    if "cpml_b_ex" not in fix.files:
        pytest.skip("fixture predates the stored profiles")
    probes, fields = oracle.run(sc, profile_override=ref_profiles(fix))
    assert bitwise_equal(probes, fix["probes"])
    for c, n in enumerate(FIELDS):
        if n in fix.files:
            assert bitwise_equal(fields[c], fix[n]), n
        else:
            assert bitwise_equal(fields[c][sc.nz // 2], fix[n + "_zmid"]), n


def test_fp64_error_statement():
    """The FP64 build of the same update at small size: the reference's FP32 probe error against it
    is small but nonzero (it is the FP32 rounding error of the scheme, reported in DESIGN)."""
    sc = gs.small_vacuum()
    fix = golden("small_vacuum")
    p64, _ = oracle.run(sc, precision="f64")
    err = rel_l2(fix["probes"], p64)
    assert 0 < err < 1e-4


def test_onestep_random_psi_bitwise():
    """Random fields and random CPML memory: every field and every psi array after one calc_e +
    calc_h equals the reference's (this pins the psi recurrences and corrections)."""
    sc = gs.onestep_scenario()
    fix = golden("onestep_psi")
    sc.sources[0].waveform = gs.onestep_signal()
    sc.steps = gs.ONESTEP_M + 1
    rng = np.random.default_rng(77)
    shape = (sc.nz, sc.ny, sc.nx)
    names = FIELDS + tuple(oracle.PSI_NAMES)
    st = {n: rng.standard_normal(shape).astype(np.float32) for n in names}
    out, psi = oracle.onestep(sc, gs.ONESTEP_M, np.stack([st[n] for n in FIELDS]),
                              profile_override=ref_profiles(golden("coefs_onestep")),
                              init_psi=np.stack([st[n] for n in oracle.PSI_NAMES]), return_psi=True)
    for c, n in enumerate(FIELDS):
        key = n + ("_after_e" if c < 3 else "_after_h")
        assert bitwise_equal(out[c], fix[key]), key
    for q, n in enumerate(oracle.PSI_NAMES):
        assert bitwise_equal(psi[q], fix[n + "_after"]), n


def test_aniso_coefficients_bitwise():
    """Per-axis bricks: every per-edge array of setSigmaEpsSigmaMu / setCoefficients / setABCPML /
    defineSourceZ equals the reference's (each component averages its own axis' values)."""
    if not os.path.exists(os.path.join(GOLDEN, "aniso.npz")):
        pytest.skip("fixture not generated")
    sc = gs.aniso_scenario()
    fix = golden("aniso")
    names = [n[5:] for n in fix.files if n.startswith("coef_")]
    assert "eps_r_y" in names and "mu_r_z" in names
    for name in names:
        o = oracle.coef(sc, COEF_MAP.get(name, name))
        assert bitwise_equal(o, fix["coef_" + name]), name
