"""fdtd_marching_loop (the reference's whole run behind marchingLoop's parameter list) and
fdtd_source_waveform against the reference's own kernels.

- the waveform equals setGauss / setSine bit for bit;
- V(t) and the time-averaged I(t) of the reduced microstrip case equal the reference pipeline's
  (setGauss, the setup kernels with plates, calc_e / calc_h sampling, voltMgpu / currMgpu /
  correcI) bit for bit: against the committed fixture, and live through the reference-kernel
  harness for other current directions, waveforms and NUMDEV values when it is present.
"""
import os

import numpy as np
import pytest

import golden_scenarios as gs
from conftest import GOLDEN, bitwise_equal, golden
from fdtd_gb300 import scenario as S

pytestmark = pytest.mark.gpu


def harness():
    import refharness
    if not refharness.available():
        pytest.skip("reference-kernel harness not built")
    return refharness.RefHarness()


def reference_run(a):
    """The reference's pipeline for marchingLoop parameters ``a`` through the harness."""
    n = a["n_t_steps"]
    h = harness()
    try:
        src = S.marching_indices(a)["source"]
        sig, per = h.waveform(a["source_tp"], a["source_amp"], src[5] - src[2], a["source_freq"], a["dt"], a["t_0"],
                              a["tau"], a["pi"], n)
        sc, vbox, cbox = S.marching_scenario(a, sig)
        h.setup(sc)
        h.set_port(vbox, cbox, n)
        h.run(n, src_slot=0, signal=per)
        v, _, i_avg = h.port_reduce(n, a["current_direction"])
        return sig, v, i_avg
    finally:
        h.close()


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "marching.npz")), reason="fixture not generated")
def test_marching_loop_vs_fixture(gpu_lib):
    from fdtd_gb300 import solver
    a = gs.marching_params()
    fix = golden("marching")
    V, I = solver.marching_loop(a)
    assert bitwise_equal(V, fix["voltage"])
    assert bitwise_equal(I, fix["current_avg"])
    assert np.abs(V).max() > 1e-3 and np.abs(I).max() > 1e-6
    src = S.marching_indices(a)["source"]
    w = solver.source_waveform(1, a["source_amp"], a["source_freq"], a["dt"], a["t_0"], a["tau"], a["pi"], a["n_t_steps"])
    assert bitwise_equal(w, fix["signal"])
    assert src[5] - src[2] == 3


@pytest.mark.parametrize("kw", [dict(current_direction=3), dict(current_direction=2, source_tp=3),
                                dict(current_direction=2, numdev=4, resistor_opt=1)])
def test_marching_loop_vs_reference_live(gpu_lib, kw):
    from fdtd_gb300 import solver
    a = gs.marching_params(n_t_steps=300, **kw)
    sig, v_ref, i_ref = reference_run(a)
    w = solver.source_waveform(a["source_tp"], a["source_amp"], a["source_freq"], a["dt"], a["t_0"], a["tau"], a["pi"],
                               a["n_t_steps"])
    assert bitwise_equal(w, sig)
    V, I = solver.marching_loop(a)
    assert bitwise_equal(V, v_ref)
    assert bitwise_equal(I, i_ref)


def test_marching_loop_validation(gpu_lib):
    from fdtd_gb300 import solver
    for change in [dict(source_direction=1), dict(voltage_direction=2), dict(current_direction=4),
                   dict(brick_eps_r_y=[3.0]), dict(NUMDEV=0)]:
        a = gs.marching_params(n_t_steps=20)
        a.update(change)
        with pytest.raises(solver.FDTDError):
            solver.marching_loop(a)
