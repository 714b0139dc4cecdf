"""fdtd_marching_loop (the reference's whole run behind marchingLoop's parameter list), the
exact-signature marchingLoop shim (include/compat/fdtdrav.h) and fdtd_source_waveform against the
reference's own kernels.

- the waveform equals setGauss / setSine bit for bit;
- V(t) and the time-averaged I(t) of the reduced microstrip case equal the reference pipeline's
  (setGauss, the setup kernels with plates, calc_e / calc_h sampling, voltMgpu / currMgpu /
  correcI) bit for bit: against the committed fixture, and live through the reference-kernel
  harness for other current directions, waveforms and NUMDEV values when it is present.
"""
import os
import subprocess

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
        v, _, i_avg = h.port_reduce(n, a["current_direction"], a["voltage_direction"])
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


@pytest.mark.parametrize("kw,extra", [(dict(current_direction=3), {}), (dict(current_direction=2, source_tp=3), {}),
                                      (dict(current_direction=2, numdev=4, resistor_opt=1), {}),
                                      (dict(current_direction=2, aniso=True), {}),
                                      (dict(current_direction=1), dict(voltage_direction=1)),
                                      (dict(current_direction=2), dict(voltage_direction=2))])
def test_marching_loop_vs_reference_live(gpu_lib, kw, extra):
    """Also the x and y voltage directions (voltMgpu 1 and 2); for y the voltage box gets two
    rows."""
    from fdtd_gb300 import solver
    a = gs.marching_params(n_t_steps=300, **kw)
    a.update(extra)
    if a["voltage_direction"] == 2:
        a["sampled_voltage_max_y"] = np.float32(a["sampled_voltage_max_y"] + 2 * a["dy"])
    sig, v_ref, i_ref = reference_run(a)
    w = solver.source_waveform(a["source_tp"], a["source_amp"], a["source_freq"], a["dt"], a["t_0"], a["tau"], a["pi"],
                               a["n_t_steps"])
    assert bitwise_equal(w, sig)
    V, I = solver.marching_loop(a)
    assert bitwise_equal(V, v_ref)
    assert bitwise_equal(I, i_ref)


def test_marching_loop_validation(gpu_lib):
    from fdtd_gb300 import solver
    for change in [dict(source_direction=1), dict(voltage_direction=4), dict(current_direction=4),
                   dict(brick_sigma_m_y=[0.0]), dict(NUMDEV=0)]:
        a = gs.marching_params(n_t_steps=20)
        a.update(change)
        with pytest.raises(solver.FDTDError):
            solver.marching_loop(a)


def write_params(a, path):
    """marchingLoop's parameters as the driver reads them: "name kind value" lines in signature
    order, arrays as "name a n v0 .. vn-1"; floats with 9 significant digits (exact for float32)."""
    with open(path, "w") as f:
        for name, kind in S.MARCHING_PARAMS:
            v = a[name]
            if kind == "a":
                arr = np.asarray(v, dtype=np.float32).reshape(-1)
                f.write(f"{name} a {arr.size} " + " ".join(f"{float(x):.9g}" for x in arr) + "\n")
            elif kind == "i":
                f.write(f"{name} i {int(v)}\n")
            else:
                f.write(f"{name} f {float(np.float32(v)):.9g}\n")


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "marching.npz")), reason="fixture not generated")
def test_marching_loop_shim_writes_reference_result_files(gpu_lib, tmp_path):
    """A source.cu-shaped driver compiled against include/compat/fdtdrav.h calls marchingLoop by
    position; results1003.dat / results1004.dat hold, line for line, what the reference's
    saveTDomain writes for its own V(t) and averaged I(t) ("%e \\n" of the fixture's values)."""
    from fdtd_gb300 import solver
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "marching_driver")
    lib_dir = os.path.dirname(solver.LIB_PATH)
    subprocess.check_call(["g++", "-O1", "-std=c++17", os.path.join(root, "tests", "marching_driver.cpp"),
                           "-I" + os.path.join(root, "include", "compat"), "-L" + lib_dir, "-lfdtd_gb300",
                           "-Wl,-rpath," + lib_dir, "-o", exe])
    a = gs.marching_params()
    write_params(a, str(tmp_path / "params.txt"))
    out = subprocess.run([exe, str(tmp_path / "params.txt")], cwd=str(tmp_path), capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    assert "End of Program" in out.stdout
    fix = golden("marching")
    for name, key in (("results1003.dat", "voltage"), ("results1004.dat", "current_avg")):
        with open(tmp_path / name) as f:
            lines = f.read().splitlines()
        want = ["%e " % float(v) for v in fix[key]]
        assert lines == want, name
