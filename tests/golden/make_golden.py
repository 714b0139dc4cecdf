"""Generate golden fixtures by running the reference's own kernels (needs a GPU and the
reference-kernel harness built under oracle/_ref by oracle/build_ref.sh).

    python tests/golden/make_golden.py --out <dir> [--analysis <dir>]

Writes one compressed .npz per scenario: the probe series of every step and, for the small grids,
the six final fields; plus ``onestep.npz`` (one calc_e and one calc_h applied to a seeded random
state) and ``coefs.npz`` (the reference's per-edge coefficients and 1-D CPML profiles for the
random-box scenario); ``port.npz`` (the reference's own port sampling and time-series kernels,
voltMgpu / currMgpu / correcI, on the port scenario, plus c_zinS11 on seeded spectra);
``aniso.npz`` (per-axis bricks: the run and the reference's per-edge coefficient arrays);
``port_xy.npz`` (voltMgpu's x and y directions on the port run's samples). The
scenarios are defined in golden_scenarios.py so the tests rebuild them
bit-for-bit without running this script.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref_harness"))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import refharness  # noqa: E402
import golden_scenarios as gs  # noqa: E402

COEF_NAMES = ["Cexe", "Cexhz", "Cexhy", "Ceye", "Ceyhx", "Ceyhz", "Ceze", "Cezhy", "Cezhx", "Cezj",
              "Chxh", "Chxey", "Chxez", "Chyh", "Chyez", "Chyex", "Chzh", "Chzex", "Chzey",
              "eps_r_x", "sigma_e_x", "eps_r_y", "sigma_e_y", "eps_r_z", "sigma_e_z",
              "mu_r_x", "sigma_m_x", "mu_r_y", "sigma_m_y", "mu_r_z", "sigma_m_z",
              "cpsi_eyx", "cpsi_ezx", "cpsi_hyx", "cpsi_hzx", "cpsi_exy", "cpsi_ezy", "cpsi_hxy", "cpsi_hzy",
              "cpsi_exz", "cpsi_eyz", "cpsi_hxz", "cpsi_hyz"]
LINE_NAMES = [("cpml_b_ex", "x"), ("cpml_a_ex", "x"), ("cpml_b_mx", "x"), ("cpml_a_mx", "x"),
              ("cpml_b_ey", "y"), ("cpml_a_ey", "y"), ("cpml_b_my", "y"), ("cpml_a_my", "y"),
              ("cpml_b_ez", "z"), ("cpml_a_ez", "z"), ("cpml_b_mz", "z"), ("cpml_a_mz", "z")]
PSI_E = ["Psi_eyx", "Psi_ezx", "Psi_exy", "Psi_ezy", "Psi_exz", "Psi_eyz"]
PSI_H = ["Psi_hyx", "Psi_hzx", "Psi_hxy", "Psi_hzy", "Psi_hxz", "Psi_hyz"]


def line_len(sc, axis):
    return {"x": sc.nx, "y": sc.ny, "z": sc.nz}[axis]


def run_scenario(sc, full_fields: bool):
    t0 = time.time()
    probes, fields = refharness.run_reference(sc, with_fields=True)
    out = {"probes": probes}
    if full_fields:
        for k, v in fields.items():
            out[k] = v
    else:
        for k, v in fields.items():
            out[k + "_l2"] = np.array(np.linalg.norm(v.astype(np.float64)))
            out[k + "_zmid"] = v[sc.nz // 2].copy()
    h = refharness.RefHarness()
    try:
        h.setup(sc)
        for n, ax in LINE_NAMES:
            out[n] = h.get(n, line_len(sc, ax))
    finally:
        h.close()
    print(f"{sc.name}: {sc.nx}x{sc.ny}x{sc.nz} x {sc.steps} steps, {len(sc.sources)} source(s) "
          f"in {time.time() - t0:.1f}s", flush=True)
    return out


def coef_dump(sc):
    h = refharness.RefHarness()
    try:
        h.setup(sc)
        out = {n: h.get(n) for n in COEF_NAMES}
        for n, ax in LINE_NAMES:
            out[n] = h.get(n, line_len(sc, ax))
        return out
    finally:
        h.close()


def onestep(sc, seed=99):
    """Seeded random E and H, one reference calc_e (source slot 0 at step m) then one calc_h."""
    rng = np.random.default_rng(seed)
    shape = (sc.nz, sc.ny, sc.nx)
    state = {n: rng.standard_normal(shape).astype(np.float32) for n in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")}
    m = gs.ONESTEP_M
    h = refharness.RefHarness()
    try:
        h.setup(sc)
        for n, v in state.items():
            h.set(n, v)
        sig = gs.onestep_signal()
        h.calc_e(m, 0, sig)
        out = {n + "_after_e": h.get(n) for n in ("Ex", "Ey", "Ez")}
        out["signal"] = sig
        for n in PSI_E:
            out[n] = h.get(n)
        h.calc_h(m)
        for n in ("Hx", "Hy", "Hz"):
            out[n + "_after_h"] = h.get(n)
        for n in PSI_H:
            out[n] = h.get(n)
        return out
    finally:
        h.close()


def onestep_psi(sc, seed=77):
    """Seeded random E, H and all 12 CPML psi arrays, one reference calc_e then one calc_h: pins
    the rounding of the psi recurrences and of the psi corrections."""
    rng = np.random.default_rng(seed)
    shape = (sc.nz, sc.ny, sc.nx)
    names = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz") + tuple(PSI_E) + tuple(PSI_H)
    state = {n: rng.standard_normal(shape).astype(np.float32) for n in names}
    m = gs.ONESTEP_M
    h = refharness.RefHarness()
    try:
        h.setup(sc)
        for n, v in state.items():
            h.set(n, v)
        sig = gs.onestep_signal()
        h.calc_e(m, 0, sig)
        out = {n + "_after_e": h.get(n) for n in ("Ex", "Ey", "Ez")}
        for n in PSI_E:
            out[n + "_after"] = h.get(n)
        h.calc_h(m)
        for n in ("Hx", "Hy", "Hz"):
            out[n + "_after_h"] = h.get(n)
        for n in PSI_H:
            out[n + "_after"] = h.get(n)
        return out
    finally:
        h.close()


def port_xy_fixture():
    """voltMgpu's three voltage directions (1 / 2 / 3 = x / y / z) on the reference's own Ez samples
    of the port run: the same sampled array, other ranges and scale (fdtdrav.h:2214-2290)."""
    sc = gs.port_scenario()
    h = refharness.RefHarness()
    try:
        h.setup(sc)
        h.set_port(gs.PORT_BOX, gs.PORT_BOX, sc.steps)
        h.run(sc.steps, src_slot=0, signal=sc.signal_per_node(0))
        return {f"voltage_d{d}": h.port_reduce(sc.steps, 3, d)[0] for d in (1, 2, 3)}
    finally:
        h.close()


def port_fixture():
    """Port V(t) / I(t) of the reference's own sampling (calc_e / calc_h sample boxes) and
    reductions; and c_zinS11 applied to seeded random spectra (n = 700, 351 bins)."""
    sc = gs.port_scenario()
    h = refharness.RefHarness()
    try:
        h.setup(sc)
        h.set_port(gs.PORT_BOX, gs.PORT_BOX, sc.steps)
        probes, _ = h.run(sc.steps, src_slot=0, signal=sc.signal_per_node(0), probes=sc.probes)
        v, i_raw, i_avg = h.port_reduce(sc.steps)
        # the same run with the current box that all three loop directions fit
        h.setup(sc)
        h.set_port(gs.PORT_BOX, gs.PORT_CURRENT_BOX, sc.steps)
        h.run(sc.steps, src_slot=0, signal=sc.signal_per_node(0))
        loops = {}
        for d in (1, 2, 3):
            _, loops[f"current_raw_d{d}"], loops[f"current_avg_d{d}"] = h.port_reduce(sc.steps, d)
        rng = np.random.default_rng(321)
        nf = sc.steps // 2 + 1
        sv = (rng.standard_normal(nf) + 1j * rng.standard_normal(nf)).astype(np.complex64)
        si = (rng.standard_normal(nf) + 1j * rng.standard_normal(nf)).astype(np.complex64) * np.float32(0.02)
        z0 = complex(50.0, 0.0)
        s11, zin = h.zin(sc.steps, sv, si, z0)
        z1 = complex(75.0, -12.5)
        s11b, zinb = h.zin(sc.steps, sv, si, z1)
        lines = {n: h.get(n, line_len(sc, ax)) for n, ax in LINE_NAMES}
    finally:
        h.close()
    return {"probes": probes, "voltage": v, "current_raw": i_raw, "current_avg": i_avg,
            "spec_v": sv, "spec_i": si, "z0": np.array([z0, z1], dtype=np.complex64),
            "s11": np.stack([s11, s11b]), "zin": np.stack([zin, zinb]), **lines, **loops}


def marching_fixture():
    """The reference's own pipeline on the reduced microstrip case (marchingLoop's index set-up
    restated in fdtd_gb300.scenario): setGauss, the setup kernels, calc_e / calc_h with its sample
    boxes, voltMgpu / currMgpu (y loop) / correcI."""
    from fdtd_gb300 import scenario as S
    a = gs.marching_params()
    n = a["n_t_steps"]
    h = refharness.RefHarness()
    try:
        ix = S.marching_indices(a)
        src = ix["source"]
        sig, per = h.waveform(1, a["source_amp"], src[5] - src[2], a["source_freq"], a["dt"], a["t_0"], a["tau"],
                              a["pi"], n)
        sc, vbox, cbox = S.marching_scenario(a, sig)
        h.setup(sc)
        h.set_port(vbox, cbox, n)
        h.run(n, src_slot=0, signal=per)
        v, i_raw, i_avg = h.port_reduce(n, a["current_direction"])
    finally:
        h.close()
    return {"signal": sig, "voltage": v, "current_raw": i_raw, "current_avg": i_avg}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--analysis", default=None, help="also write large analysis-only dumps here")
    ap.add_argument("--only", default=None, choices=["port", "plates", "marching", "aniso", "port_xy"],
                    help="write one fixture only")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)
    if args.only == "port":
        np.savez_compressed(os.path.join(args.out, "port.npz"), **port_fixture())
        print("port fixture written to", args.out)
    if args.only == "port_xy":
        np.savez_compressed(os.path.join(args.out, "port_xy.npz"), **port_xy_fixture())
        print("port_xy fixture written to", args.out)
        return
    if args.only == "marching":
        np.savez_compressed(os.path.join(args.out, "marching.npz"), **marching_fixture())
        print("marching fixture written to", args.out)
        return
    if args.only == "aniso":
        sc = gs.aniso_scenario()
        out = run_scenario(sc, True)
        out.update({"coef_" + k: v for k, v in coef_dump(sc).items() if not k.startswith("cpml_")})
        np.savez_compressed(os.path.join(args.out, "aniso.npz"), **out)
        print("aniso fixture written to", args.out)
        return
    if args.only == "plates":
        np.savez_compressed(os.path.join(args.out, "plates.npz"), **run_scenario(gs.plates_scenario(), True))
        print("plates fixture written to", args.out)
        return
    np.savez_compressed(os.path.join(args.out, "port.npz"), **port_fixture())
    for sc, full in gs.fixture_scenarios():
        np.savez_compressed(os.path.join(args.out, sc.name + ".npz"), **run_scenario(sc, full))
    np.savez_compressed(os.path.join(args.out, "onestep.npz"), **onestep(gs.onestep_scenario()))
    np.savez_compressed(os.path.join(args.out, "coefs_onestep.npz"), **coef_dump(gs.onestep_scenario()))
    np.savez_compressed(os.path.join(args.out, "onestep_psi.npz"), **onestep_psi(gs.onestep_scenario()))
    if args.analysis:
        os.makedirs(args.analysis, exist_ok=True)
        np.savez_compressed(os.path.join(args.analysis, "coefs_boxes.npz"), **coef_dump(gs.boxes_scenario()))
        sc = gs.boxes_scenario()
        for n in (39, 41, 45):
            _, f = refharness.run_reference(sc, steps=n)
            np.savez_compressed(os.path.join(args.analysis, f"boxes_fields_{n}.npz"), **f)
    print("golden fixtures written to", args.out)


if __name__ == "__main__":
    main()
