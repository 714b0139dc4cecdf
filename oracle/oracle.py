"""ctypes wrapper of the CPU oracle (oracle/fdtd_oracle.cpp). TEST INFRASTRUCTURE ONLY.

The oracle restates the reference's setup and calc_e / calc_h on the CPU (FP32 with the
reference's rounding sequence, and FP64 as the error reference). Only tests, smoke() and the
benchmark's CPU-baseline leg may use it, always as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libfdtd_oracle.so")
SRC = os.path.join(HERE, "fdtd_oracle.cpp")

_i = ctypes.c_int
_f = ctypes.c_float
_pi = ctypes.POINTER(ctypes.c_int)
_pf = ctypes.POINTER(ctypes.c_float)
_pd = ctypes.POINTER(ctypes.c_double)
_pu8 = ctypes.POINTER(ctypes.c_uint8)

# Override slots: per axis b_e, a_e, b_m, a_m, kappa_e, kappa_m.
OVERRIDE_NAMES = ["b_ex", "a_ex", "b_mx", "a_mx", "k_ex", "k_mx", "b_ey", "a_ey", "b_my", "a_my", "k_ey", "k_my",
                  "b_ez", "a_ez", "b_mz", "a_mz", "k_ez", "k_mz"]
# 1-D arrays the reference keeps (its kappa values are locals of setABCPML).
PROFILE_NAMES = ["b_ex", "a_ex", "b_mx", "a_mx", "b_ey", "a_ey", "b_my", "a_my", "b_ez", "a_ez", "b_mz", "a_mz"]


class _Scenario(ctypes.Structure):
    _fields_ = [("nx", _i), ("ny", _i), ("nz", _i), ("pml", _i * 6),
                ("dx", _f), ("dy", _f), ("dz", _f), ("dt", _f), ("eps0", _f), ("mu0", _f), ("pi", _f),
                ("mat", _pu8), ("table", _pf), ("n_mat", _i),
                ("nsrc", _i), ("src_box", _pi), ("src_r", _pf),
                ("nres", _i), ("res_box", _pi), ("res_r", _pf),
                ("nprobe", _i), ("probe", _pi),
                ("profile_override", ctypes.POINTER(_pf)),
                ("design_box", _i * 6), ("design_eps", ctypes.POINTER(ctypes.c_double)),
                ("nplate", _i), ("plate", _pi), ("plate_sig", _pf),
                ("nsrcx", _i), ("srcx_box", _pi), ("srcx_r", _pf)]


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (no contraction: the FMA sequence is written out in the source)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-shared", "-fPIC",
                               "-o", LIB, SRC])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.or_error.restype = ctypes.c_char_p
        L.or_run_f32.argtypes = [ctypes.POINTER(_Scenario), _i, _pf, _i, _pf, _pf, _pf, _i]
        L.or_run_f64.argtypes = [ctypes.POINTER(_Scenario), _i, _pf, _i, _pf, _pd, _pd, _i]
        L.or_onestep_f32.argtypes = [ctypes.POINTER(_Scenario), _i, _pf, _i, _pf, _pf, _pf, _pf]
        L.or_coef_f32.argtypes = [ctypes.POINTER(_Scenario), ctypes.c_char_p, _pf]
        L.or_port_vi.argtypes = [_pf, _i, _i, _i, _pi, _pi, _i, _i, _f, _f, _f, _i, _pf, _pf]
        L.or_last_step_seconds.restype = ctypes.c_double
        L.or_last_step_seconds.argtypes = []
        for fn in (L.or_fom_grad_f64, L.or_fom_grad_f32, L.or_fom_grad_box_f64):
            fn.argtypes = [ctypes.POINTER(_Scenario), _i, _pf, _i, _i, _i, _i, _pd, _pd]
        _lib = L
    return _lib


class _Prepared:
    def __init__(self, sc, profile_override: Optional[dict] = None, probes: Optional[Sequence] = None,
                 design=None):
        self.keep = []
        s = _Scenario()
        if design is not None:  # (box (6 ints), eps array (nz_d, ny_d, nx_d) float64)
            box, eps = design
            e = np.ascontiguousarray(eps, dtype=np.float64)
            self.keep.append(e)
            for q in range(6):
                s.design_box[q] = int(box[q])
            s.design_eps = e.ctypes.data_as(_pd)
        s.nx, s.ny, s.nz = sc.nx, sc.ny, sc.nz
        for q in range(6):
            s.pml[q] = sc.pml[q]
        s.dx, s.dy, s.dz, s.dt = sc.dx, sc.dy, sc.dz, sc.dt
        s.eps0, s.mu0, s.pi = sc.eps0, sc.mu0, sc.pi
        mat = np.ascontiguousarray(sc.material_index())
        tab = np.ascontiguousarray(sc.material_table_axes())
        sb = np.array([x.box for x in sc.sources], dtype=np.int32).reshape(-1, 6)
        sr = np.array([x.resistance for x in sc.sources], dtype=np.float32)
        rb = np.array([x.box for x in sc.resistors], dtype=np.int32).reshape(-1, 6)
        rr = np.array([x.resistance for x in sc.resistors], dtype=np.float32)
        probes = sc.probes if probes is None else probes
        pr = np.array([[p.component, p.i, p.j, p.k] for p in probes], dtype=np.int32).reshape(-1, 4)
        plates = getattr(sc, "plates", [])
        pl = np.array([[q.axis, *q.box] for q in plates], dtype=np.int32).reshape(-1, 7)
        ps = np.array([[q.sigma_1, q.sigma_2] for q in plates], dtype=np.float32).reshape(-1, 2)
        xs = getattr(sc, "x_sources", [])
        xb = np.array([x.box for x in xs], dtype=np.int32).reshape(-1, 6)
        xr = np.array([x.resistance for x in xs], dtype=np.float32)
        self.keep += [mat, tab, sb, sr, rb, rr, pr, pl, ps, xb, xr]
        s.nsrcx, s.srcx_box, s.srcx_r = len(xs), xb.ctypes.data_as(_pi), xr.ctypes.data_as(_pf)
        s.nplate, s.plate, s.plate_sig = len(plates), pl.ctypes.data_as(_pi), ps.ctypes.data_as(_pf)
        s.mat, s.table, s.n_mat = mat.ctypes.data_as(_pu8), tab.ctypes.data_as(_pf), tab.shape[0]
        s.nsrc, s.src_box, s.src_r = len(sc.sources), sb.ctypes.data_as(_pi), sr.ctypes.data_as(_pf)
        s.nres, s.res_box, s.res_r = len(sc.resistors), rb.ctypes.data_as(_pi), rr.ctypes.data_as(_pf)
        s.nprobe, s.probe = len(probes), pr.ctypes.data_as(_pi)
        if profile_override:
            arr = (_pf * 18)()
            for q, n in enumerate(OVERRIDE_NAMES):
                if n in profile_override:
                    a = np.ascontiguousarray(profile_override[n], dtype=np.float32)
                    self.keep.append(a)
                    arr[q] = a.ctypes.data_as(_pf)
                else:
                    arr[q] = None
            self.keep.append(arr)
            s.profile_override = ctypes.cast(arr, ctypes.POINTER(_pf))
        else:
            s.profile_override = None
        steps = max(sc.steps, 1)
        sig = np.zeros((max(len(sc.sources), 1), steps), dtype=np.float32)
        for q in range(len(sc.sources)):
            v = sc.signal_per_node(q)[:steps]
            sig[q, :v.size] = v
        self.sig = np.ascontiguousarray(sig)
        self.n_sig = steps
        self.s = s
        self.n_probes = len(probes)


def run(sc, steps: Optional[int] = None, precision: str = "f32", init_fields: Optional[np.ndarray] = None,
        profile_override: Optional[dict] = None, threads: int = 0, probes: Optional[Sequence] = None,
        design=None):
    """Run the oracle. Returns (probes (steps, n_probes), fields (6, nz, ny, nx)). ``design`` =
    (box, eps_r array) overrides eps_r of the design cells."""
    steps = sc.steps if steps is None else steps
    p = _Prepared(sc, profile_override, probes, design)
    dt = np.float32 if precision == "f32" else np.float64
    pout = np.zeros((steps, max(p.n_probes, 1)), dtype=dt)
    fout = np.zeros((6, sc.nz, sc.ny, sc.nx), dtype=dt)
    init = None
    if init_fields is not None:
        init = np.ascontiguousarray(init_fields, dtype=np.float32)
    L = lib()
    fn = L.or_run_f32 if precision == "f32" else L.or_run_f64
    ptr = _pf if precision == "f32" else _pd
    rc = fn(ctypes.byref(p.s), steps, p.sig.ctypes.data_as(_pf), p.n_sig,
            None if init is None else init.ctypes.data_as(_pf),
            pout.ctypes.data_as(ptr), fout.ctypes.data_as(ptr), threads)
    if rc != 0:
        raise RuntimeError("oracle: " + L.or_error().decode())
    return pout[:, :p.n_probes], fout


def last_step_seconds() -> float:
    """Wall time of the time loop of the last ``run`` (setup and copies excluded)."""
    return float(lib().or_last_step_seconds())


# Order of the 12 psi arrays in onestep's init_psi / psi output.
PSI_NAMES = ["Psi_eyx", "Psi_ezx", "Psi_exy", "Psi_ezy", "Psi_exz", "Psi_eyz",
             "Psi_hyx", "Psi_hzx", "Psi_hxy", "Psi_hzy", "Psi_hxz", "Psi_hyz"]


def onestep(sc, m: int, init_fields: np.ndarray, profile_override: Optional[dict] = None,
            init_psi: Optional[np.ndarray] = None, return_psi: bool = False):
    """One calc_e then one calc_h from ``init_fields`` (6, nz, ny, nx) and optionally ``init_psi``
    (12, nz, ny, nx, order PSI_NAMES); returns the 6 fields after (and the 12 psi arrays)."""
    p = _Prepared(sc, profile_override)
    init = np.ascontiguousarray(init_fields, dtype=np.float32)
    out = np.zeros((6, sc.nz, sc.ny, sc.nx), dtype=np.float32)
    ipsi = None if init_psi is None else np.ascontiguousarray(init_psi, dtype=np.float32)
    psi = np.zeros((12, sc.nz, sc.ny, sc.nx), dtype=np.float32) if return_psi else None
    L = lib()
    rc = L.or_onestep_f32(ctypes.byref(p.s), m, p.sig.ctypes.data_as(_pf), p.n_sig, init.ctypes.data_as(_pf),
                          out.ctypes.data_as(_pf), None if ipsi is None else ipsi.ctypes.data_as(_pf),
                          None if psi is None else psi.ctypes.data_as(_pf))
    if rc != 0:
        raise RuntimeError("oracle: " + L.or_error().decode())
    return (out, psi) if return_psi else out


def coef(sc, name: str, profile_override: Optional[dict] = None) -> np.ndarray:
    """A per-edge coefficient array (reference naming) after the oracle's setup."""
    p = _Prepared(sc, profile_override)
    n_line = {"x": sc.nx, "y": sc.ny, "z": sc.nz}
    if name in PROFILE_NAMES:
        out = np.zeros(n_line[name[-1]], dtype=np.float32)
    else:
        out = np.zeros((sc.nz, sc.ny, sc.nx), dtype=np.float32)
    L = lib()
    if L.or_coef_f32(ctypes.byref(p.s), name.encode(), out.ctypes.data_as(_pf)) != 0:
        raise RuntimeError("oracle: " + L.or_error().decode())
    return out


def fom_grad(sc, probe, design_box, design_eps, steps: Optional[int] = None, precision: str = "f64",
             grad: bool = True, box_history: bool = False):
    """Figure of merit J = sum_m dt * Ez(probe)^2 over ``steps`` and, if ``grad``, the discrete-adjoint
    gradient dJ/deps_r of the design cells (array shaped like ``design_eps``). The design region
    ``design_box`` = (i0, j0, k0, i1, j1, k1) overrides the cells' eps_r with ``design_eps``.
    box_history (FP64 only): keep only the design region's field history (long runs, large grids;
    same result)."""
    steps = sc.steps if steps is None else steps
    p = _Prepared(sc, design=(design_box, design_eps))
    g = np.zeros(np.shape(design_eps), dtype=np.float64) if grad else None
    J = ctypes.c_double(0.0)
    L = lib()
    if box_history and precision != "f64":
        raise ValueError("box_history is an FP64 form")
    fn = L.or_fom_grad_box_f64 if box_history else L.or_fom_grad_f64 if precision == "f64" else L.or_fom_grad_f32
    rc = fn(ctypes.byref(p.s), steps, p.sig.ctypes.data_as(_pf), p.n_sig, int(probe[0]), int(probe[1]), int(probe[2]),
            ctypes.byref(J), None if g is None else g.ctypes.data_as(_pd))
    if rc != 0:
        raise RuntimeError("oracle: " + L.or_error().decode())
    return (J.value, g) if grad else J.value


def port_probes(voltage_box: Sequence[int], current_box: Sequence[int], current_axis: int = 2,
                voltage_axis: int = 2) -> list:
    """Point probes (component, i, j, k) a port samples, in the order or_port_vi reads them: Ez of the
    voltage box (k outer, j, i; half-open along ``voltage_axis``, closed across it, as voltMgpu's
    directions sum them, fdtdrav.h:2214-2290), then the four H groups of currMgpu's loop for
    ``current_axis`` (fdtdrav.h:2318-2480; i, j, k over the current box's ranges):
    x: Hy(ie-1, j, ks-1), Hz(ie-1, je, k), Hy(ie-1, j, ke), Hz(ie-1, js-1, k);
    y: Hz(is-1, je-1, k), Hx(i, je-1, ke), Hz(ie, je-1, k), Hx(i, je-1, ks-1);
    z: Hy(ie, j, ke-1), Hx(i, js-1, ke-1), Hy(is-1, j, ke-1), Hx(i, je, ke-1)."""
    from fdtd_gb300 import scenario as S
    v, c = [int(x) for x in voltage_box], [int(x) for x in current_box]
    end = [v[3] + (voltage_axis != 0), v[4] + (voltage_axis != 1), v[5] + (voltage_axis != 2)]
    out = [S.Probe(S.EZ, i, j, k) for k in range(v[2], end[2]) for j in range(v[1], end[1])
           for i in range(v[0], end[0])]
    I, J, K = range(c[0], c[3] + 1), range(c[1], c[4] + 1), range(c[2], c[5] + 1)
    if current_axis == 0:
        out += [S.Probe(S.HY, c[3] - 1, j, c[2] - 1) for j in J] + [S.Probe(S.HZ, c[3] - 1, c[4], k) for k in K]
        out += [S.Probe(S.HY, c[3] - 1, j, c[5]) for j in J] + [S.Probe(S.HZ, c[3] - 1, c[1] - 1, k) for k in K]
    elif current_axis == 1:
        out += [S.Probe(S.HZ, c[0] - 1, c[4] - 1, k) for k in K] + [S.Probe(S.HX, i, c[4] - 1, c[5]) for i in I]
        out += [S.Probe(S.HZ, c[3], c[4] - 1, k) for k in K] + [S.Probe(S.HX, i, c[4] - 1, c[2] - 1) for i in I]
    else:
        kc = c[5] - 1
        out += [S.Probe(S.HY, c[3], j, kc) for j in J] + [S.Probe(S.HX, i, c[1] - 1, kc) for i in I]
        out += [S.Probe(S.HY, c[0] - 1, j, kc) for j in J] + [S.Probe(S.HX, i, c[4], kc) for i in I]
    return out


def port_vi(series: np.ndarray, voltage_box: Sequence[int], current_box: Sequence[int], sc, col0: int = 0,
            time_average: bool = True, current_axis: int = 2, voltage_axis: int = 2):
    """(V(t), I(t)) float32 of a port from probe series (steps, n) whose columns from ``col0`` are
    ``port_probes(voltage_box, current_box, current_axis, voltage_axis)``."""
    a = np.ascontiguousarray(series, dtype=np.float32)
    steps, stride = a.shape
    vb = np.ascontiguousarray(voltage_box, dtype=np.int32)
    cb = np.ascontiguousarray(current_box, dtype=np.int32)
    V = np.zeros(steps, dtype=np.float32)
    I = np.zeros(steps, dtype=np.float32)
    L = lib()
    if L.or_port_vi(a.ctypes.data_as(_pf), steps, stride, col0, vb.ctypes.data_as(_pi), cb.ctypes.data_as(_pi),
                    current_axis, voltage_axis, sc.dx, sc.dy, sc.dz, int(time_average), V.ctypes.data_as(_pf),
                    I.ctypes.data_as(_pf)) != 0:
        raise RuntimeError("oracle: " + L.or_error().decode())
    return V, I


def port_spectra(V: np.ndarray, I: np.ndarray, z0: complex = 50.0) -> dict:
    """FP64 restatement of calc_otm + c_zinS11 (fdtdrav.h:2988-3051, 2510-2548): unnormalised real
    FFTs of V and the time-averaged I (n // 2 + 1 bins), a = (V + z0 I) / (2 sqrt(Re z0)),
    b = (V - z0 I) / (2 sqrt(Re z0)), s11 = b / a, zin = z0 (1 + s11) / (1 - s11)."""
    z0 = complex(z0)
    Vf = np.fft.rfft(np.asarray(V, dtype=np.float64))
    If = np.fft.rfft(np.asarray(I, dtype=np.float64))
    return dict(v=Vf, i=If, **zin_s11(Vf, If, z0))


def zin_s11(Vf: np.ndarray, If: np.ndarray, z0: complex = 50.0) -> dict:
    """The per-bin part of port_spectra in complex128."""
    z0 = complex(z0)
    scale = 2.0 * np.sqrt(z0.real)
    a = (Vf + z0 * If) / scale
    b = (Vf - z0 * If) / scale
    s11 = b / a
    return {"a": a, "b": b, "s11": s11, "zin": z0 * (1 + s11) / (1 - s11)}
