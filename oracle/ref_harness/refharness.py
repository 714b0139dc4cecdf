"""Python driver for the reference-kernel harness (test infrastructure only).

Runs the reference's own setup kernels and calc_e / calc_h (fdtdrav.h, compiled unmodified except
for its barrier calls, see ref_kernels.cu) on a single slab through ``librefharness.so``. Used to
generate golden fixtures, to compare coefficient arrays and single steps, and as the timed
reference arm of the benchmark. Never imported by the product package.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(os.path.dirname(HERE), "_ref")
CUBIN = os.path.join(REF_DIR, "fdtdrav_sm103a.cubin")
RUNNER = os.path.join(REF_DIR, "librefharness.so")

_i = ctypes.c_int
_f = ctypes.c_float
_pi = ctypes.POINTER(ctypes.c_int)
_pf = ctypes.POINTER(ctypes.c_float)


class _Scenario(ctypes.Structure):
    _fields_ = [("nxx", _i), ("nyy", _i), ("nz", _i), ("pml", _i * 6),
                ("dx", _f), ("dy", _f), ("dz", _f), ("dt", _f), ("eps0", _f), ("pi", _f), ("mu0", _f),
                ("nbricks", _i), ("brick_box", _pi), ("brick_mat", _pf),
                ("nsources", _i), ("src_box", _pi), ("src_r", _pf),
                ("nres", _i), ("res_box", _pi), ("res_r", _pf),
                ("nplates", _i), ("plate", _pi), ("plate_sig", _pf),
                ("nsrcx", _i), ("srcx_box", _pi), ("srcx_r", _pf)]


def available() -> bool:
    return os.path.exists(CUBIN) and os.path.exists(RUNNER)


class RefHarness:
    """One reference simulation on the current GPU (single slab, NUMDEV = 1)."""

    def __init__(self, cubin: str = CUBIN, runner: str = RUNNER):
        if not os.path.exists(cubin):
            raise FileNotFoundError(f"reference cubin missing: {cubin}")
        self.lib = ctypes.CDLL(runner)
        L = self.lib
        L.rh_error.restype = ctypes.c_char_p
        L.rh_load.argtypes = [ctypes.c_char_p]
        L.rh_setup.argtypes = [ctypes.POINTER(_Scenario)]
        L.rh_get.argtypes = [ctypes.c_char_p, _pf, ctypes.c_longlong]
        L.rh_set.argtypes = [ctypes.c_char_p, _pf]
        L.rh_calc_e.argtypes = [_i, _i, _pf, ctypes.c_longlong]
        L.rh_calc_h.argtypes = [_i]
        L.rh_run.argtypes = [_i, _i, _i, _pf, ctypes.c_longlong, _i, _pi, _pi, _pi, _pi, _pf, _pf]
        L.rh_set_port.argtypes = [_pi, _pi, _i]
        L.rh_port_reduce.argtypes = [_i, _i, _pf, _pf, _pf]
        L.rh_port_reduce_dir.argtypes = [_i, _i, _i, _pf, _pf, _pf]
        L.rh_sector.argtypes = [_pi, _i, _f, _i, _i, _f, _f]
        L.rh_zin.argtypes = [_i, _pf, _pf, _f, _f, _pf, _pf]
        L.rh_waveform.argtypes = [_i, _f, _i, _f, _f, _f, _f, _f, _i, _pf, _pf]
        self._check(L.rh_load(cubin.encode()))
        self.sc = None

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("reference harness: " + self.lib.rh_error().decode())

    def setup(self, sc) -> None:
        """Run the reference setup sequence for a ``fdtd_gb300.scenario.Scenario``."""
        self.sc = sc
        s = _Scenario()
        s.nxx, s.nyy, s.nz = sc.nx, sc.ny, sc.nz
        for q in range(6):
            s.pml[q] = sc.pml[q]
        s.dx, s.dy, s.dz, s.dt = sc.dx, sc.dy, sc.dz, sc.dt
        s.eps0, s.pi, s.mu0 = sc.eps0, sc.pi, sc.mu0
        tab = sc.material_table_axes()
        bb = np.array([b.box for b in sc.bricks], dtype=np.int32).reshape(-1, 6)
        bm = np.array([tab[b.material] for b in sc.bricks], dtype=np.float32).reshape(-1, 12)
        sb = np.array([x.box for x in sc.sources], dtype=np.int32).reshape(-1, 6)
        sr = np.array([x.resistance for x in sc.sources], dtype=np.float32)
        rb = np.array([x.box for x in sc.resistors], dtype=np.int32).reshape(-1, 6)
        rr = np.array([x.resistance for x in sc.resistors], dtype=np.float32)
        plates = getattr(sc, "plates", [])
        pl = np.array([[q.axis, *q.box] for q in plates], dtype=np.int32).reshape(-1, 7)
        ps = np.array([[q.sigma_1, q.sigma_2] for q in plates], dtype=np.float32).reshape(-1, 2)
        xs = getattr(sc, "x_sources", [])
        xb = np.array([x.box for x in xs], dtype=np.int32).reshape(-1, 6)
        xr = np.array([x.resistance for x in xs], dtype=np.float32)
        self._keep = [np.ascontiguousarray(a) for a in (bb, bm, sb, sr, rb, rr, pl, ps, xb, xr)]
        bb, bm, sb, sr, rb, rr, pl, ps, xb, xr = self._keep
        s.nsrcx, s.srcx_box, s.srcx_r = len(xs), xb.ctypes.data_as(_pi), xr.ctypes.data_as(_pf)
        s.nplates, s.plate, s.plate_sig = len(plates), pl.ctypes.data_as(_pi), ps.ctypes.data_as(_pf)
        s.nbricks, s.brick_box, s.brick_mat = len(sc.bricks), bb.ctypes.data_as(_pi), bm.ctypes.data_as(_pf)
        s.nsources, s.src_box, s.src_r = len(sc.sources), sb.ctypes.data_as(_pi), sr.ctypes.data_as(_pf)
        s.nres, s.res_box, s.res_r = len(sc.resistors), rb.ctypes.data_as(_pi), rr.ctypes.data_as(_pf)
        self._check(self.lib.rh_setup(ctypes.byref(s)))

    def get(self, name: str, length: Optional[int] = None) -> np.ndarray:
        """A reference array: volume arrays come back as (nz, ny, nx) float32, 1-D arrays as ``length``."""
        if length is None:
            out = np.empty((self.sc.nz, self.sc.ny, self.sc.nx), dtype=np.float32)
            n = out.size
        else:
            out = np.empty(length, dtype=np.float32)
            n = length
        self._check(self.lib.rh_get(name.encode(), out.ctypes.data_as(_pf), n))
        return out

    def set(self, name: str, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float32).reshape(self.sc.nz, self.sc.ny, self.sc.nx)
        self._check(self.lib.rh_set(name.encode(), a.ctypes.data_as(_pf)))

    def calc_e(self, m: int, src_slot: int = -1, signal: Optional[np.ndarray] = None) -> None:
        sig = None if signal is None else np.ascontiguousarray(signal, dtype=np.float32)
        self._check(self.lib.rh_calc_e(m, src_slot, None if sig is None else sig.ctypes.data_as(_pf),
                                       0 if sig is None else sig.size))

    def calc_h(self, m: int) -> None:
        self._check(self.lib.rh_calc_h(m))

    def run(self, steps: int, m0: int = 0, src_slot: int = -1, signal: Optional[np.ndarray] = None,
            probes: Sequence = ()) -> tuple:
        """Run ``steps`` reference steps; returns (probe array (steps, n_probes), elapsed ms)."""
        sig = None if signal is None else np.ascontiguousarray(signal, dtype=np.float32)
        n = len(probes)
        pc = np.array([p.component for p in probes], dtype=np.int32)
        pi = np.array([p.i for p in probes], dtype=np.int32)
        pj = np.array([p.j for p in probes], dtype=np.int32)
        pk = np.array([p.k for p in probes], dtype=np.int32)
        out = np.zeros((steps, max(n, 1)), dtype=np.float32)
        ms = _f(0.0)
        self._check(self.lib.rh_run(m0, steps, src_slot,
                                    None if sig is None else sig.ctypes.data_as(_pf), 0 if sig is None else sig.size,
                                    n, pc.ctypes.data_as(_pi), pi.ctypes.data_as(_pi), pj.ctypes.data_as(_pi),
                                    pk.ctypes.data_as(_pi), out.ctypes.data_as(_pf), ctypes.byref(ms)))
        return out[:, :n], ms.value

    def set_port(self, voltage_box: Sequence[int], current_box: Sequence[int], steps: int) -> None:
        """Place the reference's own z-directed voltage / current sample boxes for a run of
        ``steps`` steps from m = 0 (after ``setup``, before ``run``)."""
        v = np.ascontiguousarray(voltage_box, dtype=np.int32)
        c = np.ascontiguousarray(current_box, dtype=np.int32)
        self._check(self.lib.rh_set_port(v.ctypes.data_as(_pi), c.ctypes.data_as(_pi), steps))

    def port_reduce(self, steps: int, current_direction: int = 3, voltage_direction: int = 3) -> tuple:
        """The reference's voltMgpu / currMgpu / correcI on its samples: (V, I before correcI,
        I after correcI), float32 arrays of ``steps``; directions 1 / 2 / 3 = x / y / z."""
        out = [np.zeros(steps, dtype=np.float32) for _ in range(3)]
        self._check(self.lib.rh_port_reduce_dir(steps, voltage_direction, current_direction,
                                                *(o.ctypes.data_as(_pf) for o in out)))
        return tuple(out)

    def sector(self, tri, pz0: int, radius: float, max_x: int, max_y: int, sigma_x: float, sigma_y: float) -> None:
        """The reference's defineSec on the set-up grid's sigma_e_x / sigma_e_y (read them with get)."""
        t = np.ascontiguousarray(tri, dtype=np.int32)
        self._check(self.lib.rh_sector(t.ctypes.data_as(_pi), pz0, radius, max_x, max_y, sigma_x, sigma_y))

    def zin(self, n_t_steps: int, V: np.ndarray, I: np.ndarray, z0: complex) -> tuple:
        """The reference's c_zinS11 on spectra V, I (complex64, n_t_steps // 2 + 1 bins)."""
        nf = n_t_steps // 2 + 1
        v = np.ascontiguousarray(V, dtype=np.complex64)
        i = np.ascontiguousarray(I, dtype=np.complex64)
        assert v.size == nf and i.size == nf
        s11 = np.zeros(nf, dtype=np.complex64)
        zin = np.zeros(nf, dtype=np.complex64)
        self._check(self.lib.rh_zin(n_t_steps, v.ctypes.data_as(_pf), i.ctypes.data_as(_pf),
                                    complex(z0).real, complex(z0).imag, s11.ctypes.data_as(_pf),
                                    zin.ctypes.data_as(_pf)))
        return s11, zin

    def waveform(self, type_: int, amp: float, v_mag_factor: int, freq: float, dt: float, t_0: float, tau: float,
                 pi: float, n: int) -> tuple:
        """The reference's setGauss (type 1) / setSine (type 3): (signal, signal per node) float32."""
        sig = np.zeros(n, dtype=np.float32)
        per = np.zeros(n, dtype=np.float32)
        self._check(self.lib.rh_waveform(type_, amp, v_mag_factor, freq, dt, t_0, tau, pi, n,
                                         sig.ctypes.data_as(_pf), per.ctypes.data_as(_pf)))
        return sig, per

    def fields(self) -> dict:
        return {n: self.get(n) for n in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")}

    def close(self) -> None:
        self.lib.rh_free()


def run_reference(sc, steps: Optional[int] = None, with_fields: bool = True):
    """Full reference run of a scenario. Several sources are run one at a time and summed
    (the reference's calc_e injects a single source box per launch, fdtdrav.h:726)."""
    steps = sc.steps if steps is None else steps
    h = RefHarness()
    try:
        if not sc.sources:
            h.setup(sc)
            probes, _ = h.run(steps, probes=sc.probes)
            return probes, (h.fields() if with_fields else None)
        tot_p, tot_f = None, None
        for s in range(len(sc.sources)):
            h.setup(sc)
            p, _ = h.run(steps, src_slot=s, signal=sc.signal_per_node(s), probes=sc.probes)
            f = h.fields() if with_fields else None
            if tot_p is None:
                tot_p, tot_f = p, f
            else:
                tot_p = tot_p + p
                if with_fields:
                    tot_f = {k: tot_f[k] + f[k] for k in tot_f}
        return tot_p, tot_f
    finally:
        h.close()
