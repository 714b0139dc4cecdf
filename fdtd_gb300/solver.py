"""Python host API over the C ABI of libfdtd_gb300.so (include/fdtd_api.h).

This mirrors the setup-and-run sequence of the reference's marchingLoop (fdtdrav.h:3425-4387):
materials and bricks (setBrick), lumped sources and resistors (defineSourceZ / defineResistor),
probes (sampleField), then the time loop (solver). All compute runs in the CUDA library; there is no
CPU fallback: constructing a Simulation without the built library or without a GPU raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import Iterable, Optional, Sequence

import numpy as np

from . import scenario as S

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfdtd_gb300.so")

FDTD_OK = 0
SCHEDULE_AUTO, SCHEDULE_TWO_PASS, SCHEDULE_FUSED, SCHEDULE_FUSED_CPML = 0, 1, 2, 3

_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_f = ctypes.c_float
_pf = ctypes.POINTER(ctypes.c_float)
_pi32 = ctypes.POINTER(ctypes.c_int32)
_pu8 = ctypes.POINTER(ctypes.c_uint8)
_vp = ctypes.c_void_p


class Grid(ctypes.Structure):
    _fields_ = [("nx", _i32), ("ny", _i32), ("nz", _i32),
                ("dx", _f), ("dy", _f), ("dz", _f), ("dt", _f),
                ("eps0", _f), ("mu0", _f), ("pi", _f), ("pml", _i32 * 6)]


class Material(ctypes.Structure):
    _fields_ = [("eps_r", _f), ("sigma_e", _f), ("mu_r", _f), ("sigma_m", _f)]


class MaterialAxes(ctypes.Structure):
    _fields_ = [("eps_r", _f * 3), ("sigma_e", _f * 3), ("mu_r", _f * 3), ("sigma_m", _f * 3)]


class FDTDError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"fdtd error {code}: {msg}")
        self.code = code


# Every exported symbol of include/fdtd_api.h with its ctypes signature.
SIGNATURES = {
    "fdtd_last_error": (ctypes.c_char_p, []),
    "fdtd_version": (ctypes.c_char_p, []),
    "fdtd_create": (ctypes.c_int, [ctypes.POINTER(Grid), ctypes.POINTER(_vp)]),
    "fdtd_destroy": (ctypes.c_int, [_vp]),
    "fdtd_set_stream": (ctypes.c_int, [_vp, _vp]),
    "fdtd_set_schedule": (ctypes.c_int, [_vp, _i32]),
    "fdtd_set_materials": (ctypes.c_int, [_vp, ctypes.POINTER(Material), _i32]),
    "fdtd_set_materials_axes": (ctypes.c_int, [_vp, ctypes.POINTER(MaterialAxes), _i32]),
    "fdtd_set_material_index": (ctypes.c_int, [_vp, _pu8]),
    "fdtd_add_brick": (ctypes.c_int, [_vp, _pi32, _i32]),
    "fdtd_add_lumped_source": (ctypes.c_int, [_vp, _i32, _pi32, _f, _pf, _i64, _pi32]),
    "fdtd_add_resistor": (ctypes.c_int, [_vp, _i32, _pi32, _f]),
    "fdtd_add_probe": (ctypes.c_int, [_vp, _i32, _i32, _i32, _i32, _pi32]),
    "fdtd_set_probe_capacity": (ctypes.c_int, [_vp, _i64]),
    "fdtd_prepare": (ctypes.c_int, [_vp]),
    "fdtd_step": (ctypes.c_int, [_vp, _i64]),
    "fdtd_synchronize": (ctypes.c_int, [_vp]),
    "fdtd_current_step": (_i64, [_vp]),
    "fdtd_active_schedule": (_i32, [_vp]),
    "fdtd_tune_schedule": (ctypes.c_int, [_vp]),
    "fdtd_read_probes": (ctypes.c_int, [_vp, _i64, _i64, _pf]),
    "fdtd_probe_count": (_i32, [_vp]),
    "fdtd_get_field": (ctypes.c_int, [_vp, _i32, _pf]),
    "fdtd_set_field": (ctypes.c_int, [_vp, _i32, _pf]),
    "fdtd_get_field_device": (ctypes.c_int, [_vp, _i32, _vp]),
    "fdtd_set_field_device": (ctypes.c_int, [_vp, _i32, _vp]),
    "fdtd_state_bytes": (_i64, [_vp]),
    "fdtd_save_state": (ctypes.c_int, [_vp, _vp]),
    "fdtd_load_state": (ctypes.c_int, [_vp, _vp]),
    "fdtd_get_cpml_profile": (ctypes.c_int, [_vp, _i32, _i32, _pf]),
    "fdtd_set_cpml_grading": (ctypes.c_int, [_vp, ctypes.c_float]),
    "fdtd_device_bytes": (_i64, [_vp]),
    "fdtd_step_static_scratch": (ctypes.c_int, [_vp, _i64]),
    "fdtd_set_design_region": (ctypes.c_int, [_vp, _pi32, ctypes.POINTER(Material), _pf]),
    "fdtd_adjoint_forward": (ctypes.c_int, [_vp, _i64, _i32, _i32, _i32, _i32, ctypes.POINTER(ctypes.c_double)]),
    "fdtd_adjoint_backward": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double)]),
    "fdtd_batch_adjoint": (ctypes.c_int, [ctypes.POINTER(_vp), _i32, _i64, _i32, _pi32, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]),
    "fdtd_add_plate": (ctypes.c_int, [_vp, _i32, _pi32, ctypes.c_float, ctypes.c_float]),
    "fdtd_add_sector": (ctypes.c_int, [_vp, _pi32, _i32, ctypes.c_float, _i32, _i32, ctypes.c_float, ctypes.c_float]),
    "fdtd_add_port": (ctypes.c_int, [_vp, _i32, _pi32, _i32, _pi32, _pi32]),
    "fdtd_read_port": (ctypes.c_int, [_vp, _i32, _i64, _i64, _i32, _pf, _pf]),
    "fdtd_port_spectrum": (ctypes.c_int, [_vp, _i32, _i64, _i64, ctypes.c_float, ctypes.c_float, _pf, _pf, _pf, _pf]),
    "fdtd_port_zin": (ctypes.c_int, [_i64, _pf, _pf, ctypes.c_float, ctypes.c_float, _pf, _pf]),
    "fdtd_source_waveform": (ctypes.c_int, [_i32, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                            ctypes.c_float, ctypes.c_float, _i64, _pf]),
    "fdtd_marching_loop": (ctypes.c_int, [{"i": ctypes.c_int, "f": ctypes.c_float, "a": _pf}[k]
                                          for _, k in S.MARCHING_PARAMS] + [_pf, _pf]),
    "fdtd_batch_create": (ctypes.c_int, [ctypes.POINTER(_vp), _i32, ctypes.POINTER(_vp)]),
    "fdtd_batch_destroy": (ctypes.c_int, [_vp]),
    "fdtd_batch_set_stream": (ctypes.c_int, [_vp, _vp]),
    "fdtd_batch_set_config": (ctypes.c_int, [_vp, _i32, _i32]),
    "fdtd_batch_get_config": (ctypes.c_int, [_vp, _pi32, _pi32, _pi32]),
    "fdtd_batch_tune": (ctypes.c_int, [_vp, _i64, ctypes.POINTER(ctypes.c_double)]),
    "fdtd_batch_step": (ctypes.c_int, [_vp, _i64]),
    "fdtd_batch_synchronize": (ctypes.c_int, [_vp]),
}

_lib = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libfdtd_gb300.so and declare its C ABI. Raises if the library was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m fdtd_gb300.build` "
                           "(the solver has no CPU fallback)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(rc: int) -> None:
    if rc != FDTD_OK:
        raise FDTDError(rc, _lib.fdtd_last_error().decode())


def _box(box: Sequence[int]):
    return (_i32 * 6)(*[int(v) for v in box])


class Simulation:
    """One simulation handle on the current CUDA device."""

    def __init__(self, nx: int, ny: int, nz: int, dx: float, dy: float, dz: float, dt: float,
                 pml: Sequence[int] = (10,) * 6, eps0: float = float(S.REF_EPS0), mu0: float = float(S.REF_MU0),
                 pi: float = float(S.REF_PI), schedule: int = SCHEDULE_AUTO):
        lib = load_library()
        g = Grid()
        g.nx, g.ny, g.nz = nx, ny, nz
        g.dx, g.dy, g.dz, g.dt = dx, dy, dz, dt
        g.eps0, g.mu0, g.pi = eps0, mu0, pi
        for q in range(6):
            g.pml[q] = int(pml[q])
        h = _vp()
        _check(lib.fdtd_create(ctypes.byref(g), ctypes.byref(h)))
        self._h = h
        self.shape = (nz, ny, nx)
        self.dt = float(np.float32(dt))
        self.n_probes = 0
        if schedule != SCHEDULE_AUTO:
            _check(lib.fdtd_set_schedule(self._h, schedule))

    # -- lifetime -------------------------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.fdtd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- setup ----------------------------------------------------------------------------------
    def set_stream(self, stream_ptr: int) -> None:
        _check(_lib.fdtd_set_stream(self._h, _vp(stream_ptr)))

    def set_schedule(self, schedule: int) -> None:
        _check(_lib.fdtd_set_schedule(self._h, schedule))

    def set_materials(self, table: np.ndarray) -> None:
        """Material table (n, 4): eps_r, sigma_e, mu_r, sigma_m; or (n, 3, 4) with those values per
        axis x, y, z (fdtd_set_materials_axes)."""
        t = np.asarray(table, dtype=np.float32)
        if t.ndim == 3:
            # MaterialAxes holds eps_r[3], sigma_e[3], mu_r[3], sigma_m[3]: the (n, 3, 4) table transposed
            rows = np.ascontiguousarray(t.transpose(0, 2, 1))
            arr = (MaterialAxes * len(rows)).from_buffer_copy(rows.tobytes())
            _check(_lib.fdtd_set_materials_axes(self._h, arr, len(rows)))
            return
        t = np.ascontiguousarray(t.reshape(-1, 4))  # rows laid out as Material (four floats)
        arr = (Material * len(t)).from_buffer_copy(t.tobytes())
        _check(_lib.fdtd_set_materials(self._h, arr, len(t)))

    def set_material_index(self, cells: np.ndarray) -> None:
        c = np.ascontiguousarray(cells, dtype=np.uint8)
        if c.shape != self.shape:
            raise ValueError(f"material index must have shape {self.shape}")
        _check(_lib.fdtd_set_material_index(self._h, c.ctypes.data_as(_pu8)))

    def add_brick(self, box: Sequence[int], material: int) -> None:
        _check(_lib.fdtd_add_brick(self._h, _box(box), material))

    def add_source(self, box: Sequence[int], resistance: float, voltage: np.ndarray, axis: int = 2) -> int:
        v = np.ascontiguousarray(voltage, dtype=np.float32)
        out = _i32()
        _check(_lib.fdtd_add_lumped_source(self._h, axis, _box(box), resistance, v.ctypes.data_as(_pf), v.size,
                                           ctypes.byref(out)))
        return out.value

    def add_resistor(self, box: Sequence[int], resistance: float, axis: int = 2) -> None:
        _check(_lib.fdtd_add_resistor(self._h, axis, _box(box), resistance))

    def add_probe(self, component: int, i: int, j: int, k: int) -> int:
        out = _i32()
        _check(_lib.fdtd_add_probe(self._h, component, i, j, k, ctypes.byref(out)))
        self.n_probes = out.value + 1
        return out.value

    def add_plate(self, normal_axis: int, box: Sequence[int], sigma_1: float, sigma_2: float) -> None:
        """Zero-thickness plate normal to ``normal_axis`` (fdtd_add_plate)."""
        _check(_lib.fdtd_add_plate(self._h, normal_axis, _box(box), sigma_1, sigma_2))

    def add_sector(self, tri: Sequence[int], pz0: int, radius: float, max_x: int, max_y: int, sigma_x: float,
                   sigma_y: float) -> None:
        """Zero-thickness sector plate in plane pz0 (fdtd_add_sector); tri = (px0, py0, px1, py1,
        px2, py2), apex (px1, py1)."""
        t = (ctypes.c_int32 * 6)(*[int(v) for v in tri])
        _check(_lib.fdtd_add_sector(self._h, t, pz0, radius, max_x, max_y, sigma_x, sigma_y))

    def add_port(self, voltage_box: Sequence[int], current_box: Sequence[int], current_axis: int = 2,
                 voltage_axis: int = 2) -> int:
        """A port (voltage along ``voltage_axis`` from the Ez samples of the box, current loop around
        ``current_axis``); returns its id."""
        pid = _i32(-1)
        _check(_lib.fdtd_add_port(self._h, voltage_axis, _box(voltage_box), current_axis, _box(current_box),
                                  ctypes.byref(pid)))
        self.n_probes = _lib.fdtd_probe_count(self._h)
        return pid.value

    def read_port(self, pid: int, first: int = 0, n: Optional[int] = None, time_average: bool = True):
        """(V(t), I(t)) float32 arrays of the port's steps [first, first + n); I(t) time-averaged
        over the window unless ``time_average`` is False."""
        n = self.current_step - first if n is None else n
        v = np.zeros(n, dtype=np.float32)
        i = np.zeros(n, dtype=np.float32)
        _check(_lib.fdtd_read_port(self._h, pid, first, n, int(time_average), v.ctypes.data_as(_pf),
                                   i.ctypes.data_as(_pf)))
        return v, i

    def port_spectrum(self, pid: int, z0: complex = 50.0, first: int = 0, n: Optional[int] = None) -> dict:
        """Spectra of a port over steps [first, first + n): complex64 arrays ``v``, ``i``, ``s11``,
        ``zin`` of n // 2 + 1 bins and ``freq`` (Hz, bin f at f / (n dt))."""
        n = self.current_step - first if n is None else n
        nf = n // 2 + 1
        out = {k: np.zeros(nf, dtype=np.complex64) for k in ("v", "i", "s11", "zin")}
        z = complex(z0)
        _check(_lib.fdtd_port_spectrum(self._h, pid, first, n, z.real, z.imag,
                                       *(out[k].ctypes.data_as(_pf) for k in ("v", "i", "s11", "zin"))))
        out["freq"] = np.arange(nf, dtype=np.float64) / (n * float(self.dt))
        return out

    def set_probe_capacity(self, steps: int) -> None:
        _check(_lib.fdtd_set_probe_capacity(self._h, steps))

    def prepare(self) -> None:
        _check(_lib.fdtd_prepare(self._h))

    # -- run ------------------------------------------------------------------------------------
    def step(self, n: int = 1) -> None:
        _check(_lib.fdtd_step(self._h, n))

    def step_static_scratch(self, n: int = 1) -> None:
        """n fused steps that allocate no device memory (the handle must be prepared; small grids)."""
        _check(_lib.fdtd_step_static_scratch(self._h, n))

    def synchronize(self) -> None:
        _check(_lib.fdtd_synchronize(self._h))

    @property
    def current_step(self) -> int:
        return _lib.fdtd_current_step(self._h)

    def tune_schedule(self) -> None:
        """Under SCHEDULE_AUTO, choose the schedule now by timing both (the handle's state is kept)."""
        _check(_lib.fdtd_tune_schedule(self._h))

    @property
    def active_schedule(self) -> int:
        """The schedule the next step runs (SCHEDULE_TWO_PASS or SCHEDULE_FUSED; AUTO resolved)."""
        return _lib.fdtd_active_schedule(self._h)

    def read_probes(self, first: int = 0, n: Optional[int] = None) -> np.ndarray:
        n = self.current_step - first if n is None else n
        out = np.zeros((n, max(self.n_probes, 1)), dtype=np.float32)
        _check(_lib.fdtd_read_probes(self._h, first, n, out.ctypes.data_as(_pf)))
        return out[:, :self.n_probes]

    def get_field(self, component: int) -> np.ndarray:
        out = np.empty(self.shape, dtype=np.float32)
        _check(_lib.fdtd_get_field(self._h, component, out.ctypes.data_as(_pf)))
        return out

    def set_field(self, component: int, values: np.ndarray) -> None:
        v = np.ascontiguousarray(values, dtype=np.float32).reshape(self.shape)
        _check(_lib.fdtd_set_field(self._h, component, v.ctypes.data_as(_pf)))

    def fields(self) -> np.ndarray:
        return np.stack([self.get_field(c) for c in range(6)])

    def get_field_device(self, component: int, dev_ptr: int) -> None:
        _check(_lib.fdtd_get_field_device(self._h, component, _vp(dev_ptr)))

    def set_field_device(self, component: int, dev_ptr: int) -> None:
        _check(_lib.fdtd_set_field_device(self._h, component, _vp(dev_ptr)))

    def state_bytes(self) -> int:
        return _lib.fdtd_state_bytes(self._h)

    def save_state(self, dev_ptr: int) -> None:
        _check(_lib.fdtd_save_state(self._h, _vp(dev_ptr)))

    def load_state(self, dev_ptr: int) -> None:
        _check(_lib.fdtd_load_state(self._h, _vp(dev_ptr)))

    def set_cpml_grading(self, r0: float = 0.0) -> None:
        """0: the reference's sigma_opt grading (default); 0 < r0 < 1: sigma_max per slab from the
        reflection coefficient r0 (fdtd_set_cpml_grading)."""
        _check(_lib.fdtd_set_cpml_grading(self._h, float(r0)))

    def cpml_profile(self, axis: int, kind: int) -> np.ndarray:
        """1-D CPML profile: kind 0 b_e, 1 a_e, 2 b_m, 3 a_m, 4 kappa_e, 5 kappa_m."""
        n = (self.shape[2], self.shape[1], self.shape[0])[axis]
        out = np.empty(n, dtype=np.float32)
        _check(_lib.fdtd_get_cpml_profile(self._h, axis, kind, out.ctypes.data_as(_pf)))
        return out

    def cpml_profiles(self) -> dict:
        """All 18 profiles keyed like the oracle's override names (b_ex, a_ex, b_mx, a_mx, k_ex, k_mx, ...)."""
        out = {}
        for a, ax in enumerate("xyz"):
            for kind, nm in enumerate(("b_e", "a_e", "b_m", "a_m", "k_e", "k_m")):
                out[nm + ax] = self.cpml_profile(a, kind)
        return out

    def device_bytes(self) -> int:
        return _lib.fdtd_device_bytes(self._h)

    # -- design region and adjoint ---------------------------------------------------------------
    def set_design_region(self, box: Sequence[int], eps_r: np.ndarray, sigma_e: float = float(S.REF_TINY),
                          mu_r: float = 1.0, sigma_m: float = float(S.REF_TINY)) -> None:
        """Design cells ``box`` = (i0, j0, k0, i1, j1, k1) with per-cell eps_r (shape (k1-k0, j1-j0, i1-i0))."""
        e = np.ascontiguousarray(eps_r, dtype=np.float32)
        want = (box[5] - box[2], box[4] - box[1], box[3] - box[0])
        if e.shape != want:
            raise ValueError(f"eps_r shape {e.shape} != design box shape {want}")
        base = Material(1.0, sigma_e, mu_r, sigma_m)
        _check(_lib.fdtd_set_design_region(self._h, _box(box), ctypes.byref(base), e.ctypes.data_as(_pf)))
        self._design_shape = want

    def adjoint_forward(self, steps: int, probe: Sequence[int], checkpoint_every: int = 64) -> float:
        """J = sum_m dt * Ez(probe)^2 over ``steps`` steps, recording for adjoint_backward."""
        J = ctypes.c_double(0.0)
        _check(_lib.fdtd_adjoint_forward(self._h, steps, checkpoint_every, int(probe[0]), int(probe[1]), int(probe[2]),
                                         ctypes.byref(J)))
        return J.value

    def adjoint_backward(self) -> np.ndarray:
        """dJ/deps_r of the design cells (float64, shaped like the design eps_r)."""
        g = np.zeros(self._design_shape, dtype=np.float64)
        _check(_lib.fdtd_adjoint_backward(self._h, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return g

    # -- scenarios ------------------------------------------------------------------------------
    @classmethod
    def from_scenario(cls, sc: "S.Scenario", schedule: int = SCHEDULE_AUTO, material_index: Optional[np.ndarray] = None,
                      probe_capacity: Optional[int] = None) -> "Simulation":
        """Build a simulation from a scenario in the reference's setup order (fdtdrav.h:4104-4310)."""
        sim = cls(sc.nx, sc.ny, sc.nz, sc.dx, sc.dy, sc.dz, sc.dt, sc.pml, sc.eps0, sc.mu0, sc.pi, schedule)
        if getattr(sc, "cpml_r0", 0.0):
            sim.set_cpml_grading(sc.cpml_r0)
        sim.set_materials(sc.material_table_axes() if sc.anisotropic else sc.material_table())
        if material_index is not None:
            sim.set_material_index(material_index)
        else:
            for b in sc.bricks:
                sim.add_brick(b.box, b.material)
        for s in sc.sources:
            sim.add_source(s.box, s.resistance, s.waveform)
        for s in getattr(sc, "x_sources", []):
            sim.add_source(s.box, s.resistance, np.zeros(0, np.float32), axis=0)
        for r in sc.resistors:
            sim.add_resistor(r.box, r.resistance)
        for q in sc.plates:
            sim.add_plate(q.axis, q.box, q.sigma_1, q.sigma_2)
        for p in sc.probes:
            sim.add_probe(p.component, p.i, p.j, p.k)
        if probe_capacity is not None:
            sim.set_probe_capacity(probe_capacity)
        return sim


def source_waveform(type_: int, amp: float, freq: float, dt: float, t_0: float, tau: float, pi: float, n: int):
    """setGauss (type 1) / setSine (type 3) voltage waveform of n steps, float32 (fdtd_source_waveform)."""
    out = np.zeros(n, dtype=np.float32)
    _check(load_library().fdtd_source_waveform(type_, amp, freq, dt, t_0, tau, pi, n, out.ctypes.data_as(_pf)))
    return out


def marching_loop(params: dict):
    """The reference's whole run (fdtd_marching_loop) for marchingLoop's parameters ``params`` (the
    names of scenario.MARCHING_PARAMS): returns (V(t), I(t)) float32."""
    lib = load_library()
    keep, args = [], []
    for name, kind in S.MARCHING_PARAMS:
        v = params[name]
        if kind == "a":
            arr = np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(-1))
            keep.append(arr)
            args.append(arr.ctypes.data_as(_pf))
        else:
            args.append(v)
    n = int(params["n_t_steps"])
    V = np.zeros(n, dtype=np.float32)
    I = np.zeros(n, dtype=np.float32)
    _check(lib.fdtd_marching_loop(*args, V.ctypes.data_as(_pf), I.ctypes.data_as(_pf)))
    return V, I


def port_zin(v_spectrum: np.ndarray, i_spectrum: np.ndarray, z0: complex = 50.0):
    """s11 and zin (complex64) of given V and I spectra for reference impedance z0 (fdtd_port_zin)."""
    v = np.ascontiguousarray(v_spectrum, dtype=np.complex64)
    i = np.ascontiguousarray(i_spectrum, dtype=np.complex64)
    if v.shape != i.shape or v.ndim != 1:
        raise ValueError("spectra must be 1-D arrays of equal length")
    s11 = np.zeros_like(v)
    zin = np.zeros_like(v)
    z = complex(z0)
    _check(load_library().fdtd_port_zin(v.size, v.ctypes.data_as(_pf), i.ctypes.data_as(_pf), z.real, z.imag,
                                        s11.ctypes.data_as(_pf), zin.ctypes.data_as(_pf)))
    return s11, zin


class Batch:
    """Many simulations advanced together by one persistent launch per step call (fdtd_batch_*).
    The simulations stay usable on their own (fields, probes, state); the batch only refers to them."""

    def __init__(self, sims: Sequence[Simulation]):
        self._sims = list(sims)
        arr = (_vp * len(self._sims))(*[s.handle for s in self._sims])
        h = _vp()
        _check(_lib.fdtd_batch_create(arr, len(self._sims), ctypes.byref(h)))
        self._b = h

    def close(self) -> None:
        if getattr(self, "_b", None):
            _lib.fdtd_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_ptr: int) -> None:
        _check(_lib.fdtd_batch_set_stream(self._b, _vp(stream_ptr)))

    def set_config(self, cluster: int, threads: int) -> None:
        _check(_lib.fdtd_batch_set_config(self._b, cluster, threads))

    @property
    def config(self) -> dict:
        c, t, n = _i32(), _i32(), _i32()
        _check(_lib.fdtd_batch_get_config(self._b, ctypes.byref(c), ctypes.byref(t), ctypes.byref(n)))
        return {"cluster": c.value, "threads": t.value, "n_clusters": n.value}

    def tune(self, steps: int = 10) -> float:
        """Autotune the form (flat, or persistent with its cluster and CTA size) on `steps` steps
        (states restored); returns the best time."""
        ms = ctypes.c_double(0.0)
        _check(_lib.fdtd_batch_tune(self._b, steps, ctypes.byref(ms)))
        return ms.value

    def step(self, n: int = 1) -> None:
        _check(_lib.fdtd_batch_step(self._b, n))

    def synchronize(self) -> None:
        _check(_lib.fdtd_batch_synchronize(self._b))


def batch_adjoint(sims: Sequence[Simulation], steps: int, probes: Sequence[Sequence[int]], checkpoint_every: int = 64):
    """adjoint_forward then adjoint_backward of every simulation (each with its design region),
    all enqueued before any is waited for (fdtd_batch_adjoint). Returns (J list, gradient list);
    they equal the per-simulation calls bit for bit. Give the simulations separate streams
    (set_stream) to run them concurrently."""
    sims = list(sims)
    if len(probes) != len(sims):
        raise ValueError("one probe per simulation")
    n = len(sims)
    handles = (_vp * n)(*[s.handle for s in sims])
    pr = (_i32 * (3 * n))(*[int(v) for p in probes for v in p])
    J = (ctypes.c_double * n)()
    grads = [np.zeros(getattr(s, "_design_shape", (0,)), dtype=np.float64) for s in sims]
    gp = (ctypes.POINTER(ctypes.c_double) * n)(*[g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for g in grads])
    _check(_lib.fdtd_batch_adjoint(handles, n, steps, checkpoint_every, pr, J, gp))
    return list(J), grads


def run_scenario(sc: "S.Scenario", steps: Optional[int] = None, schedule: int = SCHEDULE_AUTO,
                 fields: bool = True):
    """Run a scenario on the GPU; returns (probes (steps, n_probes), fields (6, nz, ny, nx) or None)."""
    steps = sc.steps if steps is None else steps
    with Simulation.from_scenario(sc, schedule, probe_capacity=max(steps, 1)) as sim:
        sim.step(steps)
        sim.synchronize()
        p = sim.read_probes(0, steps)
        f = sim.fields() if fields else None
    return p, f
