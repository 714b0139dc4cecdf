"""Scenario description and seeded generators for the FDTD workloads.

A scenario is everything the reference's host driver ``marchingLoop`` (fdtdrav.h:3425) derives
before its time loop, expressed in index space:

* grid: node counts ``nx, ny, nz`` (the reference's NXX, NYY, NZ, fdtdrav.h:3487-3491), cell sizes,
  time step and the physical constants the reference passes around as floats (source.cu:30-46);
* CPML thickness per face (x_n, x_p, y_n, y_p, z_n, z_p);
* bricks: cell boxes ``[is,ie) x [js,je) x [ks,ke)`` painted with a material id, the last box
  painted wins (setBrick, fdtdrav.h:1524-1571, applied in order at fdtdrav.h:4104-4128);
* lumped z-directed sources ``i in [is,ie], j in [js,je], k in [ks,ke)`` with a resistance and a
  voltage waveform (defineSourceZ fdtdrav.h:1368-1426, injection fdtdrav.h:726-733) and
  resistors (defineResistor fdtdrav.h:1429-1483);
* point probes (component, i, j, k), the point form of sampleField (fdtdrav.h:234-246).

The generators reproduce the workload shapes used for parity and benchmarking: a vacuum cube
with one Gaussian-derivative source (64^3), seeded random dielectric boxes with several delayed
sources (512^3 and its scaled-down forms), and the HBM-sized 1024x1024x896 domain.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence, Tuple, Union

import numpy as np

# Components, in the order the C ABI numbers them.
EX, EY, EZ, HX, HY, HZ = range(6)
COMPONENT_NAMES = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")

# Constants exactly as the reference's main() builds them in float (source.cu:30-33).
REF_EPS0 = np.float32(8.854187817e-12)
REF_PI = np.float32(3.1415)
REF_MU0 = np.float32(np.float64(np.float32(4.0) * REF_PI) * 1e-7)
# Background cells hold eps_r = mu_r = 1 and conductivities 1.2e-38 (setZero, fdtdrav.h:939-962).
REF_TINY = np.float32(1.2e-38)


def ref_light_speed(eps0=REF_EPS0, mu0=REF_MU0) -> np.float32:
    """c = 1 / sqrt(mu0 * eps0) in float (source.cu:33)."""
    return np.float32(np.float32(1.0) / np.sqrt(np.float32(np.float32(mu0) * np.float32(eps0))))


def courant_dt(dx, dy, dz, courant=1.0, eps0=REF_EPS0, mu0=REF_MU0) -> np.float32:
    """Time step of source.cu:45-46: 1/(c*sqrt(1/dx^2+1/dy^2+1/dz^2)) times the Courant factor.

    The reference evaluates the sum with double-precision pow and stores the result in a float.
    """
    c = float(ref_light_speed(eps0, mu0))
    dx, dy, dz = float(np.float32(dx)), float(np.float32(dy)), float(np.float32(dz))
    dt = np.float32(1.0 / (np.float32(c) * math.sqrt(1.0 / dx ** 2 + 1.0 / dy ** 2 + 1.0 / dz ** 2)))
    return np.float32(np.float32(courant) * dt)


def calc_index(coordinate: float, delta: float) -> int:
    """Metre -> node index, ``(int)round(coordinate / delta)`` in float (calc_index, fdtdrav.h:198-206)."""
    q = np.float32(np.float32(coordinate) / np.float32(delta))
    # C round(): half away from zero
    return int(math.floor(abs(float(q)) + 0.5)) * (1 if q >= 0 else -1)


@dataclasses.dataclass
class Material:
    """A brick material. Each property is one value (isotropic) or three (x, y, z): setBrick takes
    the eps_r, sigma_e, mu_r and sigma_m of each axis separately (fdtdrav.h:1524-1531), and each
    field component averages its own axis' values (setSigmaEpsSigmaMu, fdtdrav.h:1097-1220)."""
    eps_r: Union[float, Sequence[float]] = 1.0
    sigma_e: Union[float, Sequence[float]] = float(REF_TINY)
    mu_r: Union[float, Sequence[float]] = 1.0
    sigma_m: Union[float, Sequence[float]] = float(REF_TINY)

    def axes(self) -> np.ndarray:
        """float32 (3, 4): per axis x, y, z the values eps_r, sigma_e, mu_r, sigma_m."""
        vals = (self.eps_r, self.sigma_e, self.mu_r, self.sigma_m)
        if not any(isinstance(v, (list, tuple, np.ndarray)) for v in vals):  # isotropic: one row, thrice
            return np.array([vals] * 3, dtype=np.float32)
        out = np.zeros((3, 4), dtype=np.float32)
        for q, v in enumerate(vals):
            out[:, q] = np.broadcast_to(np.asarray(v, dtype=np.float32), (3,))
        return out

    @property
    def anisotropic(self) -> bool:
        vals = (self.eps_r, self.sigma_e, self.mu_r, self.sigma_m)
        if not any(isinstance(v, (list, tuple, np.ndarray)) for v in vals):
            return False
        a = self.axes()
        return not (np.array_equal(a[0], a[1]) and np.array_equal(a[0], a[2]))


@dataclasses.dataclass
class Brick:
    box: Tuple[int, int, int, int, int, int]  # is, js, ks, ie, je, ke (half-open cell box)
    material: int                             # index into Scenario.materials


@dataclasses.dataclass
class LumpedSource:
    box: Tuple[int, int, int, int, int, int]  # is, js, ks, ie, je, ke (i,j closed, k half-open)
    resistance: float
    waveform: np.ndarray                      # float32 voltage V(t) per time step


@dataclasses.dataclass
class Resistor:
    box: Tuple[int, int, int, int, int, int]
    resistance: float


@dataclasses.dataclass
class Plate:
    axis: int                                 # normal axis: 0 x, 1 y, 2 z (plate at the box's low coordinate)
    box: Tuple[int, int, int, int, int, int]  # is, js, ks, ie, je, ke (definePlateX / Y / Z)
    sigma_1: float                            # sigma_e of the first tangential component (axis order)
    sigma_2: float                            # sigma_e of the second


def sector_edges(tri: Sequence[int], pz0: int, radius: float, max_x: int, max_y: int, dx: float, dy: float,
                 nx: int, ny: int):
    """Boolean (ny, nx) masks of the Ex and Ey edges in plane pz0 that a sector plate covers
    (fdtd_add_sector; defineSec / tricheck, fdtdrav.h:1681-1744, 56-128): node (i, j) on the side
    of the third vertex of the sides p0-p1 and p1-p2 (or on them) and within ``radius`` of the apex
    p1; Ex for i < max_x, j <= max_y, Ey for i <= max_x, j < max_y. Evaluated as fdtd_add_sector
    does: a coordinate difference a*d - b*d is the float multiply-add fma(a, d, -(b*d)), the side
    tests multiply differences in double, the distance is the float fma(u, u, v*v) under a double
    square root. The float multiply-adds are formed exactly in extended precision (64-bit or wider
    mantissa) and rounded once."""
    f32, ld = np.float32, np.longdouble
    if np.finfo(ld).nmant < 63:
        raise RuntimeError("sector_edges needs an extended-precision long double")
    dxf, dyf = f32(dx), f32(dy)

    def sub(a, b, d):  # fma(a, d, -(b * d)) in float: a, b integer arrays or scalars
        a = np.asarray(a, dtype=np.int64).astype(f32)
        b = np.asarray(b, dtype=np.int64).astype(f32)
        return (a.astype(ld) * ld(d) - (b * d).astype(ld)).astype(f32)

    def cross(ax, ay, bx, by):  # fma(ax, by, -(ay * bx)) in double; the products of float values are exact
        return (np.asarray(ax, np.float64) * np.asarray(by, np.float64)
                - np.asarray(ay, np.float64) * np.asarray(bx, np.float64))

    t = [int(v) for v in tri]
    i = np.arange(nx)[None, :]
    j = np.arange(ny)[:, None]
    ax, ay = sub(t[2], t[0], dxf), sub(t[3], t[1], dyf)
    bx, by = sub(t[4], t[2], dxf), sub(t[5], t[3], dyf)
    cx, cy = sub(t[4], t[0], dxf), sub(t[5], t[1], dyf)
    ex0, ey0 = sub(t[0], t[2], dxf), sub(t[1], t[3], dyf)
    s1 = cross(ax, ay, cx, cy) * cross(ax, ay, sub(i, t[0], dxf), sub(j, t[1], dyf))
    s2 = cross(bx, by, ex0, ey0) * cross(bx, by, sub(i, t[2], dxf), sub(j, t[3], dyf))
    u, v = sub(t[2], i, dxf), sub(t[3], j, dyf)
    d2 = (u.astype(ld) * u.astype(ld) + (v * v).astype(ld)).astype(f32)
    inside = (s1 >= 0) & (s2 >= 0) & ~(np.sqrt(d2.astype(np.float64)) > float(f32(radius)))
    i, j = np.arange(nx)[None, :], np.arange(ny)[:, None]
    return inside & (i < max_x) & (j <= max_y), inside & (i <= max_x) & (j < max_y)


def sector_plates(tri: Sequence[int], pz0: int, radius: float, max_x: int, max_y: int, sigma_x: float,
                  sigma_y: float, dx: float, dy: float, nx: int, ny: int) -> List["Plate"]:
    """The sector plate as plates with the same edges (as fdtd_add_sector builds it): per row, runs
    of covered Ex edges as one-row z plates; per column, runs of covered Ey edges as one-column x
    plates."""
    ex, ey = sector_edges(tri, pz0, radius, max_x, max_y, dx, dy, nx, ny)
    out = []
    for j in range(ny):
        row = np.flatnonzero(ex[j])
        for run in np.split(row, np.flatnonzero(np.diff(row) > 1) + 1) if row.size else []:
            out.append(Plate(2, (int(run[0]), j, pz0, int(run[-1]) + 1, j, pz0), sigma_x, 0.0))
    for i in range(nx):
        col = np.flatnonzero(ey[:, i])
        for run in np.split(col, np.flatnonzero(np.diff(col) > 1) + 1) if col.size else []:
            out.append(Plate(0, (i, int(run[0]), pz0, i, int(run[-1]) + 1, pz0), sigma_y, 0.0))
    return out


@dataclasses.dataclass
class Probe:
    component: int
    i: int
    j: int
    k: int


@dataclasses.dataclass
class Scenario:
    name: str
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    dt: float
    pml: Tuple[int, int, int, int, int, int]  # x_n, x_p, y_n, y_p, z_n, z_p
    steps: int
    materials: List[Material]
    bricks: List[Brick] = dataclasses.field(default_factory=list)
    sources: List[LumpedSource] = dataclasses.field(default_factory=list)
    resistors: List[Resistor] = dataclasses.field(default_factory=list)
    probes: List[Probe] = dataclasses.field(default_factory=list)
    plates: List[Plate] = dataclasses.field(default_factory=list)
    # x-directed lumped elements of defineSourceX (fdtdrav.h:1311-1365): Ex edges i in [is,ie),
    # j in [js,ie], k in [ks,ke] with its load coefficients; never injected (waveform unused)
    x_sources: List[LumpedSource] = dataclasses.field(default_factory=list)
    eps0: float = float(REF_EPS0)
    mu0: float = float(REF_MU0)
    pi: float = float(REF_PI)
    seed: Optional[int] = None
    # CPML grading: 0 = the reference's sigma_opt; 0 < r0 < 1 = sigma_max from that reflection
    # coefficient (fdtd_set_cpml_grading)
    cpml_r0: float = 0.0

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz

    def material_index(self) -> np.ndarray:
        """uint8 cell material index, shape (nz, ny, nx), bricks painted in order (last wins)."""
        idx = np.zeros((self.nz, self.ny, self.nx), dtype=np.uint8)
        for b in self.bricks:
            is_, js, ks, ie, je, ke = b.box
            is_, js, ks = max(is_, 0), max(js, 0), max(ks, 0)
            ie, je, ke = min(ie, self.nx), min(je, self.ny), min(ke, self.nz)
            if is_ < ie and js < je and ks < ke:
                idx[ks:ke, js:je, is_:ie] = b.material
        return idx

    def material_table(self) -> np.ndarray:
        """float32 table (n_materials, 4): eps_r, sigma_e, mu_r, sigma_m (the x values of
        anisotropic materials)."""
        return np.array([(m.eps_r, m.sigma_e, m.mu_r, m.sigma_m) if not m.anisotropic else tuple(m.axes()[0])
                         for m in self.materials], dtype=np.float32).reshape(-1, 4)

    def material_table_axes(self) -> np.ndarray:
        """float32 table (n_materials, 3, 4): per axis x, y, z the values eps_r, sigma_e, mu_r, sigma_m."""
        return np.array([m.axes() for m in self.materials], dtype=np.float32).reshape(-1, 3, 4)

    @property
    def anisotropic(self) -> bool:
        return any(m.anisotropic for m in self.materials)

    def signal_per_node(self, s: int) -> np.ndarray:
        """Per-edge source signal, V(t) / (ke - ks) in float (setGauss, fdtdrav.h:1494; fdtdrav.h:3613)."""
        src = self.sources[s]
        n = np.float32(src.box[5] - src.box[2])
        return (np.asarray(src.waveform, dtype=np.float32) / n).astype(np.float32)


# ----------------------------------------------------------------------------------------------
# Waveforms
# ----------------------------------------------------------------------------------------------

def gaussian_derivative(steps: int, dt: float, fmax: float, dmin: float, delay_steps: float = 0.0,
                        amp: float = 1.0) -> np.ndarray:
    """s(t) = -sqrt(2e) * ((t - t0)/tau) * exp(-((t - t0)/tau)^2), unit peak.

    tau = nc * delta / (2 c) with nc = c / (fmax * delta) (the reference's tau formula of
    source.cu:176-177 with nc derived from fmax), t0 = 4.5 tau, plus an optional delay.
    Evaluated in float64, stored as float32.
    """
    c = float(ref_light_speed())
    nc = c / (fmax * dmin)
    tau = nc * dmin / (2.0 * c)
    t0 = 4.5 * tau + delay_steps * float(dt)
    t = np.arange(steps, dtype=np.float64) * float(np.float32(dt))
    u = (t - t0) / tau
    return (amp * -math.sqrt(2.0 * math.e) * u * np.exp(-u * u)).astype(np.float32)


def gaussian(steps: int, dt: float, tau: float, t0: float, amp: float = 1.0) -> np.ndarray:
    """amp * exp(-((m dt - t0)^2) / tau^2) (setGauss, fdtdrav.h:1486-1501), float64 -> float32."""
    t = np.arange(steps, dtype=np.float64) * float(np.float32(dt))
    return (amp * np.exp(-((t - t0) ** 2) / tau ** 2)).astype(np.float32)


# ----------------------------------------------------------------------------------------------
# Workloads
# ----------------------------------------------------------------------------------------------

def vacuum_cube(n: int = 64, steps: int = 1000, pml: int = 10, delta: float = 1e-3,
                courant: float = 0.99, fmax: float = 30e9, probe_offset: int = 20,
                name: Optional[str] = None) -> Scenario:
    """Vacuum cube with one 50-ohm z-edge source at the centre and an Ez probe ``probe_offset``
    cells away along x (the 64^3 small / FP64-oracle workload)."""
    dt = courant_dt(delta, delta, delta, courant)
    c = n // 2
    wf = gaussian_derivative(steps, dt, fmax, delta)
    src = LumpedSource((c, c, c, c, c, c + 1), 50.0, wf)
    probes = [Probe(EZ, c + probe_offset, c, c)]
    return Scenario(name or f"vacuum{n}", n, n, n, delta, delta, delta, float(dt), (pml,) * 6, steps,
                    [Material()], [], [src], [], probes)


def random_boxes(nx: int, ny: int, nz: int, steps: int, seed: int = 2024, n_boxes: int = 64,
                 edge: Tuple[int, int] = (16, 128), pml: int = 10, n_sources: int = 4,
                 n_probes: int = 16, src_margin: int = 20, delta: float = 1e-3,
                 courant: float = 0.99, fmax: float = 30e9, max_delay: int = 200,
                 eps_range=(1.0, 12.0), sigma_range=(0.0, 0.05), name: Optional[str] = None) -> Scenario:
    """Seeded random dielectric boxes with delayed lumped sources and Ez/Hx probes.

    64 boxes with per-axis edge lengths uniform in ``edge`` cells, positions uniform and clipped to
    the non-CPML interior, eps_r ~ U(eps_range), sigma ~ U(sigma_range) S/m, last box wins; one
    material per box (65 materials with the background). ``n_sources`` 50-ohm z-edge sources at
    least ``src_margin`` cells from the CPML, with delays ~ U[0, max_delay] steps. Half the probes
    are Ez and half Hx, at random interior nodes.
    """
    rng = np.random.default_rng(seed)
    dt = courant_dt(delta, delta, delta, courant)
    lo = np.array([pml, pml, pml])
    hi = np.array([nx - pml, ny - pml, nz - pml])
    mats = [Material()]
    bricks = []
    for b in range(n_boxes):
        size = rng.integers(edge[0], edge[1] + 1, size=3)
        start = np.array([rng.integers(lo[a], max(lo[a] + 1, hi[a] - 1)) for a in range(3)])
        end = np.minimum(start + size, hi)
        eps = float(rng.uniform(*eps_range))
        sig = float(rng.uniform(*sigma_range))
        mats.append(Material(eps_r=eps, sigma_e=sig))
        bricks.append(Brick((int(start[0]), int(start[1]), int(start[2]), int(end[0]), int(end[1]), int(end[2])),
                            len(mats) - 1))
    sources = []
    m = pml + src_margin
    used = set()
    for s in range(n_sources):
        while True:
            i = int(rng.integers(m, nx - m)); j = int(rng.integers(m, ny - m)); k = int(rng.integers(m, nz - m - 1))
            if (i, j, k) not in used:
                used.add((i, j, k))
                break
        delay = float(rng.uniform(0, max_delay))
        wf = gaussian_derivative(steps, dt, fmax, delta, delay_steps=delay)
        sources.append(LumpedSource((i, j, k, i, j, k + 1), 50.0, wf))
    probes = []
    pm = pml + 2
    for p in range(n_probes):
        comp = EZ if p < n_probes // 2 else HX
        probes.append(Probe(comp, int(rng.integers(pm, nx - pm)), int(rng.integers(pm, ny - pm)),
                            int(rng.integers(pm, nz - pm))))
    return Scenario(name or f"boxes{nx}x{ny}x{nz}", nx, ny, nz, delta, delta, delta, float(dt), (pml,) * 6,
                    steps, mats, bricks, sources, [], probes, seed=seed)


def config_small() -> Scenario:
    """64^3 vacuum, 10-cell CPML, centre z-edge Gaussian-derivative source, Ez probe 20 cells away,
    1000 steps."""
    return vacuum_cube(64, 1000, name="vacuum64")


def config_512() -> Scenario:
    """512^3 with 64 seeded random dielectric boxes, 4 delayed sources, 16 probes, 2000 steps."""
    return random_boxes(512, 512, 512, 2000, seed=512, name="boxes512")


def config_hbm() -> Scenario:
    """1024 x 1024 x 896 single domain, same box generator (seed family of the 512^3 case, box
    edges scaled with the domain), 1000 steps."""
    return random_boxes(1024, 1024, 896, 1000, seed=1024, edge=(32, 256), name="boxes1024x1024x896")


def scaled_boxes(nx: int, ny: int, nz: int, steps: int, seed: int = 7, pml: int = 6,
                 n_boxes: int = 12, n_sources: int = 1, n_probes: int = 8, name=None) -> Scenario:
    """A small version of the random-box workload for parity runs the oracle finishes in seconds."""
    e0 = max(2, min(nx, ny, nz) // 8)
    e1 = max(e0 + 1, min(nx, ny, nz) // 2)
    return random_boxes(nx, ny, nz, steps, seed=seed, n_boxes=n_boxes, edge=(e0, e1), pml=pml,
                        n_sources=n_sources, n_probes=n_probes, src_margin=2, max_delay=20,
                        name=name or f"small_boxes{nx}x{ny}x{nz}")


@dataclasses.dataclass
class DesignProblem:
    """A figure-of-merit problem: scenario, design box (cells), eps_r per design cell, Ez probe."""
    scenario: Scenario
    box: Tuple[int, int, int, int, int, int]
    eps: np.ndarray  # float32, (box[5]-box[2], box[4]-box[1], box[3]-box[0])
    probe: Tuple[int, int, int]


def design_problem(n: int = 128, steps: int = 4000, design=(32, 32, 16), pml: int = 10, seed: int = 4,
                   delta: float = 1e-3, courant: float = 0.99, fmax: float = 30e9) -> DesignProblem:
    """Vacuum n^3 with a centred design region of continuous eps_r ~ U[1, 12], one 50-ohm z-edge
    Gaussian-derivative source a quarter of the way along x and the Ez output probe three quarters
    of the way, both on the centre line (the 128^3 / 4000-step adjoint workload by default)."""
    dt = courant_dt(delta, delta, delta, courant)
    c = n // 2
    src = LumpedSource((n // 4, c, c, n // 4, c, c + 1), 50.0, gaussian_derivative(steps, dt, fmax, delta))
    sc = Scenario(f"design{n}", n, n, n, delta, delta, delta, float(dt), (pml,) * 6, steps, [Material()], [], [src], [],
                  [])
    dx, dy, dz = design
    box = (c - dx // 2, c - dy // 2, c - dz // 2, c - dx // 2 + dx, c - dy // 2 + dy, c - dz // 2 + dz)
    eps = np.random.default_rng(seed).uniform(1.0, 12.0, size=(dz, dy, dx)).astype(np.float32)
    return DesignProblem(sc, box, eps, (3 * n // 4, c, c))


def batch_instances(n: int = 256, size=(32, 96), steps: int = 2000, pml: int = 8, n_boxes: int = 8, seed: int = 5,
                    delta: float = 1e-3, courant: float = 0.99, fmax: float = 30e9) -> List[Scenario]:
    """Independent instances with per-axis sizes uniform in ``size`` (inclusive), ``pml``-cell
    CPML, ``n_boxes`` random dielectric boxes (eps_r ~ U[1, 12], lossless), one 50-ohm z-edge
    source and one Ez probe each (the 256-instance batched workload by default)."""
    rng = np.random.default_rng(seed)
    dt = courant_dt(delta, delta, delta, courant)
    out = []
    for q in range(n):
        dims = [int(v) for v in rng.integers(size[0], size[1] + 1, size=3)]
        mats = [Material()]
        bricks = []
        for b in range(n_boxes):
            lo = [int(rng.integers(pml, m - pml - 2)) for m in dims]
            hi = [min(lo[a] + int(rng.integers(4, max(5, dims[a] // 3))), dims[a] - pml) for a in range(3)]
            mats.append(Material(eps_r=float(rng.uniform(1.0, 12.0))))
            bricks.append(Brick((lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]), len(mats) - 1))
        i, j, k = (int(rng.integers(pml + 2, m - pml - 3)) for m in dims)
        src = LumpedSource((i, j, k, i, j, k + 1), 50.0, gaussian_derivative(steps, dt, fmax, delta))
        pi_, pj, pk = (int(rng.integers(pml + 2, m - pml - 2)) for m in dims)
        out.append(Scenario(f"batch{q}", dims[0], dims[1], dims[2], delta, delta, delta, float(dt), (pml,) * 6, steps,
                            mats, bricks, [src], [], [Probe(EZ, pi_, pj, pk)], seed=seed))
    return out


# ---------------------------------------------------------------------------------------------
# marchingLoop's parameter list (fdtdrav.h:3425-3453) and its metre-to-index set-up
# ---------------------------------------------------------------------------------------------
_BRICK_ARRAYS = ["brick_min_x", "brick_min_y", "brick_min_z", "brick_max_x", "brick_max_y", "brick_max_z",
                 "brick_sigma_e_x", "brick_sigma_e_y", "brick_sigma_e_z", "brick_eps_r_x", "brick_eps_r_y",
                 "brick_eps_r_z", "brick_sigma_m_x", "brick_sigma_m_y", "brick_sigma_m_z", "brick_mu_r_x",
                 "brick_mu_r_y", "brick_mu_r_z"]
_PEC_ARRAYS = ["pec_min_x", "pec_min_y", "pec_min_z", "pec_max_x", "pec_max_y", "pec_max_z",
               "pec_sigma_e_x", "pec_sigma_e_y", "pec_sigma_e_z"]
# (name, kind): i int, f float, a float array; in the order of the reference's signature
MARCHING_PARAMS = (
    [("NUMDEV", "i"), ("eps_0", "f"), ("pi", "f"), ("mu_0", "f"), ("c", "f"), ("dx", "f"), ("dy", "f"), ("dz", "f"),
     ("dt", "f"), ("X", "i"), ("Y", "i"), ("Z", "i"), ("n_t_steps", "i")]
    + [(n, "i") for n in ("pml_x_n", "pml_y_n", "pml_z_n", "pml_x_p", "pml_y_p", "pml_z_p",
                          "air_buff_x_n", "air_buff_y_n", "air_buff_z_n", "air_buff_x_p", "air_buff_y_p", "air_buff_z_p")]
    + [("source_tp", "i"), ("source_freq", "f"), ("source_amp", "f")]
    + [(n, "f") for n in ("source_min_x", "source_min_y", "source_min_z", "source_max_x", "source_max_y", "source_max_z")]
    + [("source_direction", "i"), ("rs", "f"), ("nc", "f"), ("tau", "f"), ("t_0", "f")]
    + [(n, "a") for n in _BRICK_ARRAYS] + [("brick_opt", "i"), ("brick_num", "i")]
    + [(n, "a") for n in _PEC_ARRAYS] + [("pec_opt", "i"), ("pec_num", "i")]
    + [(n, "f") for n in ("resistor_min_x", "resistor_min_y", "resistor_min_z", "resistor_max_x", "resistor_max_y",
                          "resistor_max_z", "resistor_resist")]
    + [("resistor_direction", "i"), ("resistor_opt", "i")]
    + [(n, "f") for n in ("sampled_voltage_min_x", "sampled_voltage_min_y", "sampled_voltage_min_z",
                          "sampled_voltage_max_x", "sampled_voltage_max_y", "sampled_voltage_max_z")]
    + [("voltage_direction", "i")]
    + [(n, "f") for n in ("sampled_current_min_x", "sampled_current_min_y", "sampled_current_min_z",
                          "sampled_current_max_x", "sampled_current_max_y", "sampled_current_max_z")]
    + [("current_direction", "i")])


def marching_indices(a: dict) -> dict:
    """Grid size and index boxes of marchingLoop (fdtdrav.h:3485-3653) for parameters ``a`` (names
    of MARCHING_PARAMS): node counts nx, ny, nz (nz rounded up to a multiple of NUMDEV) and the
    boxes of bricks, plates, source, resistor, voltage and current samples."""
    f32 = np.float32
    nx = a["X"] + a["air_buff_x_n"] + a["air_buff_x_p"] + a["pml_x_n"] + a["pml_x_p"]
    ny = a["Y"] + a["air_buff_y_n"] + a["air_buff_y_p"] + a["pml_y_n"] + a["pml_y_p"]
    nz = a["Z"] + a["air_buff_z_n"] + a["air_buff_z_p"] + a["pml_z_n"] + a["pml_z_p"]
    nd = a["NUMDEV"]
    nz = nz if nz % nd == 0 else (nz // nd + 1) * nd
    o = (a["air_buff_x_n"] + a["pml_x_n"], a["air_buff_y_n"] + a["pml_y_n"], a["air_buff_z_n"] + a["pml_z_n"])
    d = (f32(a["dx"]), f32(a["dy"]), f32(a["dz"]))

    def box(lo, hi):
        return tuple([o[q] + calc_index(lo[q], d[q]) for q in range(3)] + [o[q] + calc_index(hi[q], d[q]) for q in range(3)])

    def named(prefix, q=None):
        g = (lambda n: a[n][q]) if q is not None else (lambda n: a[n])
        return box([g(prefix + "_min_" + c) for c in "xyz"], [g(prefix + "_max_" + c) for c in "xyz"])

    out = {"nx": nx, "ny": ny, "nz": nz,
           "bricks": [named("brick", q) for q in range(a["brick_num"] if a["brick_opt"] else 0)],
           "pecs": [named("pec", q) for q in range(a["pec_num"] if a["pec_opt"] else 0)],
           "source": named("source"), "resistor": named("resistor") if a["resistor_opt"] else None,
           "voltage": named("sampled_voltage"), "current": named("sampled_current")}
    return out


def marching_scenario(a: dict, waveform: np.ndarray) -> Tuple[Scenario, Tuple[int, ...], Tuple[int, ...]]:
    """The scenario marchingLoop builds from ``a`` (bricks with per-axis materials, z plates, z
    source and resistor), with the source voltage ``waveform``; returns it with the voltage and
    current boxes."""
    ix = marching_indices(a)
    mats = [Material()]
    bricks = []

    def axes(name, q):
        return tuple(float(a[f"brick_{name}_{c}"][q]) for c in "xyz")
    for q, b in enumerate(ix["bricks"]):
        mats.append(Material(eps_r=axes("eps_r", q), sigma_e=axes("sigma_e", q), mu_r=axes("mu_r", q),
                             sigma_m=axes("sigma_m", q)))
        bricks.append(Brick(b, q + 1))
    sc = Scenario(name="marching", nx=ix["nx"], ny=ix["ny"], nz=ix["nz"], dx=float(a["dx"]), dy=float(a["dy"]),
                  dz=float(a["dz"]), dt=float(a["dt"]),
                  pml=(a["pml_x_n"], a["pml_x_p"], a["pml_y_n"], a["pml_y_p"], a["pml_z_n"], a["pml_z_p"]),
                  steps=a["n_t_steps"], materials=mats, bricks=bricks, eps0=float(a["eps_0"]), mu0=float(a["mu_0"]),
                  pi=float(a["pi"]))
    sc.plates = [Plate(2, b, float(a["pec_sigma_e_x"][q]), float(a["pec_sigma_e_y"][q])) for q, b in enumerate(ix["pecs"])]
    sc.sources = [LumpedSource(ix["source"], float(a["rs"]), np.asarray(waveform, dtype=np.float32))]
    if ix["resistor"] is not None:
        sc.resistors = [Resistor(ix["resistor"], float(a["resistor_resist"]))]
    return sc, ix["voltage"], ix["current"]
