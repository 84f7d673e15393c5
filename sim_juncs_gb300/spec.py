"""Python descriptions of one simulation instance, converted to the C ABI
structs of include/sj.h.  Each ``to_c`` keeps the numpy/ctypes buffers it
points into alive on the returned holder object.
"""
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import ctypes as C
import numpy as np

from . import _abi
from .geometry import as_program


@dataclass
class Grid:
    nx: int
    ny: int
    nz: int
    dx: float
    dt: float = 0.0                    # <= 0 -> dx / 2 (Courant 0.5)
    origin: Tuple[float, float, float] = (0.0, 0.0, 0.0)

    def to_c(self):
        g = _abi.GridDesc()
        g.nx, g.ny, g.nz = self.nx, self.ny, self.nz
        g.dx, g.dt = self.dx, self.dt
        for a in range(3):
            g.origin[a] = self.origin[a]
        return g

    @property
    def voxels(self):
        return self.nx * self.ny * self.nz


def reference_grid(length, pml_thickness, resolution, grid_num=-1, courant=0.5, origin=(0.0, 0.0, 0.0)):
    """The reference's grid rounding (correct_defaults, src/argparse.h:171-191)
    for a cubic cell of side length + 2 pml_thickness: unless grid_num is
    given, grid_num = 2 int(0.5 (1 + L_tot res)) + 1 (an odd number of
    points), then res = grid_num / L_tot.  Returns (Grid with dx = 1 / res
    and dt = courant dx, the rounded resolution)."""
    total = length + 2 * pml_thickness
    if grid_num < 0:
        grid_num = 2 * int(0.5 * (1 + total * resolution)) + 1
    res = grid_num / total
    dx = 1.0 / res
    return Grid(grid_num, grid_num, grid_num, dx, courant * dx, tuple(origin)), res


@dataclass
class Susceptibility:
    """One drude_suscept (src/disp.hpp:88-93) in meep units (already / um_scale)."""
    omega_0: float
    gamma: float
    sigma: float
    drude: bool = False


@dataclass
class Region:
    """A scene root: CSG object, its ``eps`` scale and susceptibilities."""
    obj: object
    eps: float = 1.0
    susceptibilities: List[Susceptibility] = field(default_factory=list)


@dataclass
class Scene:
    regions: List[Region]
    ambient_eps: float = 1.0
    combine: int = _abi.EPS_SUM
    # stochastic smoothing of cgs_material_function (src/disp.cpp:56-112,
    # 264-283): 0 = off, the reference's default; smooth_rad in length units
    smooth_n: int = 0
    smooth_rad: float = 0.05


@dataclass
class ClassMaterial:
    """Explicit per-component class map ([3][nz][ny][nx] uint8) + class table."""
    class_map: np.ndarray
    eps_inf: Sequence[float]
    poles: Sequence[Tuple[float, float, bool]] = ()     # (omega_0, gamma, drude)
    sigma: Optional[np.ndarray] = None                  # [n_classes][n_poles]


@dataclass
class PML:
    thickness: object = 0.0            # scalar (all faces) or [3][2]
    r_asymptotic: float = 1e-15
    power: float = 2.0
    alpha: float = 0.0

    def to_c(self):
        p = _abi.PmlDesc()
        th = self.thickness
        for a in range(3):
            for s in range(2):
                p.thickness[a][s] = float(th) if np.isscalar(th) else float(th[a][s])
        p.r_asymptotic, p.power, p.alpha = self.r_asymptotic, self.power, self.alpha
        return p


@dataclass
class Source:
    """A Gaussian_source / CW_source added with add_volume_source (meep units)."""
    component: int
    frequency: float
    width: float
    start_time: float
    end_time: float
    lo: Tuple[float, float, float]
    hi: Tuple[float, float, float]
    phase: float = 0.0
    amplitude: complex = 1.0
    kind: int = _abi.SRC_GAUSSIAN

    def to_c(self):
        s = _abi.SourceDesc()
        s.component, s.kind = self.component, self.kind
        s.frequency, s.width, s.phase = self.frequency, self.width, self.phase
        s.start_time, s.end_time = self.start_time, self.end_time
        s.amplitude[0], s.amplitude[1] = complex(self.amplitude).real, complex(self.amplitude).imag
        for a in range(3):
            s.lo[a], s.hi[a] = self.lo[a], self.hi[a]
        return s


@dataclass
class Probe:
    component: int
    pos: Tuple[float, float, float]
    monitor: bool = True
    dft: bool = False

    def to_c(self):
        p = _abi.ProbeDesc()
        p.component = self.component
        p.flags = (_abi.PROBE_MONITOR if self.monitor else 0) | (_abi.PROBE_DFT if self.dft else 0)
        for a in range(3):
            p.pos[a] = self.pos[a]
        return p


class _Holder:
    """Keeps every buffer a C descriptor points into alive."""

    def __init__(self):
        self.refs = []

    def keep(self, x):
        self.refs.append(x)
        return x


def _array(ctype, values):
    arr = (ctype * max(1, len(values)))(*values)
    return arr


@dataclass
class Instance:
    grid: Grid
    material: object                   # Scene or ClassMaterial
    pml: PML = field(default_factory=PML)
    sources: List[Source] = field(default_factory=list)
    probes: List[Probe] = field(default_factory=list)
    freqs: Sequence[float] = ()
    save_span: int = 20

    def to_c(self, holder=None):
        h = holder or _Holder()
        d = _abi.InstanceDesc()
        d.grid = self.grid.to_c()
        d.pml = self.pml.to_c()
        m = _abi.MaterialDesc()
        mat = self.material
        if isinstance(mat, ClassMaterial):
            cm = h.keep(np.ascontiguousarray(mat.class_map, dtype=np.uint8))
            if cm.shape != (3, self.grid.nz, self.grid.ny, self.grid.nx):
                raise ValueError(f"class_map shape {cm.shape} != (3, nz, ny, nx)")
            m.class_map = cm.ctypes.data_as(C.POINTER(C.c_uint8))
            m.n_classes = len(mat.eps_inf)
            m.eps_inf = h.keep(_array(C.c_double, [float(e) for e in mat.eps_inf]))
            m.n_poles = len(mat.poles)
            m.poles = h.keep(_array(_abi.Pole, [_abi.Pole(w, g, int(dr), 0) for (w, g, dr) in mat.poles]))
            sig = mat.sigma if mat.sigma is not None else np.zeros((m.n_classes, m.n_poles))
            sig = h.keep(np.ascontiguousarray(sig, dtype=np.float64).reshape(-1))
            m.sigma = sig.ctypes.data_as(C.POINTER(C.c_double))
        elif isinstance(mat, Scene):
            regs = []
            for r in mat.regions:
                prog = as_program(r.obj)
                rd = _abi.RegionDesc()
                rd.n_nodes = len(prog)
                rd.nodes = h.keep(_array(_abi.CsgNode, prog))
                rd.eps = r.eps
                rd.n_poles = len(r.susceptibilities)
                rd.poles = h.keep(_array(_abi.Pole, [_abi.Pole(s.omega_0, s.gamma, int(s.drude), 0)
                                                      for s in r.susceptibilities]))
                rd.sigma = h.keep(_array(C.c_double, [s.sigma for s in r.susceptibilities]))
                regs.append(rd)
            sc = _abi.SceneDesc()
            sc.ambient_eps = mat.ambient_eps
            sc.n_regions = len(regs)
            sc.combine = mat.combine
            sc.smooth_n = int(mat.smooth_n)
            sc.smooth_rad = float(mat.smooth_rad)
            sc.regions = h.keep(_array(_abi.RegionDesc, regs))
            h.keep(sc)
            m.scene = C.pointer(sc)
        else:
            raise TypeError("material must be Scene or ClassMaterial")
        d.material = m
        d.n_sources = len(self.sources)
        d.sources = h.keep(_array(_abi.SourceDesc, [s.to_c() for s in self.sources]))
        d.n_probes = len(self.probes)
        d.probes = h.keep(_array(_abi.ProbeDesc, [p.to_c() for p in self.probes]))
        d.n_freqs = len(self.freqs)
        d.freqs = h.keep(_array(C.c_double, [float(f) for f in self.freqs]))
        d.save_span = int(self.save_span)
        return d, h

    @property
    def n_monitors(self):
        return sum(1 for p in self.probes if p.monitor)

    @property
    def n_dft(self):
        return sum(1 for p in self.probes if p.dft)


def scene_to_c(scene, holder=None):
    """Just the sj_scene_desc of a Scene (for sj_rasterize)."""
    inst = Instance(Grid(1, 1, 1, 1.0), scene)
    d, h = inst.to_c(holder)
    return d.material.scene, h


@dataclass
class Design:
    """A design region: per-voxel eps_inf on the box lo .. lo + eps.shape[::-1]
    (eps indexed [k][j][i]), applied at each voxel's Ex, Ey and Ez points."""
    lo: Tuple[int, int, int]
    eps: np.ndarray

    def to_c(self):
        eps = np.ascontiguousarray(self.eps, dtype=np.float64)
        assert eps.ndim == 3
        d = _abi.DesignDesc()
        for a in range(3):
            d.lo[a] = int(self.lo[a])
            d.n[a] = int(eps.shape[2 - a])
        d.eps = eps.ctypes.data_as(C.POINTER(C.c_double))
        return d, eps


@dataclass
class Objective:
    """F = sum over `cells` and E components `comps` of |DFT_f(E_c)|^2, the
    DFT summed over the run (dt E^n e^{+i 2 pi f n dt}, sampled before step n)."""
    cells: np.ndarray                  # [n][3] voxel indices (i, j, k)
    frequency: float
    comps: Tuple[int, ...] = (0, 1, 2)

    def to_c(self):
        cells = np.ascontiguousarray(self.cells, dtype=np.int32).reshape(-1, 3)
        o = _abi.ObjectiveDesc()
        o.n_cells = len(cells)
        o.cells = cells.ctypes.data_as(C.POINTER(C.c_int32))
        o.comp_mask = sum(1 << c for c in self.comps)
        o.frequency = float(self.frequency)
        return o, cells
