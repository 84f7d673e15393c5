"""The workloads the stepper is measured and checked on, as Instance specs.

All lengths in um with um_scale = 1 (one meep length unit = 1 um), so
meep frequencies are 1/wavelength(um) and times are um/c.

  junction      3.2 um cube at 20 px/um (64^3), 0.5 um PML, two Au boxes
                1.0 x 0.5 x 0.1 um with a 0.2 um x-gap, current sheet 1.0 um
                below the junction, fcen = 1/0.7, fwidth = 0.5, 2000 steps,
                Courant 0.457 (stable_courant at 20 px/um)
  bowtie        512 x 512 x 384 at 40 px/um, 1.0 um PML, two Au triangular
                prisms (2.0 um tip-to-base, 60 deg apex, 0.05 um thick,
                0.1 um tip gap) on a 1.0 um SiO2 slab (eps 2.13), fcen = 1/0.8,
                32 x 32 Ez monitor plane + 50-frequency flux DFT
  sweep         96 junction instances: 32 each at 96^3 (30 px/um), 128^3
                (40 px/um), 192^3 (60 px/um), CEP ~ U[0, 2pi) and amplitude
                log-uniform in [0.1, 10] from seed 0, Ez at 4 gap points
Au: eps_inf = 1, Drude (omega_p = 7.3, gamma = 0.043 -> omega_0 = 1,
sigma = omega_p^2) + Lorentz (f0 = 0.33, gamma = 0.29, sigma = 1.1).

The drive is an x-polarised sheet (SHEET_COMPONENT), as in the reference's
junction files (junctions/Au_SiO2_box/junc.geom:11): a z-directed current in
a z-normal sheet launches no propagating wave, so an Ez sheet below the
junction would leave the gap dark.
"""
import math

import numpy as np

from . import _abi
from .geometry import Box, Intersect, Plane, Union
from .spec import PML, Grid, Instance, Probe, Region, Scene, Source, Susceptibility

AU = [Susceptibility(1.0, 0.043, 7.3 ** 2, drude=True),
      Susceptibility(0.33, 0.29, 1.1, drude=False)]
QUARTZ = [Susceptibility(10.0, 0.0, 0.25, drude=False)]
SHEET_COMPONENT = _abi.EX


def stable_courant(res, omega_p=7.3, courant=0.5):
    """Largest Courant number <= `courant` that keeps the leapfrog + explicit
    Drude ADE stable: 12 S^2 + (2 pi omega_p S / res)^2 <= 4 (with a 5% margin).

    At 20 px/um the Au Drude term (omega_p = 7.3) violates this at S = 0.5
    (the field grows ~1.5x per step), so the 64^3 junction runs at 0.4573."""
    w = 2 * math.pi * omega_p / res
    smax = math.sqrt(4.0 / (12.0 + w * w)) * 0.95
    return min(courant, smax)


def gaussian_pulse(component, z_sheet, L, fcen, fwidth=0.5, cutoff=5.0, phase=0.0,
                   amplitude=1.0, start_time=0.0):
    """A Gaussian_source sheet spanning the cell in x and y at z = z_sheet.

    Timing follows source_info (src/disp.cpp:318-376): width = 1/fwidth,
    end_time = start_time + 2 * cutoff * width (cutoff = 5 unless the CGS
    source sets one)."""
    width = 1.0 / fwidth
    end = start_time + 2 * cutoff * width
    return Source(component, fcen, width, start_time, end, (0.0, 0.0, z_sheet), (L, L, z_sheet),
                  phase=phase, amplitude=amplitude)


def junction_instance(n=64, res=20.0, pml_um=0.5, phase=0.0, amplitude=1.0,
                      fcen=1 / 0.7, probe_components=("Ex", "Ez"), dft=True, save_span=20,
                      component=SHEET_COMPONENT):
    """The Au box-pair junction (3.2 um cube, 0.2 um gap) at grid n^3."""
    dx = 1.0 / res
    L = n * dx
    c = L / 2
    gap, bx, by, bz = 0.2, 1.0, 0.5, 0.1
    au = Union(Box((c - gap / 2 - bx, c - by / 2, c - bz / 2), (c - gap / 2, c + by / 2, c + bz / 2)),
               Box((c + gap / 2, c - by / 2, c - bz / 2), (c + gap / 2 + bx, c + by / 2, c + bz / 2)))
    scene = Scene([Region(au, eps=1.0, susceptibilities=list(AU))], ambient_eps=1.0)
    src = gaussian_pulse(component, c - 1.0, L, fcen, phase=phase, amplitude=amplitude)
    pts = [(c + dxp, c, c) for dxp in (-0.075, -0.025, 0.025, 0.075)]
    probes = []
    for comp in probe_components:
        for p in pts:
            probes.append(Probe(_abi.COMPONENTS[comp], p, monitor=True, dft=dft))
    freqs = [0.9 * fcen, fcen, 1.1 * fcen] if dft else []
    dt = stable_courant(res) * dx
    return Instance(Grid(n, n, n, dx, dt), scene, PML(pml_um), [src], probes, freqs, save_span)


def bowtie_instance(nx=512, ny=512, nz=384, res=40.0, pml_um=1.0, n_freq=50, plane_n=32):
    """The 512 x 512 x 384 bowtie: Au prisms on an SiO2 slab; FIRST-containing-root eps."""
    dx = 1.0 / res
    Lx, Ly, Lz = nx * dx, ny * dx, nz * dx
    cx, cy, cz = Lx / 2, Ly / 2, Lz / 2
    thick, gap, hgt = 0.05, 0.1, 2.0
    half_apex = math.radians(30.0)
    top, bot = cz + thick / 2, cz - thick / 2
    slab = Box((0.0, 0.0, bot - 1.0), (Lx, Ly, bot))
    prisms = []
    for side in (-1, 1):
        tip = cx + side * gap / 2
        base = tip + side * hgt
        # triangle in x-y: beyond the tip, before the base, inside the two slanted edges
        # |y - cy| <= tan(30 deg) * side * (x - tip), as two half-spaces
        # dot(r, n) <= offset with a unit normal (plane() normalises only n)
        tan = math.tan(half_apex)
        nrm = math.sqrt(tan * tan + 1.0)
        e_up = Plane((-side * tan / nrm, 1.0 / nrm, 0.0), (cy - side * tan * tip) / nrm)
        e_dn = Plane((-side * tan / nrm, -1.0 / nrm, 0.0), (-cy - side * tan * tip) / nrm)
        lo_x, hi_x = (tip, base) if side > 0 else (base, tip)
        zbox = Box((lo_x, 0.0, bot), (hi_x, Ly, top))
        prisms.append(Intersect(e_up, e_dn, zbox))
    au = Union(*prisms)
    scene = Scene([Region(au, 1.0, list(AU)), Region(slab, 2.13, [])], ambient_eps=1.0,
                  combine=_abi.EPS_FIRST)
    fcen = 1 / 0.8
    src = gaussian_pulse(SHEET_COMPONENT, bot - 1.5, Lx, fcen)
    src.hi = (Lx, Ly, bot - 1.5)
    h = plane_n * dx
    pts = [(cx - h / 2 + (i + 0.5) * dx, cy - h / 2 + (j + 0.5) * dx, cz)
           for j in range(plane_n) for i in range(plane_n)]
    probes = [Probe(_abi.EZ, p, monitor=True, dft=False) for p in pts]
    for comp in (_abi.EX, _abi.EY, _abi.HX, _abi.HY):
        probes += [Probe(comp, p, monitor=False, dft=True) for p in pts]
    freqs = list(np.linspace(0.5 * fcen, 1.5 * fcen, n_freq))
    dt = stable_courant(res) * dx
    return Instance(Grid(nx, ny, nz, dx, dt), scene, PML(pml_um), [src], probes, freqs, save_span=20)


def bowtie_flux_rows(plane_n=32):
    """DFT rows (Ex, Ey, Hx, Hy) of each point of bowtie_instance's plane, the
    quadruples sj_flux takes for the z-normal flux through it."""
    m = plane_n * plane_n
    return [[p, m + p, 2 * m + p, 3 * m + p] for p in range(m)]


def sweep_instances(per_size=32, sizes=((96, 30.0), (128, 40.0), (192, 60.0)), seed=0):
    """The 96-instance CEP/amplitude sweep over uneven grids (same 3.2 um junction cell)."""
    rng = np.random.default_rng(seed)
    out = []
    for n, res in sizes:
        for _ in range(per_size):
            cep = float(rng.uniform(0.0, 2 * math.pi))
            amp = float(10 ** rng.uniform(-1.0, 1.0))
            out.append(junction_instance(n=n, res=res, phase=cep, amplitude=amp,
                                         probe_components=("Ez",), dft=False))
    return out


def adjoint_case(n=160, res=30.0, seed=1, design_um=(0.6, 0.6, 0.1), patch=5):
    """The adjoint case: the Au box-pair junction at n^3 (30 px/um: 160^3), a design region
    of design_um centred in the gap with eps ~ U[1, 4] from `seed`, and
    |E(fcen)|^2 summed over a patch x patch gap patch in the junction's
    mid plane.  Returns (instance, design, objective)."""
    from .spec import Design, Objective
    inst = junction_instance(n=n, res=res, probe_components=("Ex",), dft=False)
    dx = 1.0 / res
    nd = [max(1, int(round(u / dx))) for u in design_um]
    c = n // 2
    lo = (c - nd[0] // 2, c - nd[1] // 2, c - nd[2] // 2)
    eps = np.random.default_rng(seed).uniform(1.0, 4.0, size=(nd[2], nd[1], nd[0]))
    cells = np.array([[c - patch // 2 + a, c - patch // 2 + b, c] for b in range(patch) for a in range(patch)])
    return inst, Design(lo, eps), Objective(cells, frequency=1 / 0.7, comps=(0, 1, 2))


def inverse_design_case(index, n=192, res=30.0, design_um=(0.8, 0.8, 0.1), patch=5):
    """Inverse-design instance `index`: the Au box pair of the junction (Drude + Lorentz Au) on a
    quartz substrate (eps_inf 2.1 plus one Lorentz term, f0 = 10, gamma = 0,
    sigma = 0.25) filling the cell below the boxes, at n^3 and `res` px/um
    (192^3, 30 px/um); a design_um region in the gap with eps ~ U[1, 4]
    from seed `index`; |E(fcen)|^2 over a patch x patch gap patch as the
    objective.  Returns (instance, design, objective)."""
    from .spec import Design, Objective
    inst = junction_instance(n=n, res=res, probe_components=("Ex",), dft=False)
    dx = 1.0 / res
    L = n * dx
    c = L / 2
    gap, bx, by, bz = 0.2, 1.0, 0.5, 0.1
    au = Union(Box((c - gap / 2 - bx, c - by / 2, c - bz / 2), (c - gap / 2, c + by / 2, c + bz / 2)),
               Box((c + gap / 2, c - by / 2, c - bz / 2), (c + gap / 2 + bx, c + by / 2, c + bz / 2)))
    substrate = Box((0.0, 0.0, 0.0), (L, L, c - bz / 2))
    # the first root containing a point decides (Au over quartz)
    inst.material = Scene([Region(au, eps=1.0, susceptibilities=list(AU)),
                           Region(substrate, eps=2.1, susceptibilities=list(QUARTZ))],
                          ambient_eps=1.0, combine=_abi.EPS_FIRST)
    nd = [max(1, int(round(u / dx))) for u in design_um]
    m = n // 2
    lo = (m - nd[0] // 2, m - nd[1] // 2, m - nd[2] // 2)
    eps = np.random.default_rng(index).uniform(1.0, 4.0, size=(nd[2], nd[1], nd[0]))
    cells = np.array([[m - patch // 2 + a, m - patch // 2 + b, m] for b in range(patch) for a in range(patch)])
    return inst, Design(lo, eps), Objective(cells, frequency=1 / 0.7, comps=(0, 1, 2))
