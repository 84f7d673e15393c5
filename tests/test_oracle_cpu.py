"""Analytic checks of the FP64 CPU oracle (no GPU needed).

The reference's own tests pin no field value (meep is external), so the
oracle is pinned by physics instead:
  - exact discrete energy conservation of the leapfrog in a closed cavity;
  - the local polarisation recurrence (meep's Lorentzian update) and the
    resulting resonance omega_0 * sqrt(1 + sigma/eps_inf);
  - CPML reflection against a larger domain whose walls are out of reach;
  - mirror symmetry of the junction's gap field.
"""
import math

import numpy as np
import pytest

from oracle.oracle import OracleFields
from sim_juncs_gb300 import _abi
from sim_juncs_gb300.configs import junction_instance
from sim_juncs_gb300.spec import PML, ClassMaterial, Grid, Instance, Probe, Source


def uniform_material(n, eps=1.0, poles=(), sigma=None):
    cm = np.zeros((3, n, n, n), dtype=np.uint8)
    sig = None if sigma is None else np.array([sigma], dtype=np.float64)
    return ClassMaterial(cm, [eps], list(poles), sig)


def energy(o, n_next):
    """Discrete leapfrog energy sum(eps E^n^2) + sum(H^{n-1/2} H^{n+1/2})."""
    E = [o.get_array(c) for c in range(3)]
    Ha = [o.get_array(c) for c in range(3, 6)]
    o.step(1)
    Hb = [o.get_array(c) for c in range(3, 6)]
    return sum((e * e).sum() for e in E) + sum((a * b).sum() for a, b in zip(Ha, Hb))


def test_closed_cavity_conserves_discrete_energy(oracle_lib):
    n = 20
    inst = Instance(Grid(n, n, n, 0.1), uniform_material(n), PML(0.0), save_span=1)
    o = OracleFields(inst)
    rng = np.random.default_rng(7)
    for c in range(3):
        o.set_array(c, rng.standard_normal((n, n, n)))
    w0 = energy(o, 1)
    o.step(200)
    w1 = energy(o, 1)
    assert abs(w1 - w0) / w0 < 1e-11


@pytest.mark.parametrize("drude", [False, True])
def test_local_polarisation_recurrence(oracle_lib, drude):
    # uniform E in a uniform dispersive medium: the centre voxel sees no curl
    # until the walls' influence arrives (at most one cell per step)
    n = 41
    w0, g, sig, eps = (0.8, 0.05, 2.0, 1.5)
    inst = Instance(Grid(n, n, n, 0.05), uniform_material(n, eps, [(w0, g, drude)], [sig]),
                    PML(0.0), save_span=1)
    o = OracleFields(inst)
    for c in range(3):
        o.set_array(c, np.ones((n, n, n)))
    dt = o.dt()
    w, gm = 2 * math.pi * w0, 2 * math.pi * g
    den = 1 + gm * dt / 2
    A = (2 - w * w * dt * dt * (0.0 if drude else 1.0)) / den
    B = -(1 - gm * dt / 2) / den
    Cs = w * w * dt * dt / den * sig
    e, p, pm = 1.0, 0.0, 0.0
    steps = 18
    for _ in range(steps):
        pn = A * p + B * pm + Cs * e
        e = e + (0.0 - (pn - p)) / eps
        pm, p = p, pn
    o.step(steps)
    c = n // 2
    for comp in range(3):
        assert o.get_array(comp)[c, c, c] == pytest.approx(e, rel=1e-13, abs=1e-15)


def test_lorentz_resonance_frequency(oracle_lib):
    # the recurrence above oscillates at omega_0 * sqrt(1 + sigma/eps)
    w0, sig, eps = 0.5, 3.0, 1.0
    dt = 0.002
    w = 2 * math.pi * w0
    A, B, Cs = 2 - w * w * dt * dt, -1.0, w * w * dt * dt * sig
    e, p, pm = 1.0, 0.0, 0.0
    xs = []
    for _ in range(40000):
        pn = A * p + B * pm + Cs * e
        e = e - (pn - p) / eps
        pm, p = p, pn
        xs.append(e)
    x = np.array(xs) - np.mean(xs)
    spec = np.abs(np.fft.rfft(x * np.hanning(len(x)), 1 << 20))
    f = np.fft.rfftfreq(1 << 20, dt)[np.argmax(spec)]
    assert f == pytest.approx(w0 * math.sqrt(1 + sig / eps), rel=2e-3)


def test_cpml_reflection_small(oracle_lib):
    # probe near a small source: PML-bounded box vs a box large enough that
    # its walls cannot be reached and heard back within the window
    dx = 0.1
    steps = 90

    def run(n, pml_cells):
        L = n * dx
        c = L / 2
        src = Source(_abi.EZ, 1.0, 0.3, 0.0, 2.4, (c - 0.05, c - 0.05, c - 0.05),
                     (c + 0.05, c + 0.05, c + 0.05))
        probe = Probe(_abi.EZ, (c + 0.6, c, c))
        inst = Instance(Grid(n, n, n, dx), uniform_material(n), PML(pml_cells * dx), [src], [probe],
                        save_span=1)
        o = OracleFields(inst)
        o.step(steps)
        return o.monitors()[0]

    small = run(36, 8)
    big = run(36 + 2 * 50, 0)
    err = np.max(np.abs(small - big)) / np.max(np.abs(big))
    print("PML reflection error", err)
    assert err < 2e-2
    assert np.max(np.abs(big)) > 1e-5


def test_junction_gap_field_is_mirror_symmetric(oracle_lib):
    # res 16: no box face falls exactly on a Yee point, so inclusion at the
    # faces is not decided by rounding and the structure is mirror symmetric
    inst = junction_instance(n=48, res=16.0, pml_um=0.4)
    o = OracleFields(inst)
    o.step(600)
    m = o.monitors()
    # probes 0..3 are Ex at x = c -0.075, -0.025, +0.025, +0.075.  The grid
    # itself is not exactly mirror symmetric (integer-x components exist at
    # i = 0 but not at i = n, deep in the PML), which leaves ~1e-8 residue.
    assert np.max(np.abs(m[0])) > 1e-3
    np.testing.assert_allclose(m[0], m[3], rtol=0, atol=1e-7 * np.max(np.abs(m[0])))
    np.testing.assert_allclose(m[1], m[2], rtol=0, atol=1e-7 * np.max(np.abs(m[0])))


def cavity_energy(arrays_n, h_next, eps_maps, dx):
    """W = 1/2 dx^3 [sum eps E^n E^n + sum H^{n-1/2} H^{n+1/2}] from the E^n,
    H^{n-1/2} arrays and the H^{n+1/2} arrays one step later."""
    w = sum((eps_maps[c] * arrays_n[c] * arrays_n[c]).sum() for c in range(3))
    w += sum((arrays_n[3 + c] * h_next[c]).sum() for c in range(3))
    return 0.5 * dx ** 3 * w


def dielectric_cavity(n=20, seed=3):
    """A closed cavity with a dielectric block (eps 2.5) in one corner and
    random initial E."""
    cm = np.zeros((3, n, n, n), dtype=np.uint8)
    cm[:, 3:11, 5:14, 2:9] = 1
    inst = Instance(Grid(n, n, n, 0.1), ClassMaterial(cm, [1.0, 2.5]), PML(0.0), save_span=1)
    rng = np.random.default_rng(seed)
    init = [rng.standard_normal((n, n, n)) for _ in range(3)]
    eps = [np.where(cm[c] == 1, 2.5, 1.0) for c in range(3)]
    return inst, init, eps


def test_dielectric_cavity_conserves_the_energy_form(oracle_lib):
    inst, init, eps = dielectric_cavity()
    o = OracleFields(inst)
    for c in range(3):
        o.set_array(c, init[c])

    def w_now():
        a = [o.get_array(c) for c in range(6)]
        o.step(1)
        return cavity_energy(a, [o.get_array(c) for c in range(3, 6)], eps, inst.grid.dx)
    w0 = w_now()
    o.step(150)
    w1 = w_now()
    assert w0 > 0
    assert abs(w1 - w0) / w0 < 1e-11
