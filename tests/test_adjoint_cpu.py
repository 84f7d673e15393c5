"""The oracle's discrete adjoint against central finite differences (FP64).

A 32^3 junction (5-cell CPML, Au boxes with a Drude and a Lorentz pole, the
x-polarised current sheet) with a 4 x 4 x 2 design region in the gap and
|E(fcen)|^2 over a 2 x 2 gap patch as the objective: dF/d(eps) from one
forward and one adjoint sweep must match (F(eps+h) - F(eps-h)) / 2h."""
import numpy as np
import pytest

from oracle.oracle import OracleFields
from sim_juncs_gb300.configs import junction_instance
from sim_juncs_gb300.spec import Design, Objective

N_STEPS = 240


def setup():
    inst = junction_instance(n=32, res=10.0, probe_components=("Ex",), dft=False)
    c = 16
    eps = np.random.default_rng(1).uniform(1.0, 4.0, size=(2, 4, 4))
    des = Design((c - 2, c - 2, c - 1), eps)
    obj = Objective(np.array([[c - 1, c - 1, c], [c, c - 1, c], [c - 1, c, c], [c, c, c]]),
                    frequency=1 / 0.7, comps=(0, 2))
    return inst, des, obj


def test_oracle_adjoint_matches_finite_differences():
    inst, des, obj = setup()
    o = OracleFields(inst)
    o.set_design(des)
    F, g = o.adjoint(obj, N_STEPS)
    assert F > 0 and g.shape == des.eps.shape
    assert o.steps_done == N_STEPS
    h = 1e-3
    for idx in [(0, 0, 0), (1, 2, 3), (0, 1, 2), (1, 3, 0)]:
        fs = []
        for sgn in (1, -1):
            e2 = des.eps.copy()
            e2[idx] += sgn * h
            o.set_design(Design(des.lo, e2))
            fs.append(o.objective(obj, N_STEPS))
        fd = (fs[0] - fs[1]) / (2 * h)
        assert g[idx] == pytest.approx(fd, rel=1e-5, abs=1e-9 * abs(F)), (idx, g[idx], fd)


def test_objective_equals_the_dft_probes():
    # F from the objective path equals sum |DFT|^2 of ordinary DFT probes
    # placed at the same Yee points (same sampling time and phase convention)
    import dataclasses
    from sim_juncs_gb300 import _abi
    from sim_juncs_gb300.spec import Probe
    inst, des, obj = setup()
    o = OracleFields(inst)
    o.set_design(des)
    F = o.objective(obj, 120)
    g = inst.grid
    off = {0: (0.5, 0, 0), 1: (0, 0.5, 0), 2: (0, 0, 0.5)}
    probes = [Probe(c, tuple(g.origin[a] + (cell[a] + off[c][a]) * g.dx for a in range(3)), monitor=False, dft=True)
              for cell in obj.cells for c in obj.comps]
    inst2 = dataclasses.replace(inst, probes=probes, freqs=[obj.frequency])
    o2 = OracleFields(inst2)
    o2.set_design(des)
    o2.step(120)
    d = o2.dft()
    assert d.shape[0] == len(probes)
    assert F == pytest.approx(float(np.sum(np.abs(d) ** 2)), rel=1e-10)
