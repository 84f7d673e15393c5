"""Stepping parity on the scenes of every measured workload, through the C ABI.

test_gpu_parity.py holds the Au box-pair junction at 64^3 (the reference's
small case) to the FP64 oracle; this file does the same for the scenes the
other workloads use:

  * the bowtie (two Au prisms cut by slanted planes on a nondispersive SiO2
    slab, first-containing-root eps), at 128 x 128 x 96 and 10 px/um;
  * the inverse-design scene (Au box pair on quartz: a Lorentz term with
    gamma = 0 under first-containing-root eps), at its full 192^3 and 30 px/um;
  * the sweep's 128^3 (40 px/um) and 192^3 (60 px/um) members.

Every run starts the pulse early (peak at t = 0.5 instead of 10) so that it
crosses the sheet-to-gold distance within the few hundred steps the oracle
finishes in seconds: the gold, the PML and the sources all carry field.  Bar:
FP64 fields within 1e-10 of the oracle relative to the run's peak field,
monitors and DFT sums within 1e-10 of their own maximum; FP32 gap monitors
within 1e-4 of FP64.
"""
import numpy as np
import pytest

from oracle.oracle import OracleFields
from sim_juncs_gb300.configs import bowtie_instance, inverse_design_case, junction_instance
from sim_juncs_gb300.fields import Fields

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 1e-4


def early_pulse(inst, peak=0.5):
    """Shift every source so that its Gaussian peaks at t = peak."""
    for s in inst.sources:
        shift = 0.5 * (s.start_time + s.end_time) - peak
        s.start_time -= shift
        s.end_time -= shift
    return inst


def rel(a, b):
    scale = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / scale) if scale > 0 else float(np.max(np.abs(a)))


def check_against_oracle(inst, steps, checkpoints):
    f = Fields(inst, "f64")
    assert f.schedule_name() == "fused"
    o = OracleFields(inst)
    peak = 0.0
    for upto in checkpoints + (steps,):
        n = upto - o.steps_done
        f.step(n)
        o.step(n)
        gs = [f.get_array(c) for c in range(6)]
        rs = [o.get_array(c) for c in range(6)]
        peak = max([peak] + [float(np.max(np.abs(r))) for r in rs])
        assert peak > 0
        for c in range(6):
            err = float(np.max(np.abs(gs[c] - rs[c]))) / peak
            assert err <= TOL64, (upto, c, err)
    mg, mo = f.monitors(), o.monitors()
    assert mg.shape == mo.shape and mg.size > 0
    assert np.max(np.abs(mo)) > 0
    assert rel(mg, mo) <= TOL64
    if inst.freqs:
        dg, do = f.dft(), o.dft()
        assert rel(dg, do) <= TOL64
    return f


def gold_field(f, inst, region=0):
    """Largest |E| at E points inside the scene's first region (the gold)."""
    cm = f.class_map()
    best = 0.0
    for c in range(3):
        m = cm[c] != 0
        if m.any():
            best = max(best, float(np.max(np.abs(f.get_array(c)[m]))))
    return best


def test_bowtie_f64_matches_oracle(lib, oracle_lib):
    inst = early_pulse(bowtie_instance(nx=128, ny=128, nz=96, res=10.0, n_freq=8, plane_n=8))
    f = check_against_oracle(inst, 220, (1, 60))
    assert gold_field(f, inst) > 0
    g = Fields(inst, "f32")
    g.step(220)
    assert rel(g.monitors(), f.monitors()) <= TOL32
    assert rel(g.dft(), f.dft()) <= TOL32


def test_au_on_quartz_f64_matches_oracle(lib, oracle_lib):
    inst, _, _ = inverse_design_case(0, n=192, res=30.0)
    inst = early_pulse(inst)
    f = check_against_oracle(inst, 110, (1, 50))
    assert gold_field(f, inst) > 0
    g = Fields(inst, "f32")
    g.step(110)
    assert rel(g.monitors(), f.monitors()) <= TOL32


@pytest.mark.parametrize("n,res,steps", [(128, 40.0, 110), (192, 60.0, 150)])
def test_sweep_member_f64_matches_oracle(lib, oracle_lib, n, res, steps):
    inst = early_pulse(junction_instance(n=n, res=res, phase=1.3, amplitude=4.0,
                                         probe_components=("Ez",), dft=False))
    f = check_against_oracle(inst, steps, (1, steps // 2))
    assert gold_field(f, inst) > 0
    g = Fields(inst, "f32")
    g.step(steps)
    assert rel(g.monitors(), f.monitors()) <= TOL32


@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("f32", 2e-6)])
def test_uniform_au_follows_the_ade_recurrence(lib, precision, tol):
    """The device's polarisation update is the recurrence whose discrete
    eps(omega) tests/test_eps_cpu.py pins to the reference's dielectric model."""
    from test_eps_cpu import recurrence, uniform_au_instance
    from sim_juncs_gb300 import _abi
    from sim_juncs_gb300.configs import AU
    inst = uniform_au_instance()
    g = inst.grid
    f = Fields(inst, precision)
    f.set_array(_abi.EX, np.ones((g.nz, g.ny, g.nx)))
    f.step(16)
    series = f.monitors()[0]
    want = recurrence(1.0, AU, g.dt, 15)
    assert np.max(np.abs(series - want)) <= tol


def test_reference_rounding_65_cubed_f64_matches_oracle(lib, oracle_lib):
    """The junction on the grid the reference's correct_defaults gives the
    3.2 um cell at 20 px/um (65^3, 20.3125 px/um): an odd nx, so the
    one-column tile bodies run, over the workload's 2000 steps."""
    from sim_juncs_gb300.spec import reference_grid
    g, res = reference_grid(length=2.2, pml_thickness=0.5, resolution=20.0)  # 3.2 um in all
    assert g.nx == 65 and res == 65 / 3.2
    inst = junction_instance(n=g.nx, res=res)
    f = check_against_oracle(inst, 2000, (1, 400))
    assert gold_field(f, inst) > 0


def three_pole_gold(inst):
    """The scene's gold with a third (Lorentz) pole: every gold E point then
    carries three polarisations, the case past the polarisation kernels' two
    poles per point loaded up front."""
    from sim_juncs_gb300.configs import AU
    from sim_juncs_gb300.spec import Susceptibility
    inst.material.regions[0].susceptibilities = list(AU) + [Susceptibility(0.8, 0.1, 0.3, drude=False)]
    return inst


def test_three_pole_gold_f64_matches_oracle(lib, oracle_lib):
    inst = three_pole_gold(early_pulse(junction_instance(n=64, res=20.0)))
    f = check_against_oracle(inst, 200, (1, 100))
    assert gold_field(f, inst) > 0
    g = Fields(inst, "f32")
    g.step(200)
    assert rel(g.monitors(), f.monitors()) <= TOL32
