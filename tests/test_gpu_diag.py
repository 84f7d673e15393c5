"""The device's FP64 diagnostics against the oracle: the discrete energy of a
closed dielectric cavity (conserved exactly by the leapfrog, so FP32 drift is
the fields' rounding) and the flux spectrum of the bowtie's DFT plane."""
import numpy as np
import pytest

from oracle.oracle import OracleFields
from sim_juncs_gb300.configs import bowtie_flux_rows, bowtie_instance
from sim_juncs_gb300.fields import Fields

from test_gpu_configs import early_pulse
from test_oracle_cpu import cavity_energy, dielectric_cavity

pytestmark = pytest.mark.gpu


def test_energy_equals_oracle_form(lib, oracle_lib):
    inst, init, eps = dielectric_cavity()
    f = Fields(inst, "f64")
    o = OracleFields(inst)
    for c in range(3):
        f.set_array(c, init[c])
        o.set_array(c, init[c])
    f.step(40)
    o.step(40)
    w_dev = f.energy()
    a = [o.get_array(c) for c in range(6)]
    o.step(1)
    w_ref = cavity_energy(a, [o.get_array(c) for c in range(3, 6)], eps, inst.grid.dx)
    assert w_dev == pytest.approx(w_ref, rel=1e-12)


@pytest.mark.parametrize("precision,tol", [("f64", 1e-11), ("f32", 1e-4)])
def test_energy_is_conserved_in_a_closed_cavity(lib, precision, tol):
    inst, init, _ = dielectric_cavity(n=48)
    f = Fields(inst, precision)
    for c in range(3):
        f.set_array(c, init[c])
    f.step(1)
    w0 = f.energy()
    f.step(2000)
    w1 = f.energy()
    assert abs(w1 - w0) / w0 <= tol, (precision, abs(w1 - w0) / w0)


def test_flux_matches_oracle_dft(lib, oracle_lib):
    plane_n = 8
    inst = early_pulse(bowtie_instance(nx=128, ny=128, nz=96, res=10.0, n_freq=8, plane_n=plane_n))
    rows = bowtie_flux_rows(plane_n)
    dA = inst.grid.dx ** 2
    f = Fields(inst, "f64")
    o = OracleFields(inst)
    f.step(220)
    o.step(220)
    d = o.dft()
    r = np.asarray(rows)
    want = dA * np.sum((d[r[:, 0]] * np.conj(d[r[:, 3]])).real - (d[r[:, 1]] * np.conj(d[r[:, 2]])).real, axis=0)
    got = f.flux(rows, dA)
    assert np.max(np.abs(want)) > 0
    assert np.max(np.abs(got - want)) <= 1e-10 * np.max(np.abs(want))
    g = Fields(inst, "f32")
    g.step(220)
    got32 = g.flux(rows, dA)
    assert np.max(np.abs(got32 - got)) <= 1e-4 * np.max(np.abs(got))


def test_flux_rejects_rows_of_wrong_components(lib):
    from sim_juncs_gb300 import _abi
    inst = bowtie_instance(nx=64, ny=64, nz=48, res=5.0, n_freq=4, plane_n=4)
    f = Fields(inst, "f32")
    rows = np.asarray(bowtie_flux_rows(4))
    with pytest.raises(_abi.SJError) as e:
        f.flux(rows[:, [1, 0, 2, 3]], 1.0)
    assert e.value.code == _abi.SJ_E_INVALID


def test_field_samples_from_a_run(lib, tmp_path):
    """The monitor file of a junction run: time datasets are the device's
    monitor samples (n_t // save_span of them), frequency datasets its
    device spectra (the reference's fft)."""
    from sim_juncs_gb300 import field_samples as fsm
    from sim_juncs_gb300.configs import junction_instance
    inst = junction_instance(n=40, res=12.5)
    f = Fields(inst, "f64")
    f.step(430)                                   # 22 samples, the file keeps 430 // 20 = 21
    tree = fsm.from_fields(f, cgs_params={"l_per_um": 1.0})
    t = fsm.read(fsm.write(str(tmp_path / "field_samples"), tree))
    mon, spec = f.monitors(), f.monitor_spectrum()
    assert mon.shape[1] == 22 and int(t["info/n_time_points"][0]) == 21
    n = mon.shape[0]
    pd = len(str(n - 1)) if n > 1 else 1
    for i in range(n):
        td = t[f"cluster_0/point_{i:0{pd}d}/time"]
        np.testing.assert_array_equal(td["Re"], mon[i, :21])
        fd = t[f"cluster_0/point_{i:0{pd}d}/frequency"]
        np.testing.assert_array_equal(fd["Re"] + 1j * fd["Im"], spec[i])
    assert t["cluster_1/locations"].shape == (0,)
