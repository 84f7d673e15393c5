"""Failure detection on the GPU, without a GPU fault.

The divergence guard (bound_geom::run flags monitor samples above 1000,
src/disp.cpp:727-729) is exercised by planting the failure on the host: a
huge value or a NaN written into Ex through sj_write_field before a save
point.  The bounded waits of the TMA schedule are exercised with the test
hook that leaves one plane's copy unissued, so a wait on it runs out after a
short limit; the kernel returns, SJ_E_TIMEOUT reaches the host, and the
context stays usable for the next simulation.
"""
import numpy as np
import pytest

from sim_juncs_gb300 import _abi
from sim_juncs_gb300.configs import junction_instance
from sim_juncs_gb300.fields import Fields

pytestmark = pytest.mark.gpu


def small_junction():
    return junction_instance(n=40, res=12.5)


def plant(f, value, steps_before=20):
    """Step to a save point (save_span 20), then overwrite Ex everywhere."""
    f.step(steps_before)
    f.synchronize()
    g = f.instances[0].grid
    f.set_array(_abi.EX, np.full((g.nz, g.ny, g.nx), value))


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_guard_trips_on_large_sample(lib, precision):
    f = Fields(small_junction(), precision)
    assert f.divergence() is None
    plant(f, 5000.0)
    f.step(3)                                  # the sample before step 20 trips the guard
    with pytest.raises(_abi.SJError) as e:
        f.synchronize()
    assert e.value.code == _abi.SJ_E_DIVERGED
    step, inst, mon, val = f.divergence()
    assert (step, inst) == (20, 0)
    assert abs(val) > 1000 and np.isfinite(val)
    done = f.steps_done
    with pytest.raises(_abi.SJError) as e:    # no further steps are queued
        f.step(1)
    assert e.value.code == _abi.SJ_E_DIVERGED
    assert f.steps_done == done
    assert np.max(np.abs(f.get_array(_abi.EX))) > 1000   # read-back still works
    f.set_divergence_guard(0)                  # off: clears the record, stepping resumes
    assert f.divergence() is None
    f.step(1)
    f.synchronize()
    assert f.steps_done == done + 1


def test_guard_trips_on_nan_and_can_be_raised(lib):
    f = Fields(small_junction(), "f64")
    plant(f, np.nan)
    f.step(1)
    with pytest.raises(_abi.SJError) as e:
        f.synchronize()
    assert e.value.code == _abi.SJ_E_DIVERGED
    assert np.isnan(f.divergence()[3])
    # a bound above the planted value lets the large sample through
    g = Fields(small_junction(), "f64")
    g.set_divergence_guard(1e7)
    plant(g, 5000.0)
    g.step(1)
    g.synchronize()
    assert g.divergence() is None
    with pytest.raises(_abi.SJError) as e:
        g.set_divergence_guard(-1.0)
    assert e.value.code == _abi.SJ_E_INVALID


def test_normal_run_does_not_trip(lib):
    f = Fields(junction_instance(n=48, res=15.0, amplitude=10.0), "f32")
    f.step(400)
    f.synchronize()
    assert f.divergence() is None
    assert np.max(np.abs(f.monitors())) < 1000


def test_tma_wait_runs_out_and_context_stays_usable(lib):
    inst = junction_instance(n=64, res=20.0)
    f = Fields(inst, "f32", "tma")
    f.step(2)
    f.synchronize()
    f.set_wait_limit(1_000_000)                # 1 ms
    f.set_test_stall(True)
    f.step(1)
    with pytest.raises(_abi.SJError) as e:
        f.synchronize()
    assert e.value.code == _abi.SJ_E_TIMEOUT
    f.close()
    # a fresh simulation on the same context runs and matches the fused schedule
    a = Fields(inst, "f32", "tma")
    b = Fields(inst, "f32", "fused")
    a.step(30)
    b.step(30)
    ea, eb = a.get_array(_abi.EX), b.get_array(_abi.EX)
    assert np.max(np.abs(ea - eb)) <= 1e-5 * np.max(np.abs(eb))
