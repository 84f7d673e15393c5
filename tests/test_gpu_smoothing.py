"""Stochastic sub-voxel smoothing on the device against the oracle: the
per-region fill counts the rasteriser writes at the E-component Yee points
(bit for bit), FP64 stepping of a smoothed scene (1e-10, the parity bar of
test_gpu_parity.py) in the fused and split schedules, FP32 against FP64, and
the host's rejection of what the one-byte material layout cannot hold."""
import numpy as np
import pytest

from oracle.oracle import OracleFields, rasterize_counts as oracle_counts
from sim_juncs_gb300 import _abi
from sim_juncs_gb300.fields import Fields, rasterize, rasterize_counts
from sim_juncs_gb300.geometry import Program, Sphere
from sim_juncs_gb300.spec import Grid, Region, Scene

from test_golden_cpu import G, golden_grid
from test_gpu_parity import TOL64, compare_fields, rel
from test_smoothing_cpu import smooth_scene, smoothed_junction

pytestmark = pytest.mark.gpu


def test_device_counts_match_oracle_two_roots(lib, oracle_lib):
    g = Grid(20, 18, 16, 0.08, origin=(0.0, 0.0, 0.0))
    sc = smooth_scene()
    got = rasterize_counts(g, sc)
    np.testing.assert_array_equal(got, oracle_counts(g, sc))
    assert got.max() == 17


@pytest.mark.parametrize("n,rad", [(1, 0.05), (1, 0.25), (4, 0.03)])
def test_device_counts_match_oracle_test_geom(lib, oracle_lib, n, rad):
    e = G["files"]["tests/test.geom"]
    root = e["roots"][0]
    sc = Scene([Region(Program(root["nodes"]), eps=root["eps"])], ambient_eps=1.0, smooth_n=n, smooth_rad=rad)
    g = golden_grid(e)
    got = rasterize_counts(g, sc)
    np.testing.assert_array_equal(got, oracle_counts(g, sc))
    assert 0 < int(((got > 0) & (got < 8 * n + 1)).sum())


def test_device_counts_without_smoothing_are_the_masks(lib):
    e = G["files"]["junctions/Au_SiO2_box/junc.geom"]
    g = golden_grid(e)
    sc = Scene([Region(Program(r["nodes"]), eps=r["eps"]) for r in e["roots"]], ambient_eps=e["ambient_eps"])
    counts = rasterize_counts(g, sc)
    masks = rasterize(g, sc)
    for r in range(len(sc.regions)):
        np.testing.assert_array_equal(counts[:, r], (masks >> r) & 1)


@pytest.mark.parametrize("schedule", ["fused", "split"])
def test_smoothed_junction_f64_matches_oracle(lib, oracle_lib, schedule):
    inst = smoothed_junction(n=48, res=20.0, smooth_n=1, smooth_rad=0.08)
    f = Fields(inst, "f64", schedule)
    o = OracleFields(inst)
    try:
        # classes: ranks of the points' count tuples, the same on both sides
        np.testing.assert_array_equal(f.class_map(), o.class_map())
        peak = 0.0
        for upto in (1, 10, 300):
            k = upto - o.steps_done
            f.step(k)
            o.step(k)
            peak = compare_fields(f, o, TOL64, peak=peak)
        assert rel(f.monitors(), o.monitors()) <= TOL64
    finally:
        o.close()


def test_smoothed_f32_within_1e4_of_f64(lib):
    inst = smoothed_junction(n=48, res=20.0, smooth_n=2, smooth_rad=0.05)
    a = Fields(inst, "f64")
    b = Fields(inst, "f32")
    a.step(600)
    b.step(600)
    ma, mb = a.monitors(), b.monitors()
    assert float(np.max(np.abs(ma))) > 0
    assert rel(mb, ma) <= 1e-4


def test_smoothing_changes_the_materials(lib):
    # the same scene with and without smoothing steps to different fields
    a = Fields(smoothed_junction(n=48, res=20.0, smooth_n=1, smooth_rad=0.08), "f64")
    plain = smoothed_junction(n=48, res=20.0)
    plain.material.smooth_n = 0
    b = Fields(plain, "f64")
    a.step(300)
    b.step(300)
    ea, eb = a.get_array(_abi.EX), b.get_array(_abi.EX)
    assert float(np.max(np.abs(eb))) > 0
    assert rel(ea, eb) > 1e-6


def test_smoothing_rejections(lib):
    inst = smoothed_junction(n=24, res=20.0)
    inst.material.combine = _abi.EPS_FIRST
    with pytest.raises(_abi.SJError) as e:
        Fields(inst, "f64")
    assert e.value.code == _abi.SJ_E_INVALID
    g = Grid(16, 16, 16, 0.05)
    with pytest.raises(_abi.SJError) as e:
        rasterize(g, smooth_scene())            # masks cannot carry fill counts
    assert e.value.code == _abi.SJ_E_INVALID
    # six overlapping spheres smoothed over 0.1: thousands of distinct point
    # classes, more than the one-byte class index holds
    inst = smoothed_junction(n=24, res=20.0)
    inst.material = Scene([Region(Sphere((0.3 + 0.08 * r, 0.6 - 0.05 * r, 0.5 + 0.03 * r), 0.25), eps=1.5 + 0.1 * r)
                           for r in range(6)], ambient_eps=1.0, smooth_n=3, smooth_rad=0.1)
    with pytest.raises(_abi.SJError) as e:
        Fields(inst, "f64")
    assert e.value.code == _abi.SJ_E_INVALID
    # the context stays usable
    f = Fields(smoothed_junction(n=24, res=20.0), "f64")
    f.step(5)
    assert f.steps_done == 5
