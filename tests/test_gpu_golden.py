"""The device rasteriser against golden vectors recorded from the reference's
own composite_object::in (tests/golden/cgs_reference.json; see
tests/golden/make_golden.py): for every root of every reference geometry
file, the class bits the GPU writes at the E-component Yee points of the
golden grid equal the reference's answers bit for bit."""
import numpy as np
import pytest

from sim_juncs_gb300.fields import rasterize

from test_golden_cpu import G, golden_grid, golden_scene, unpack

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(G["files"]))
def test_device_rasterizer_matches_reference_in(lib, name):
    e = G["files"][name]
    n = e["grid"]["n"]
    masks = rasterize(golden_grid(e), golden_scene(e))
    assert masks.shape == (3, n, n, n)
    for r, root in enumerate(e["roots"]):
        want = unpack(root["inside_bits"], 3 * n ** 3).reshape(3, n, n, n)
        np.testing.assert_array_equal((masks >> r) & 1, want)


def test_device_monitor_spectrum(lib):
    # the spectrum save_field_times writes, computed on the device, against
    # the restatement pinned to the reference's fft
    from sim_juncs_gb300.configs import junction_instance
    from sim_juncs_gb300.fields import Fields
    from test_golden_cpu import reference_spectrum
    f = Fields(junction_instance(), "f32")
    for steps in (7 * 20, 2000):  # 7 samples (4 bins), 100 samples (64 bins)
        f.step(steps - f.steps_done)
        mon = f.monitors()
        spec = f.monitor_spectrum()
        assert spec.shape == (mon.shape[0], len(reference_spectrum(mon[0])))
        for m in range(mon.shape[0]):
            want = reference_spectrum(mon[m])
            assert float(np.max(np.abs(spec[m] - want))) <= 1e-12 * max(1e-300, float(np.max(np.abs(want))))


def test_device_rasterizer_reference_volume_primitives(lib, oracle_lib):
    # the sphere, cylinder and plane of src/main_test.cpp:1448-1489 rasterised
    # on the unit cube: the device's masks equal the oracle's, and the filled
    # fraction of each is within the test's EPSILON = 0.01 of its volume
    from oracle.oracle import rasterize as oracle_rasterize
    from sim_juncs_gb300.spec import Grid, Region, Scene
    from test_golden_cpu import VOLUME_KAT, volume_primitives
    n = 96
    g = Grid(n, n, n, 1.0 / n, origin=(0.0, 0.0, 0.0))
    prims = volume_primitives()
    sc = Scene([Region(o, eps=2.0) for o in prims.values()])
    masks = rasterize(g, sc)
    np.testing.assert_array_equal(masks, oracle_rasterize(g, sc))
    for r, name in enumerate(prims):
        frac = float(((masks >> r) & 1).mean())
        assert abs(frac - VOLUME_KAT[name]) / VOLUME_KAT[name] < 0.01, (name, frac)
