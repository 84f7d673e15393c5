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
