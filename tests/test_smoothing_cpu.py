"""Stochastic sub-voxel smoothing (cgs_material_function, src/disp.cpp:56-112,
264-283) on the CPU: the sample offsets the library generates on the host
against the oracle's restatement, their structure, the known answers of the
reference's own in_bound test (which runs with the header defaults smooth_n = 1,
smooth_rad = 0.05, src/disp.hpp:68-70), and the oracle's per-region counts
against an independent count through the CSG evaluator."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle
from sim_juncs_gb300 import _abi
from sim_juncs_gb300.geometry import Box, Program, Sphere, Union, as_program
from sim_juncs_gb300.spec import Grid, Region, Scene

from test_golden_cpu import IN_BOUND_POINTS, G, golden_scene


def product_points(lib, n, rad):
    out = np.zeros((8 * n, 3), dtype=np.float64)
    rc = lib.sj_smooth_points(n, rad, out.ctypes.data_as(C.POINTER(C.c_double)), out.size)
    assert rc == 0
    return out


@pytest.mark.parametrize("n,rad", [(1, 0.05), (1, 0.25), (3, 0.05), (31, 0.1)])
def test_host_offsets_match_oracle(lib, n, rad):
    got = product_points(lib, n, rad)
    want = oracle.smooth_points(n, rad)
    assert got.shape == (8 * n, 3)
    np.testing.assert_array_equal(got, want)


def test_offsets_structure():
    p = oracle.smooth_points(4, 0.05).reshape(4, 8, 3)
    for d in range(4):
        base = np.abs(p[d, 7])          # the all-positive reflection comes last
        assert p[d, 7].tolist() == [p[d, 7, 0], p[d, 7, 1], p[d, 7, 2]]
        np.testing.assert_array_equal(np.abs(p[d]), np.broadcast_to(base, (8, 3)))
        # y is written as r sin(theta) cos(phi), the same expression as x
        assert abs(p[d, 7, 0]) == abs(p[d, 7, 1])
        # sign pattern: x outermost, z innermost, negative first
        signs = np.sign(p[d]) * np.sign(p[d, 7])
        assert signs[:, 0].tolist() == [-1, -1, -1, -1, 1, 1, 1, 1]
        assert signs[:, 1].tolist() == [-1, -1, 1, 1, -1, -1, 1, 1]
        assert signs[:, 2].tolist() == [-1, 1, -1, 1, -1, 1, -1, 1]
    # the radial draw is N(0, rad): a sample of 31 draws stays within a few rad
    big = oracle.smooth_points(31, 0.1)
    r = np.linalg.norm(big, axis=1)
    assert 0 < float(np.median(r)) < 0.3 and float(r.max()) < 0.6


def test_offsets_depend_only_on_n_and_rad():
    a = oracle.smooth_points(2, 0.05)
    b = oracle.smooth_points(5, 0.05)[:16]
    np.testing.assert_array_equal(a, b)     # one sequence, drawn in order
    c = oracle.smooth_points(2, 0.1)
    # the uniform draws are shared, the radius scales with rad
    np.testing.assert_allclose(c, 2 * a, rtol=1e-14, atol=0)


def test_in_bound_with_smoothing_known_answers():
    # src/main_test.cpp:1612-1640: cgs_material_function mat_func(root) takes
    # smooth_n = 1 and smooth_rad = 0.05 from its defaults; in_bound is 3.5 at
    # the first three points of tests/test.geom and 1.0 at the others
    e = G["files"]["tests/test.geom"]
    pts = np.array(IN_BOUND_POINTS)
    root = e["roots"][0]
    for n, rad in ((1, 0.05), (0, 0.05)):
        sc = Scene([Region(Program(root["nodes"]), eps=root["eps"])], ambient_eps=1.0, smooth_n=n,
                   smooth_rad=rad)
        assert root["eps"] == 3.5
        assert oracle.in_bound(sc, pts).tolist() == [3.5, 3.5, 3.5, 1.0, 1.0, 1.0]


def test_smoothing_counts_at_the_inclusion_test_point_near_a_face():
    # (.65, .45, .41) of the in() test (src/main_test.cpp:1558) lies 0.01 above
    # the z = 0.4 face: the point is inside, and of the 8 reflections of the
    # first draw (|dz| = 0.0131) the 4 with dz < 0 fall below the face
    e = G["files"]["tests/test.geom"]
    prog = Program(e["roots"][0]["nodes"]).program()
    offs = oracle.smooth_points(1, 0.05)
    p = np.array([0.65, 0.45, 0.41])
    assert abs(offs[0, 2]) > 0.01
    assert oracle.csg_in(prog, p[None] + offs).tolist() == [int(d > 0) for d in offs[:, 2]]


def test_in_bound_fraction_at_a_face():
    # a point on a box face: about half the samples fall inside, and in_bound
    # is ambient + (s - ambient) * count / 9
    sc = Scene([Region(Box((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), eps=3.0)], ambient_eps=1.0, smooth_n=1,
               smooth_rad=0.05)
    v = oracle.in_bound(sc, np.array([[1.0, 0.5, 0.5], [0.5, 0.5, 0.5], [2.0, 2.0, 2.0]]))
    cnt = (v[0] - 1.0) / 2.0 * 9
    assert abs(cnt - round(cnt)) < 1e-12 and 1 <= round(cnt) <= 8
    assert v[1] == 3.0 and v[2] == 1.0


def independent_counts(grid, scene):
    """Counts through the oracle's csg_in at r and at r + d_j."""
    offs = oracle.smooth_points(scene.smooth_n, scene.smooth_rad) if scene.smooth_n else np.zeros((0, 3))
    idx = [np.arange(n, dtype=np.float64) for n in (grid.nx, grid.ny, grid.nz)]
    out = np.zeros((3, len(scene.regions), grid.nz, grid.ny, grid.nx), dtype=np.int64)
    for c in range(3):
        ax = [grid.origin[a] + (idx[a] + (0.5 if c == a else 0.0)) * grid.dx for a in range(3)]
        z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
        pts = np.stack([x, y, z], axis=-1).reshape(-1, 3)
        for r, reg in enumerate(scene.regions):
            prog = as_program(reg.obj)
            cnt = oracle.csg_in(prog, pts).astype(np.int64)
            for d in offs:
                cnt += oracle.csg_in(prog, pts + d)
            out[c, r] = cnt.reshape(grid.nz, grid.ny, grid.nx)
    return out


def smooth_scene():
    return Scene([Region(Union(Box((0.3, 0.3, 0.35), (0.9, 0.7, 0.5)), Sphere((1.0, 0.8, 0.9), 0.35)), eps=2.5),
                  Region(Box((0.0, 0.0, 0.0), (1.6, 1.6, 0.4)), eps=2.13)],
                 ambient_eps=1.0, smooth_n=2, smooth_rad=0.06)


def test_oracle_counts_match_independent_count():
    g = Grid(20, 18, 16, 0.08, origin=(0.0, 0.0, 0.0))
    sc = smooth_scene()
    got = oracle.rasterize_counts(g, sc)
    want = independent_counts(g, sc)
    np.testing.assert_array_equal(got.astype(np.int64), want)
    assert got.max() == 17 and got.min() == 0
    mid = (got > 0) & (got < 17)
    assert mid.sum() > 100          # the smoothing band is populated


def test_oracle_counts_without_smoothing_are_the_masks():
    e = G["files"]["tests/test.geom"]
    g = Grid(24, 24, 24, 1.0 / 24, origin=(0.0, 0.0, 0.0))
    sc = golden_scene(e)
    counts = oracle.rasterize_counts(g, sc)
    masks = oracle.rasterize(g, sc)
    for r in range(len(sc.regions)):
        np.testing.assert_array_equal(counts[:, r], (masks >> r) & 1)


def test_host_rejects_bad_smoothing_arguments(lib):
    out = np.zeros(24 * 40)
    ptr = out.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.sj_smooth_points(32, 0.05, ptr, out.size) == _abi.SJ_E_INVALID
    assert lib.sj_smooth_points(1, 0.0, ptr, out.size) == _abi.SJ_E_INVALID
    assert lib.sj_smooth_points(2, 0.05, ptr, 47) == _abi.SJ_E_RANGE
    assert lib.sj_smooth_points(0, 0.05, ptr, 0) == 0


def smoothed_junction(n=24, res=20.0, smooth_n=1, smooth_rad=0.08):
    from sim_juncs_gb300.configs import junction_instance
    inst = junction_instance(n=n, res=res)
    reg = inst.material.regions[0]
    inst.material = Scene([Region(reg.obj, eps=1.0, susceptibilities=reg.susceptibilities),
                           Region(Box((0.0, 0.0, 0.0), (n / res, n / res, 0.5 * n / res - 0.05)), eps=2.13)],
                          ambient_eps=1.0, smooth_n=smooth_n, smooth_rad=smooth_rad)
    return inst


def test_oracle_classes_are_ranked_count_tuples():
    inst = smoothed_junction()
    f = oracle.OracleFields(inst)
    try:
        cls = f.class_map()
    finally:
        f.close()
    counts = oracle.rasterize_counts(inst.grid, inst.material).astype(np.int64)
    key = counts[:, 0] | (counts[:, 1] << 8)
    uniq = np.unique(key)
    assert len(uniq) > 4                               # fractional fills present
    np.testing.assert_array_equal(cls, np.searchsorted(uniq, key))


def test_scene_smoothing_fields_reach_the_descriptor():
    from sim_juncs_gb300.spec import scene_to_c
    sc, h = scene_to_c(Scene([Region(Box((0, 0, 0), (1, 1, 1)), eps=2.0)], smooth_n=3, smooth_rad=0.2))
    assert (sc.contents.smooth_n, sc.contents.smooth_rad) == (3, 0.2)
    sc, h = scene_to_c(Scene([Region(Box((0, 0, 0), (1, 1, 1)), eps=2.0)]))
    assert (sc.contents.smooth_n, sc.contents.smooth_rad) == (0, 0.05)    # off by default


@pytest.mark.parametrize("change,why", [
    (dict(smooth_n=32), "smooth_n"),
    (dict(smooth_n=-1), "smooth_n"),
    (dict(smooth_rad=0.0), "smooth_rad"),
    (dict(smooth_rad=float("nan")), "smooth_rad"),
    (dict(combine=_abi.EPS_FIRST), "SJ_EPS_SUM"),
])
def test_host_validates_smoothing_before_device_work(lib, change, why):
    # the scene check runs on the host before any CUDA call, so it runs here
    from sim_juncs_gb300.spec import scene_to_c
    kw = dict(smooth_n=1, smooth_rad=0.05)
    kw.update({k: v for k, v in change.items() if k != "combine"})
    sc_py = Scene([Region(Box((0, 0, 0), (1, 1, 1)), eps=2.0)], combine=change.get("combine", _abi.EPS_SUM), **kw)
    sc, h = scene_to_c(sc_py)
    g = Grid(4, 4, 4, 0.25).to_c()
    out = np.zeros(3 * 4 * 4 * 4, dtype=np.uint8)
    rc = lib.sj_rasterize_counts(C.byref(g), sc, out.ctypes.data_as(C.POINTER(C.c_uint8)))
    assert rc == _abi.SJ_E_INVALID
    assert why in lib.sj_last_error(None).decode()
