"""Layout of the monitor output file (bound_geom::save_field_times,
src/disp.cpp:758-923) as the reference's own test reads it
(src/main_test.cpp:1884-2028, "Test running with a very small system"), plus
the writer's quirks that test does not reach.

The reference test's configuration (tests/run.conf with the test's overrides,
tests/run.geom): um_scale (l_per_um) 2, length 2, PML 1, so tot_len 4; two
monitors at (1, 1, 1) and (um_to_l(1), tot_len, 1.1) = (2, 4, 1.1) in one
cluster; save_span 1.  meep cannot run here, so the series are synthetic; the
layout does not depend on their values.
"""
import numpy as np
import pytest

from sim_juncs_gb300 import field_samples as fsm

LOCS = [(1.0, 1.0, 1.0), (2.0, 4.0, 1.1)]
CGS = {"l_per_um": 2.0, "sim_length": 2.0, "pml_thickness": 1.0, "tot_len": 4.0}


def series(n, n_mon, seed=0):
    rng = np.random.default_rng(seed)
    s = rng.standard_normal((n_mon, n))
    return s, np.fft.fft(s[:, : 1 << int(np.log2(n))], axis=1)


def test_reference_test_assertions(tmp_path):
    n_t, span = 64, 1
    s, f = series(n_t, 2)
    tree = fsm.build_tree(list(s), list(f), LOCS, [2], ttot=n_t * 0.1, n_t_pts=n_t, save_span=span,
                          sources=[(0.7, 10.0, 0.0, 0.0, 20.0, 1.0)], cgs_params=CGS, um_scale=2.0)
    path = fsm.write(str(tmp_path / "field_samples.h5"), tree)
    t = fsm.read(path)
    tb = t["info/time_bounds"]
    assert tb.shape == (3,) and tb[0] == 0.0 and tb[1] > 0.0 and 0.0 < tb[2] < tb[1]
    assert t["info/n_clusters"].shape == (1,) and int(t["info/n_clusters"][0]) == 1
    for name, v in CGS.items():
        d = t[f"info/cgs_params/{name}"]
        assert d.shape == (1,) and d[0] == v
    loc = t["cluster_0/locations"]
    assert loc.shape == (2,)
    for i, p in enumerate(LOCS):
        assert (loc[i]["x"], loc[i]["y"], loc[i]["z"]) == pytest.approx(p)
    for j in range(2):
        fd, td = t[f"cluster_0/point_{j}/frequency"], t[f"cluster_0/point_{j}/time"]
        assert fd.size > 0 and td.size >= fd.size
        assert td.size == s[j].size
        np.testing.assert_array_equal(td["Re"], s[j])
        np.testing.assert_array_equal(td["Im"], 0.0)
        np.testing.assert_array_equal(fd["Re"] + 1j * fd["Im"], f[j])
    src = t["info/sources"]
    assert src.dtype.names == ("wavelen", "width", "phase", "start_time", "end_time", "amplitude")
    assert src[0]["end_time"] == 20.0
    assert t["info/n_time_points"][0] == n_t


def test_time_bounds_values():
    tree = fsm.build_tree([np.zeros(5)], [np.zeros(4, complex)], [(0, 0, 0)], [1], ttot=3.0, n_t_pts=100,
                          save_span=20, um_scale=2.0)
    t1 = 3.0 / (0.299792458 * 2.0)
    np.testing.assert_allclose(tree["info/time_bounds"], [0.0, t1, t1 * 20 / 100], rtol=1e-15)


def test_extra_cluster_and_truncated_time_series():
    # 3 clusters of 4 monitors: cluster_3 is the extra, empty one; 101 steps
    # at save_span 20 record 6 samples but the time datasets keep 101 // 20 = 5
    s, f = series(6, 12)
    f = np.fft.fft(s[:, :4], axis=1)
    locs = [(float(q), 0.0, 0.0) for q in range(12)]
    tree = fsm.build_tree(list(s), list(f), locs, [4, 8, 12], ttot=1.0, n_t_pts=101, save_span=20)
    assert int(tree["info/n_time_points"][0]) == 5
    assert tree["cluster_3/locations"].shape == (0,)
    assert not any(k.startswith("cluster_3/point") for k in tree)
    # point numbers run over all monitors, two digits for 12 monitors
    assert "cluster_0/point_03/time" in tree and "cluster_1/point_04/time" in tree
    assert "cluster_2/point_11/frequency" in tree
    td = tree["cluster_2/point_11/time"]
    assert td.size == 5
    np.testing.assert_array_equal(td["Re"], s[11][:5])
    assert tree["cluster_2/point_11/frequency"].size == 4
    for k in range(3):
        assert tree[f"cluster_{k}/locations"].shape == (4,)


def test_cluster_number_width_and_short_series_stop():
    # 10 clusters: two-digit cluster names (cluster_00 .. cluster_10); a
    # monitor with fewer than 2 samples stops the writing of points there
    s = [np.arange(3.0) + q for q in range(10)]
    s[6] = np.array([1.0])
    f = [np.fft.fft(x[:2]) if x.size >= 2 else np.zeros(2, complex) for x in s]
    tree = fsm.build_tree(s, f, [(0, 0, q) for q in range(10)], list(range(1, 11)), ttot=1.0, n_t_pts=3,
                          save_span=1)
    assert "cluster_00/locations" in tree and "cluster_10/locations" in tree
    assert "cluster_05/point_05/time" in tree
    assert not any("point_06" in k or "point_07" in k or "point_09" in k for k in tree)


def test_digit_count_follows_the_reference_arithmetic():
    # (size_t)(log(n) / log(10)) + 1 in double arithmetic: 1000 monitors give
    # 3 digits there (log(1000)/log(10) rounds just below 3), not 4
    assert fsm._digits(9) == 1 and fsm._digits(10) == 2 and fsm._digits(99) == 2
    assert fsm._digits(1000) == 3
