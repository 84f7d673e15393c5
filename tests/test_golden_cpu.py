"""The oracle against golden vectors recorded from the reference's own code.

tests/golden/cgs_reference.json comes from tests/golden/make_golden.py,
which runs the reference's CGS parser and composite_object::in (compiled
unmodified, oracle/_ref) on its tests/*.geom and junctions/*/junc.geom
files.  These tests pin the oracle's CSG evaluation and rasteriser, the
eps sum of in_bound and the susceptibility mapping to those answers, and
check the literal values the reference's own tests assert
(src/main_test.cpp).  The device rasteriser is checked against the same
vectors in test_gpu_golden.py.
"""
import base64
import json
import os
import zlib

import numpy as np
import pytest

from oracle import oracle
from sim_juncs_gb300 import _abi
from sim_juncs_gb300.configs import gaussian_pulse
from sim_juncs_gb300.geometry import Program
from sim_juncs_gb300.spec import Grid, Region, Scene, Source, Susceptibility, reference_grid, scene_to_c

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "cgs_reference.json")


def golden():
    with open(GOLDEN) as fh:
        return json.load(fh)


G = golden()
ROOTS = [(name, r) for name, e in sorted(G["files"].items()) for r in range(len(e["roots"]))]


def unpack(bits, n):
    return np.unpackbits(np.frombuffer(zlib.decompress(base64.b64decode(bits)), dtype=np.uint8))[:n]


def yee_points(origin, dx, n):
    """E-component sample points of an n^3 grid, ordered [c][k][j][i] (the
    generator's and the rasteriser's order)."""
    idx = np.arange(n, dtype=np.float64)
    pts = []
    for c in range(3):
        ax = [origin[a] + (idx + (0.5 if c == a else 0.0)) * dx for a in range(3)]
        z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
        pts.append(np.stack([x, y, z], axis=-1).reshape(-1, 3))
    return np.concatenate(pts)


def golden_grid(entry):
    g = entry["grid"]
    return Grid(g["n"], g["n"], g["n"], g["dx"], origin=tuple(g["origin"]))


def golden_scene(entry):
    return Scene([Region(Program(r["nodes"]), eps=r["eps"]) for r in entry["roots"]],
                 ambient_eps=entry["ambient_eps"])


def test_golden_covers_the_reference_files():
    names = set(G["files"])
    assert "tests/test.geom" in names
    assert "junctions/Au_SiO2_box/junc.geom" in names
    assert "junctions/Au_SiO2_bowtie/junc.geom" in names
    # the box junction: two roots (Au pair, SiO2 substrate), both non-empty on the grid
    box = G["files"]["junctions/Au_SiO2_box/junc.geom"]["roots"]
    assert len(box) == 2 and all(r["n_inside"] > 0 for r in box)


@pytest.mark.parametrize("name,root", ROOTS)
def test_oracle_csg_matches_reference_in(name, root):
    e = G["files"][name]
    g = e["grid"]
    r = e["roots"][root]
    pts = yee_points(g["origin"], g["dx"], g["n"])
    want = unpack(r["inside_bits"], len(pts))
    got = oracle.csg_in(Program(r["nodes"]).program(), pts)
    assert int(want.sum()) == r["n_inside"]
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("name", sorted(G["files"]))
def test_oracle_rasterizer_matches_reference_in(name):
    e = G["files"][name]
    n = e["grid"]["n"]
    masks = oracle.rasterize(golden_grid(e), golden_scene(e))
    for r, root in enumerate(e["roots"]):
        want = unpack(root["inside_bits"], 3 * n ** 3).reshape(3, n, n, n)
        np.testing.assert_array_equal((masks >> r) & 1, want)


def test_reference_inclusion_test_points():
    # src/main_test.cpp:1555-1564: in() at six points of tests/test.geom
    e = G["files"]["tests/test.geom"]
    tp = e["test_points"]
    assert tp["inside"] == [1, 1, 1, 0, 0, 0]
    got = oracle.csg_in(Program(e["roots"][0]["nodes"]).program(), np.array(tp["points"]))
    assert got.tolist() == tp["inside"]


# the points of the reference's in_bound test (src/main_test.cpp:1629-1634);
# the third differs from the in() test's (.65, .45, .41)
IN_BOUND_POINTS = [(.45, .45, .45), (.45, .41, .6), (.65, .45, .45), (.71, .51, .51), (.55, .45, .45),
                   (.55, .41, .85)]


def test_in_bound_sum_values():
    # src/main_test.cpp:1635-1640: in_bound = 3.5 at the first three points,
    # 1.0 at the others; in_bound (src/disp.cpp:264-283 with smooth_n = 0)
    # sums def + (eps_root - def) * in(r) over the roots
    e = G["files"]["tests/test.geom"]
    pts = np.array(IN_BOUND_POINTS)
    amb = 1.0
    val = np.zeros(len(pts))
    for r in e["roots"]:
        val += amb + (r["eps"] - amb) * oracle.csg_in(Program(r["nodes"]).program(), pts)
    assert val.tolist() == [3.5, 3.5, 3.5, 1.0, 1.0, 1.0]


def test_susceptibilities_of_test_geom():
    # src/main_test.cpp:1767-1776 (the C++ test compares doubles, hence float())
    poles = G["files"]["tests/test.geom"]["roots"][0]["poles"]
    assert [(p["omega_0"], p["gamma"], p["sigma"], p["drude"]) for p in poles] == [
        (1.0, 0.48, 68.5971845, True), (8.0, 0.816, float(452848600800781300), True)]
    # what the builder receives for them: sj_pole {omega_0, gamma, drude} and
    # sigma per region
    sus = [Susceptibility(p["omega_0"], p["gamma"], p["sigma"], drude=p["drude"]) for p in poles]
    sc, holder = scene_to_c(Scene([Region(Program(G["files"]["tests/test.geom"]["roots"][0]["nodes"]),
                                          eps=3.5, susceptibilities=sus)]))
    reg = sc.contents.regions[0]
    assert reg.n_poles == 2
    for q, p in enumerate(poles):
        c = reg.poles[q]
        assert (c.omega_0, c.gamma, bool(c.drude), reg.sigma[q]) == (p["omega_0"], p["gamma"], p["drude"],
                                                                      p["sigma"])


def test_gaussian_source_timing():
    # src/main_test.cpp:1785-1791 (tests/test.geom): width 3, cutoff 6,
    # start 5.2 -> end_time = start + 2 cutoff width = 41.2
    src = gaussian_pulse(_abi.EY, 0.2, 0.4, 1 / 1.333333, fwidth=1 / 3.0, cutoff=6.0, start_time=5.2)
    assert src.width == pytest.approx(3.0)
    assert src.end_time == pytest.approx(41.2)
    # src/main_test.cpp:1876-1881: frequency 1, width 2 -> omega 2 pi, fwidth 0.5
    s2 = Source(_abi.EX, 1.0, 2.0, 0.0, 2 * 5 * 2.0, (0, 0, 0), (1, 1, 0))
    assert 2 * np.pi * s2.frequency == pytest.approx(6.283185307)
    assert 1 / s2.width == pytest.approx(0.5)


def reference_spectrum(x):
    """Restatement of the reference's fft (src/data_utils.cpp:413-427): the
    first N' = 2^floor(log2 N) samples, phase step 2 pi / N, bins
    k = -N'/2 .. N'/2 - 1 stored at k mod N'."""
    import math
    x = np.asarray(x, dtype=np.complex128)
    n = len(x)
    npow = 1 << int(math.log(n) / math.log(2))
    out = np.zeros(npow, dtype=np.complex128)
    if npow > 1:
        k = np.arange(-npow // 2, npow // 2)
        m = np.arange(npow)
        out[k % npow] = (x[:npow][None, :] * np.exp(-2j * np.pi * np.outer(k, m) / n)).sum(axis=1)
    return out


def test_spectrum_restatement_matches_reference_fft():
    with open(os.path.join(os.path.dirname(__file__), "golden", "fft_reference.json")) as fh:
        cases = json.load(fh)["cases"]
    assert {c["n"] for c in cases} >= {1, 8, 64, 100, 1000}
    for c in cases:
        want = np.array(c["out"][0::2]) + 1j * np.array(c["out"][1::2])
        got = reference_spectrum(np.array(c["re"]) + 1j * np.array(c["im"]))
        assert len(got) == c["out_len"], c["n"]
        scale = max(1.0, float(np.max(np.abs(want))))
        assert float(np.max(np.abs(got - want))) <= 1e-12 * scale, c["n"]


def test_reference_grid_rounding():
    # src/main_test.cpp:1658 (tests/test.conf: length 16, pml 2, resolution
    # 1.5 -> 31 points, 1.55 px/um) and :1703 (--length 9, pml 2,
    # --grid-res 3 -> 41 points, 3.1538 px/um); the junction cell of 3.2 um
    # at 20 px/um rounds to 65 points
    g, res = reference_grid(16.0, 2.0, 1.5)
    assert (g.nx, res) == (31, 1.55)
    g, res = reference_grid(9.0, 2.0, 3.0)
    assert g.nx == 41 and res == pytest.approx(3.1538, abs=5e-5)
    g, res = reference_grid(2.2, 0.5, 20.0)
    assert g.nx == 65 and g.dt == pytest.approx(0.5 * g.dx)
    g, res = reference_grid(2.2, 0.5, 20.0, grid_num=64)   # an explicit grid number is kept
    assert g.nx == 64 and res == 20.0


VOLUMES = os.path.join(os.path.dirname(__file__), "golden", "volume_reference.json")
# src/main_test.cpp:1483-1485 (the sphere's 4/3 written 1.33333 there)
VOLUME_KAT = {"sphere": 1.33333 * np.pi * 0.125, "plane": 5.0 / 6, "cylinder": np.pi * 0.125}


def volume_primitives():
    from sim_juncs_gb300.geometry import Cylinder, Plane, Sphere
    # src/main_test.cpp:1452-1459
    return {"sphere": Sphere((0.5, 0.5, 0.5), 0.5),
            "cylinder": Cylinder((0.5, 0.5, 0.5), 0.5, 0.5, 0.5),
            "plane": Plane((1.0, 1.0, 0.0), (0.0, 1.0, 1.0), (1.0, 0.0, 1.0))}


def volume_points():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    with open(VOLUMES) as fh:
        v = json.load(fh)
    return v, mg.lcg_points(v["n"], v["seed"])


def test_reference_volume_test_primitives():
    # src/main_test.cpp:1448-1489: sampled volume fractions of a sphere, a
    # cylinder and a plane within EPSILON = 0.01 of the exact volumes; the
    # oracle answers the reference's own in() at every sample point
    from sim_juncs_gb300.geometry import as_program
    v, pts = volume_points()
    assert pts.shape == (10000, 3) and 0.0 <= pts.min() and pts.max() <= 1.0
    for name, obj in volume_primitives().items():
        want = unpack(v["primitives"][name]["inside_bits"], len(pts))
        got = oracle.csg_in(as_program(obj), pts)
        np.testing.assert_array_equal(got, want)
        frac = float(got.mean())
        assert abs(VOLUME_KAT[name] - frac) / VOLUME_KAT[name] < 0.01, (name, frac)


PHASES = os.path.join(os.path.dirname(__file__), "golden", "phases_reference.json")


def test_phases_fixture_is_complete_and_regenerable():
    # tests/golden/make_phases_golden.py ran the reference's own CEP/envelope
    # extraction (scripts/phases.py, signal, as opt_pulse_full calls it) on
    # seeded synthetic pulses and the oracle's junction monitors; each entry
    # holds the reference's results or the exception it raised
    import importlib.util
    with open(PHASES) as fh:
        ph = json.load(fh)
    keys = {"f0", "phi", "t0_corr", "amp", "mu", "sig", "skew"}
    kinds = {s["kind"] for s in ph["series"]}
    assert kinds == {"synthetic", "junction64"}
    for s in ph["series"]:
        r = s["reference"]
        assert len(s["t"]) == len(s["v"]) > 0
        assert ("error" in r) or (keys <= set(r) and all(np.isfinite(r[k]).all() for k in keys))
    assert sum("error" not in s["reference"] for s in ph["series"]) >= 16
    spec = importlib.util.spec_from_file_location(
        "make_phases_golden", os.path.join(os.path.dirname(__file__), "golden", "make_phases_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    synth = mg.synthetic_series(np.random.default_rng(ph["seed"]))
    got = [s for s in ph["series"] if s["kind"] == "synthetic"]
    assert len(synth) == len(got)
    for a, b in zip(synth, got):
        np.testing.assert_array_equal(np.array(a["v"]), np.array(b["v"]))
