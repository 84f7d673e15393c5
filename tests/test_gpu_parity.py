"""Parity of the CUDA stepper with the FP64 CPU oracle, through the C ABI.

Bar: FP64 fields within 1e-10 of the oracle relative to the largest field
magnitude the run has reached so far (a pulse that has decayed 1e6-fold in
the PML carries the absolute rounding of its peak); FP64 monitor series and
DFT sums within 1e-10 relative to their own maximum; FP32 gap monitors and
DFTs within 1e-4 of FP64 (the target for the FP32 path).
"""
import math

import numpy as np
import pytest

from oracle.oracle import OracleFields, rasterize as oracle_rasterize
from sim_juncs_gb300 import _abi
from sim_juncs_gb300.configs import bowtie_instance, junction_instance, sweep_instances
from sim_juncs_gb300.fields import Fields, rasterize
from sim_juncs_gb300.spec import Grid

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 1e-4


def rel(a, b):
    scale = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / scale) if scale > 0 else float(np.max(np.abs(a)))


def compare_fields(f, o, tol, inst=0, peak=0.0):
    """Every component within tol of the oracle, relative to the largest
    field magnitude over all six components and over the run so far (`peak`;
    a component that symmetry keeps at roundoff level has no meaningful
    relative error of its own).  Returns the updated peak."""
    gs = [f.get_array(c, inst) for c in range(6)]
    rs = [o.get_array(c) for c in range(6)]
    scale = max([peak] + [float(np.max(np.abs(r))) for r in rs])
    assert scale > 0
    for c in range(6):
        err = float(np.max(np.abs(gs[c] - rs[c]))) / scale
        assert err <= tol, (c, err)
    return scale


@pytest.mark.parametrize("schedule", ["split", "fused"])
def test_junction_f64_matches_oracle(lib, oracle_lib, schedule):
    inst = junction_instance()            # 64^3, 20 px/um, 2000 steps
    f = Fields(inst, "f64", schedule)
    o = OracleFields(inst)
    peak = 0.0
    for upto in (1, 10, 400, 2000):
        n = upto - o.steps_done
        f.step(n)
        o.step(n)
        peak = compare_fields(f, o, TOL64, peak=peak)
    assert f.steps_done == 2000
    mg, mo = f.monitors(), o.monitors()
    assert mg.shape == mo.shape == (8, 100)
    assert rel(mg, mo) <= TOL64
    dg, do = f.dft(), o.dft()
    assert rel(dg, do) <= TOL64
    assert np.max(np.abs(mo[:4])) > 0.1           # the gap is lit


def test_junction_class_map_matches_oracle(lib, oracle_lib):
    inst = junction_instance()
    f = Fields(inst, "f64", "split")
    o = OracleFields(inst)
    np.testing.assert_array_equal(f.class_map(), o.class_map())


@pytest.mark.parametrize("n,res", [(64, 20.0), (48, 15.0)])
def test_rasterizer_matches_oracle_junction(lib, oracle_lib, n, res):
    inst = junction_instance(n=n, res=res)
    g = Grid(n, n, n, 1.0 / res)
    np.testing.assert_array_equal(rasterize(g, inst.material), oracle_rasterize(g, inst.material))


def test_rasterizer_matches_oracle_bowtie(lib, oracle_lib):
    inst = bowtie_instance(nx=128, ny=128, nz=96, res=10.0)
    g = inst.grid
    dev = rasterize(g, inst.material)
    ref = oracle_rasterize(g, inst.material)
    np.testing.assert_array_equal(dev, ref)
    assert (dev & 1).any() and (dev & 2).any()


@pytest.mark.parametrize("schedule", ["split", "fused"])
def test_f32_gap_field_within_1e4_of_f64(lib, schedule):
    inst = junction_instance()
    f64 = Fields(inst, "f64", schedule)
    f32 = Fields(inst, "f32", schedule)
    f64.step(2000)
    f32.step(2000)
    m64, m32 = f64.monitors(), f32.monitors()
    assert rel(m32[:4], m64[:4]) <= TOL32, rel(m32[:4], m64[:4])
    assert rel(f32.dft()[:4], f64.dft()[:4]) <= TOL32


@pytest.mark.parametrize("schedule", ["split", "fused"])
def test_batch_of_uneven_grids_matches_oracle(lib, oracle_lib, schedule):
    insts = [junction_instance(n=n, res=r, phase=ph, amplitude=a, probe_components=("Ex", "Ez"))
             for (n, r, ph, a) in ((32, 10.0, 0.3, 2.0), (45, 14.0, 1.7, 0.5), (40, 12.5, 4.0, 1.0))]
    f = Fields(insts, "f64", schedule)
    f.step(300)
    for q, inst in enumerate(insts):
        o = OracleFields(inst)
        o.step(300)
        assert rel(f.monitors(q), o.monitors()) <= TOL64
        assert rel(f.dft(q), o.dft()) <= TOL64
        compare_fields(f, o, TOL64, q)


@pytest.mark.parametrize("schedule", ["split", "fused"])
def test_graph_replay_matches_plain_launches(lib, schedule):
    inst = junction_instance(n=40, res=12.5)
    a = Fields(inst, "f32", schedule)
    b = Fields(inst, "f32", schedule)
    a.step(173)
    b.step_graph(173, chunk=25)
    assert a.steps_done == b.steps_done == 173
    for c in range(6):
        np.testing.assert_array_equal(a.get_array(c), b.get_array(c))
    np.testing.assert_array_equal(a.monitors(), b.monitors())


@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("f32", 1e-5)])
def test_fused_and_split_agree(lib, precision, tol):
    # same per-voxel formulas, different data staging and instruction
    # selection (fused multiply-adds may contract differently)
    inst = junction_instance(n=48, res=15.0)
    a = Fields(inst, precision, "split")
    b = Fields(inst, precision, "fused")
    a.step(137)
    b.step(137)
    scale = max(float(np.max(np.abs(a.get_array(c)))) for c in range(6))
    for c in range(6):
        assert float(np.max(np.abs(b.get_array(c) - a.get_array(c)))) <= tol * scale, c
    assert rel(b.monitors(), a.monitors()) <= tol


@pytest.mark.parametrize("ty,ring,zs", [(4, 3, 7), (16, 3, 13), (8, 4, 1000), (4, 4, 45)])
def test_tma_tilings_agree(lib, ty, ring, zs):
    # tile heights, z-segment lengths (incl. ragged ones) and ring depths
    # change only the work decomposition, never the numbers
    inst = junction_instance(n=45, res=14.0)
    a = Fields(inst, "f32", "tma")
    b = Fields(inst, "f32", "tma")
    a.set_tiling(8, 3, 64)
    b.set_tiling(ty, ring, zs)
    a.step(60)
    b.step(60)
    for c in range(6):
        np.testing.assert_array_equal(b.get_array(c), a.get_array(c))
    np.testing.assert_array_equal(b.monitors(), a.monitors())


@pytest.mark.parametrize("zs", [8, 32])
def test_fused_zsegments_agree(lib, zs):
    # the z-segment length moves tiles between the plain and the general
    # kernel; both evaluate the same formula, so the bits do not change
    inst = junction_instance(n=96, res=30.0)
    assert plain_tiles(inst, 16) > 0
    a = Fields(inst, "f32", "fused")
    b = Fields(inst, "f32", "fused")
    a.set_tiling(8, 0, 16)
    b.set_tiling(8, 0, zs)
    assert b.tiling() == (8, 0, zs)
    a.step(60)
    b.step(60)
    for c in range(6):
        np.testing.assert_array_equal(b.get_array(c), a.get_array(c))
    np.testing.assert_array_equal(b.monitors(), a.monitors())


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_two_column_tiles_equal_one_column(lib, precision):
    # nx = 96: plain, single-slab and multi-slab tiles all run two columns
    # per thread by default (CPML tiles in FP32); forcing one column per
    # thread must not change a bit
    inst = junction_instance(n=96, res=30.0, probe_components=("Ex", "Ez"))
    assert plain_tiles(inst, 16) > 0
    a = Fields(inst, precision, "fused")
    b = Fields(inst, precision, "fused")
    b.set_fused_columns(1)
    a.step(80)
    b.step(80)
    for c in range(6):
        np.testing.assert_array_equal(a.get_array(c), b.get_array(c), err_msg=f"component {c}")
    np.testing.assert_array_equal(a.monitors(), b.monitors())
    np.testing.assert_array_equal(a.dft(), b.dft())


def plain_tiles(inst, zb):
    """A lower bound on the tiles the fused schedule gives its plain kernel
    (32 x 8 x zb tiles whose footprint, one cell wider towards -x/-y/-z,
    avoids every CPML slab; slabs taken one cell wider than they are)."""
    g = inst.grid
    w = math.ceil(inst.pml.thickness / g.dx) + 1 if inst.pml.thickness > 0 else 0

    def clear(n, t):
        nt = -(-n // t)
        return sum(1 for q in range(nt) if max(q * t - 1, 0) >= w and min(q * t + t, n) - 1 < n - w)

    return clear(g.nx, 32) * clear(g.ny, 8) * clear(g.nz, zb)


@pytest.mark.parametrize("pml_um", [0.2, 0.0])
def test_fused_plain_tiles_match_oracle(lib, oracle_lib, pml_um):
    inst = junction_instance(n=80, res=25.0, pml_um=pml_um)
    assert plain_tiles(inst, 16) > 0
    f = Fields(inst, "f64", "fused")
    o = OracleFields(inst)
    f.step(250)
    o.step(250)
    compare_fields(f, o, TOL64)
    assert rel(f.monitors(), o.monitors()) <= TOL64
    assert rel(f.dft(), o.dft()) <= TOL64


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_grouped_launches_equal_single_runs(lib, precision):
    # instances with the same grid and CPML (here: three 64^3 and two 48^3
    # junctions with different pulse phases and amplitudes, interleaved
    # with a 40^3 one) share the fused schedule's tile launches, their
    # arrays packed at fixed strides; every instance must come out bit for
    # bit as it does alone (64^3: two-column plain tiles; 48^3 and 40^3:
    # one-column plain tiles and partial edge tiles)
    shapes = [(64, 20.0, 0.3, 2.0), (48, 15.0, 1.1, 0.7), (64, 20.0, 2.9, 0.2), (40, 12.5, 0.5, 1.0),
              (48, 15.0, 5.0, 3.0), (64, 20.0, 4.4, 1.3)]
    insts = [junction_instance(n=n, res=r, phase=ph, amplitude=a, probe_components=("Ex", "Ez"))
             for (n, r, ph, a) in shapes]
    f = Fields(insts, precision, "fused")
    f.autotune(2)
    singles = [Fields(i, precision, "fused") for i in insts]
    assert f.launches_per_step() < sum(s.launches_per_step() for s in singles)
    f.step(120)
    for q, s in enumerate(singles):
        s.set_tiling(*f.tiling())
        s.step(120)
        for c in range(6):
            np.testing.assert_array_equal(f.get_array(c, q), s.get_array(c), err_msg=f"instance {q} component {c}")
        np.testing.assert_array_equal(f.monitors(q), s.monitors())
        np.testing.assert_array_equal(f.dft(q), s.dft())
        s.close()


@pytest.mark.parametrize("schedule", ["fused", "tma"])
def test_autotune_leaves_state_untouched(lib, schedule):
    inst = junction_instance(n=40, res=12.5)
    a = Fields(inst, "f32", schedule)
    b = Fields(inst, "f32", schedule)
    a.step(50)
    b.step(50)
    ty, ring, zs, ms = b.autotune(steps=2)
    if schedule == "fused":
        assert (ty, ring) == (8, 0) and zs in (8, 16, 32) and ms > 0
    else:
        assert ty in (4, 8, 16) and ring in (3, 4) and zs >= 1 and ms > 0
    assert b.steps_done == 50
    a.step(50)
    b.step(50)
    for c in range(6):
        np.testing.assert_array_equal(b.get_array(c), a.get_array(c))
    np.testing.assert_array_equal(b.monitors(), a.monitors())


def test_write_read_roundtrip_and_queries(lib):
    inst = junction_instance(n=32, res=10.0)
    f = Fields(inst, "f64")
    x = np.random.default_rng(3).standard_normal((32, 32, 32))
    f.set_array(_abi.HY, x)
    np.testing.assert_array_equal(f.get_array(_abi.HY), x)
    assert f.dt() == pytest.approx(inst.grid.dt)
    f.step(7)
    assert f.time() == pytest.approx(7 * inst.grid.dt)
    assert f.n_samples() == 1
    assert f.last_source_time() == pytest.approx(20.0)
    assert f.max_abs_e() >= 0


def test_invalid_descriptors_are_rejected(lib):
    inst = junction_instance(n=32, res=10.0)
    inst.sources[0].component = 9
    with pytest.raises(_abi.SJError) as e:
        Fields(inst, "f64")
    assert e.value.code == _abi.SJ_E_INVALID


def test_sweep_instances_build(lib):
    insts = sweep_instances(per_size=1)
    f = Fields(insts, "f32")
    f.step(5)
    assert f.voxels() == 96 ** 3 + 128 ** 3 + 192 ** 3


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_snapshots_equal_field_reads(lib, precision):
    # dump_raw streamed: every snapshot is the field as sj_read_field returns
    # it before the step it was taken at (save points n % every == 0)
    inst = junction_instance(n=40, res=12.5)
    a = Fields(inst, precision)
    b = Fields(inst, precision)
    a.set_snapshots(_abi.EX, every=7, depth=3)
    got = []
    for chunk in (10, 5, 11):
        a.step(chunk)
        while (s := a.take_snapshot()) is not None:
            got.append(s)
    a.step_graph(10, chunk=4)  # graph replays step one launch at a time meanwhile
    while (s := a.take_snapshot()) is not None:
        got.append(s)
    assert [g[0] for g in got] == [0, 7, 14, 21, 28, 35]
    for step, arr in got:
        b.step(step - b.steps_done)
        np.testing.assert_array_equal(arr, b.get_array(_abi.EX))
    b.step(a.steps_done - b.steps_done)
    for c in range(6):
        np.testing.assert_array_equal(a.get_array(c), b.get_array(c))


def test_snapshot_ring_full_stops_stepping(lib):
    inst = junction_instance(n=32, res=10.0)
    f = Fields(inst, "f32")
    f.set_snapshots(_abi.EZ, every=1, depth=3)
    with pytest.raises(_abi.SJError) as e:
        f.step(5)
    assert e.value.code == _abi.SJ_E_RANGE
    assert f.steps_done == 3 and f.snapshots_pending() == 3
    assert [f.take_snapshot()[0] for _ in range(3)] == [0, 1, 2]
    assert f.take_snapshot() is None
    f.step(2)
    assert f.steps_done == 5 and f.snapshots_pending() == 2
    f.set_snapshots(_abi.EZ, every=0)
    f.step(3)
    assert f.snapshots_pending() == 0 and f.steps_done == 8


def test_queued_launch_equals_grouped_launches(lib):
    # FP32 instances with whole 32-column rows (three 64^3 and two 96^3
    # junctions): one queued launch of resident blocks claiming every
    # group's tiles gives the same bits as the grouped launches, stepped
    # directly and through graph replays
    shapes = [(64, 20.0, 0.3, 2.0), (96, 30.0, 1.1, 0.7), (64, 20.0, 2.9, 0.2), (96, 30.0, 5.0, 3.0),
              (64, 20.0, 4.4, 1.3)]
    insts = [junction_instance(n=n, res=r, phase=ph, amplitude=a, probe_components=("Ex", "Ez"))
             for (n, r, ph, a) in shapes]
    a = Fields(insts, "f32", "fused")
    b = Fields(insts, "f32", "fused")
    b.set_fused_launch("queue")
    assert b.fused_launch() == "queue" and a.fused_launch() == "grouped"
    assert b.launches_per_step() < a.launches_per_step()
    a.step(70)
    b.step(20)
    b.step_graph(50, 5)
    for q in range(len(insts)):
        for c in range(6):
            np.testing.assert_array_equal(b.get_array(c, q), a.get_array(c, q), err_msg=f"instance {q} component {c}")
        np.testing.assert_array_equal(b.monitors(q), a.monitors(q))
    g = Fields(junction_instance(n=48, res=15.0), "f32", "fused")
    with pytest.raises(_abi.SJError):          # nx = 48: no whole 32-column rows
        g.set_fused_launch("queue")
