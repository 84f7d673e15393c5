"""The CUDA adjoint (sj_adjoint_gradient) against the oracle's FP64 adjoint,
which test_adjoint_cpu.py checks against finite differences."""
import numpy as np
import pytest

from oracle.oracle import OracleFields
from sim_juncs_gb300 import _abi
from sim_juncs_gb300.fields import Fields
from sim_juncs_gb300.spec import Design

from test_adjoint_cpu import N_STEPS, setup

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def reference():
    inst, des, obj = setup()
    o = OracleFields(inst)
    o.set_design(des)
    F, g = o.adjoint(obj, N_STEPS)
    return F, g


def test_f64_adjoint_matches_oracle(lib, oracle_lib, reference):
    inst, des, obj = setup()
    f = Fields(inst, "f64")
    f.set_design(des)
    F, g = f.adjoint_gradient(obj, N_STEPS, checkpoint_every=50)
    assert F[0] == pytest.approx(reference[0], rel=1e-10)
    assert rel(g[0], reference[1]) <= 1e-8


def test_f32_adjoint_within_1e3_of_f64(lib, oracle_lib, reference):
    inst, des, obj = setup()
    f = Fields(inst, "f32")
    f.set_design(des)
    F, g = f.adjoint_gradient(obj, N_STEPS, checkpoint_every=50)
    assert F[0] == pytest.approx(reference[0], rel=1e-4)
    assert rel(g[0], reference[1]) <= 1e-3, rel(g[0], reference[1])


def test_checkpoint_interval_changes_nothing(lib):
    inst, des, obj = setup()
    out = []
    for K in (16, 37, N_STEPS):
        f = Fields(inst, "f32")
        f.set_design(des)
        out.append(f.adjoint_gradient(obj, N_STEPS, checkpoint_every=K))
        f.close()
    for F, g in out[1:]:
        assert F[0] == out[0][0][0]
        np.testing.assert_array_equal(g[0], out[0][1][0])


def test_state_after_adjoint_equals_plain_stepping(lib):
    inst, des, obj = setup()
    a = Fields(inst, "f64")
    a.set_design(des)
    a.adjoint_gradient(obj, N_STEPS, checkpoint_every=40)
    b = Fields(inst, "f64")
    b.set_design(des)
    b.step(N_STEPS)
    assert a.steps_done == b.steps_done == N_STEPS
    for c in range(6):
        np.testing.assert_array_equal(a.get_array(c), b.get_array(c))
    np.testing.assert_array_equal(a.monitors(), b.monitors())


def test_objective_is_the_forward_half(lib):
    inst, des, obj = setup()
    f = Fields(inst, "f64")
    f.set_design(des)
    F, _ = f.adjoint_gradient(obj, N_STEPS, checkpoint_every=80)
    f.synchronize()  # host and device step counters agree
    F2 = f.objective(obj, N_STEPS)
    f.synchronize()
    assert f.steps_done == N_STEPS
    assert F2[0] == F[0]


def test_batched_designs_equal_separate_runs(lib):
    inst, des, obj = setup()
    des2 = Design(des.lo, des.eps[::-1, ::-1, :].copy() * 0.8)
    both = Fields([inst, inst], "f32")
    both.set_design(des, 0)
    both.set_design(des2, 1)
    Fb, gb = both.adjoint_gradient([obj, obj], N_STEPS, checkpoint_every=60)
    for q, d in enumerate((des, des2)):
        one = Fields(inst, "f32")
        one.set_design(d)
        F1, g1 = one.adjoint_gradient(obj, N_STEPS, checkpoint_every=60)
        assert Fb[q] == F1[0]
        np.testing.assert_array_equal(gb[q], g1[0])


def test_design_region_steps_with_fused_or_split(lib):
    # the fused schedule (default) applies the design eps in its general
    # tiles, the split one in its E pass; the TMA schedule has no design path
    inst, des, obj = setup()
    f = Fields(inst, "f32")
    f.set_design(des)
    assert f.schedule_name() == "fused"
    f.set_schedule("split")
    f.set_schedule("fused")
    with pytest.raises(_abi.SJError):
        f.set_schedule("tma")
    f.set_design(None)
    f.set_schedule("tma")
    f.set_design(des)                      # a TMA simulation moves to fused
    assert f.schedule_name() == "fused"


@pytest.mark.parametrize("precision,tol", [("f64", 1e-10), ("f32", 1e-4)])
def test_fused_and_split_adjoints_agree(lib, precision, tol):
    # the same discrete adjoint whichever schedule runs the forward passes:
    # the two differ only in rounding (fused: explicit FMAs, bracket recorded
    # in pieces across the tile and correction kernels)
    inst, des, obj = setup()
    out = []
    for sched in ("fused", "split"):
        f = Fields(inst, precision, sched)
        f.set_design(des)
        f.set_schedule(sched)
        out.append(f.adjoint_gradient(obj, N_STEPS, checkpoint_every=50))
        f.close()
    (Fa, ga), (Fb, gb) = out
    assert Fa[0] == pytest.approx(Fb[0], rel=tol)
    assert rel(ga[0], gb[0]) <= tol


def test_torch_autograd_binding(lib):
    torch = pytest.importorskip("torch")
    from sim_juncs_gb300.autograd import GapFieldObjective
    inst, des, obj = setup()
    f = Fields(inst, "f32")
    eps = torch.tensor(des.eps, dtype=torch.float64, requires_grad=True)
    F = GapFieldObjective.apply(eps, f, des.lo, obj, N_STEPS, 60)
    F.backward()
    g = Fields(inst, "f32")
    g.set_design(des)
    F2, g2 = g.adjoint_gradient(obj, N_STEPS, checkpoint_every=60)
    assert float(F.detach()) == F2[0]
    np.testing.assert_allclose(eps.grad.numpy(), g2[0], rtol=1e-6, atol=0)


def test_design_on_one_member_splits_its_launch_group(lib):
    # three 64^3 junctions share launches; a design region on the middle one
    # moves its design tiles to the general class, so the group splits into
    # runs with equal tile lists; every instance still steps bit for bit as
    # it does alone
    from sim_juncs_gb300.configs import junction_instance
    insts = [junction_instance(n=64, res=20.0, phase=ph, amplitude=a) for ph, a in ((0.2, 1.0), (1.3, 0.5), (2.9, 2.0))]
    lo = (28, 28, 31)
    eps = np.random.default_rng(3).uniform(1.0, 4.0, size=(2, 6, 8))
    des = Design(lo, eps)
    f = Fields(insts, "f32")
    grouped = f.launches_per_step()
    f.set_design(des, 1)
    assert f.launches_per_step() > grouped
    f.step(90)
    for q, inst in enumerate(insts):
        s = Fields(inst, "f32")
        if q == 1:
            s.set_design(des)
        s.step(90)
        for c in range(6):
            np.testing.assert_array_equal(f.get_array(c, q), s.get_array(c), err_msg=f"instance {q} component {c}")
        s.close()


def fd_case():
    """48^3 junction at 15 px/um (the 3.2 um cell), pulse peaking at t = 2.5 so
    that it has passed the gap within the run; a 6 x 6 x 2 design region in
    the gap with eps ~ U[1, 4]; |E(fcen)|^2 of Ex and Ez over a 3 x 3 patch."""
    from sim_juncs_gb300.configs import junction_instance
    from sim_juncs_gb300.spec import Objective
    inst = junction_instance(n=48, res=15.0, probe_components=("Ex",), dft=False)
    for s in inst.sources:
        shift = 0.5 * (s.start_time + s.end_time) - 2.5
        s.start_time -= shift
        s.end_time -= shift
    c = 24
    eps = np.random.default_rng(5).uniform(1.0, 4.0, size=(2, 6, 6))
    des = Design((c - 3, c - 3, c - 1), eps)
    cells = np.array([[c - 1 + a, c - 1 + b, c] for b in range(3) for a in range(3)])
    return inst, des, Objective(cells, frequency=1 / 0.7, comps=(0, 2))


FD_STEPS = 300


@pytest.fixture(scope="module")
def central_differences():
    """(voxels, dF/deps by central differences, h = 1e-3) of the GPU FP64
    forward path (sj_objective) at the two voxels of largest FP64 adjoint
    gradient and two drawn from seed 7."""
    inst, des, obj = fd_case()
    f = Fields(inst, "f64")
    f.set_design(des)
    _, g = f.adjoint_gradient(obj, FD_STEPS, checkpoint_every=50)
    order = np.argsort(-np.abs(g[0]).reshape(-1))
    rnd = np.random.default_rng(7).choice(des.eps.size, size=2, replace=False)
    flat = list(dict.fromkeys(list(order[:2]) + list(rnd)))
    h = 1e-3
    fd = []
    for q in flat:
        idx = np.unravel_index(q, des.eps.shape)
        vals = []
        for sgn in (1, -1):
            e2 = des.eps.copy()
            e2[idx] += sgn * h
            f.set_design(Design(des.lo, e2))
            vals.append(float(f.objective(obj, FD_STEPS)[0]))
        fd.append((vals[0] - vals[1]) / (2 * h))
    return flat, np.array(fd)


@pytest.mark.parametrize("precision,schedule,tol", [("f64", "fused", 1e-5), ("f32", "fused", 1e-3),
                                                     ("f32", "split", 1e-3)])
def test_gpu_gradient_matches_central_differences(lib, central_differences, precision, schedule, tol):
    flat, fd = central_differences
    inst, des, obj = fd_case()
    f = Fields(inst, precision, schedule)
    f.set_design(des)
    f.set_schedule(schedule)
    _, g = f.adjoint_gradient(obj, FD_STEPS, checkpoint_every=50)
    got = g[0].reshape(-1)[flat]
    scale = float(np.max(np.abs(fd)))
    assert scale > 0
    err = float(np.max(np.abs(got - fd))) / scale
    assert err <= tol, (precision, schedule, err)


def test_three_pole_adjoint_matches_oracle(lib, oracle_lib):
    # every gold E point with three polarisation adjoints: past the two per
    # point the E transpose loads up front
    from test_gpu_configs import three_pole_gold
    inst, des, obj = setup()
    inst = three_pole_gold(inst)
    o = OracleFields(inst)
    o.set_design(des)
    Fo, go = o.adjoint(obj, N_STEPS)
    f = Fields(inst, "f64")
    f.set_design(des)
    F, g = f.adjoint_gradient(obj, N_STEPS, checkpoint_every=50)
    assert F[0] == pytest.approx(Fo, rel=1e-10)
    assert rel(g[0], go) <= 1e-8
