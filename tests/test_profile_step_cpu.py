"""The profiler driver's workload names (no GPU: only the instance specs)."""
import pytest

from sim_juncs_gb300 import profile_step


def test_inverse_workloads_carry_their_designs_and_objectives():
    insts = profile_step.instances("inverse2")
    des = profile_step.designs("inverse2")
    objs = profile_step.objectives("inverse2")
    assert len(insts) == len(des) == len(objs) == 2
    assert [q for q, _ in des] == [0, 1]
    for inst in insts:
        assert (inst.grid.nx, inst.grid.ny, inst.grid.nz) == (192, 192, 192)
    # the design regions differ by seed, the objective patch does not
    assert (des[0][1].eps != des[1][1].eps).any()
    assert (objs[0].cells == objs[1].cells).all()


@pytest.mark.parametrize("name", ["inverse", "inverse0", "inverse17", "inversex"])
def test_bad_inverse_names_are_refused(name):
    with pytest.raises(SystemExit):
        profile_step.instances(name)


def test_plain_workloads_have_no_designs():
    assert profile_step.designs("junction64") == []
    with pytest.raises(SystemExit):
        profile_step.objectives("sweep")
