"""Run a few steps of a named workload, for profilers (ncu) to capture.

    python -m sim_juncs_gb300.profile_step WORKLOAD [--precision f32|f64]
        [--schedule fused|tma|split] [--zseg Z] [--steps N]

Workloads: sweep (32 x 96^3 + 32 x 128^3 + 32 x 192^3 junctions),
junction192 (one 192^3 sweep member), junction192x4 (four 192^3 sweep
members: one launch group, ~3.4 GB on the device), bowtie (512 x 512 x
384), junction64 (64^3), inverseN (the first N of the 16 inverse-design
instances at 192^3: Au on a quartz substrate, each with its design region;
~1.1 GB each).  Prints the launches per step so that a capture
can skip set-up launches and warm-up steps by count.

--adjoint: instead of plain steps, one sj_adjoint_gradient over N steps
(inverseN: every instance's own objective; one checkpoint segment), so the
forward, re-run and adjoint kernels are captured;
--diag energy: after the steps, three sj_energy calls (k_energy + k_sum);
--diag phases: then the phases of 384 monitor series (the sweep's 96 x 4
gap points, here 48 copies of the 64^3 junction's 8) in one sj_extract_phases
call (k_phases).
"""
import argparse

from . import configs
from .fields import Fields


def instances(name):
    if name == "sweep":
        return configs.sweep_instances()
    if name == "junction192":
        return [configs.junction_instance(n=192, res=60.0, probe_components=("Ez",), dft=False)]
    if name == "junction192x4":
        return [m for m in configs.sweep_instances() if m.grid.nx == 192][:4]
    if name == "bowtie":
        return [configs.bowtie_instance()]
    if name == "junction64":
        return [configs.junction_instance()]
    if _inverse_count(name):
        return [configs.inverse_design_case(d)[0] for d in range(_inverse_count(name))]
    raise SystemExit(f"unknown workload {name!r}")


def _inverse_count(name):
    """N of an inverseN workload name (1..16), else 0."""
    if name.startswith("inverse") and name[7:].isdigit() and 1 <= int(name[7:]) <= 16:
        return int(name[7:])
    return 0


def objectives(name):
    """The objectives of a workload's instances (inverseN only)."""
    if _inverse_count(name):
        return [configs.inverse_design_case(d)[2] for d in range(_inverse_count(name))]
    raise SystemExit(f"{name!r} has no objectives")


def designs(name):
    """The design regions a workload's instances carry (instance, Design)."""
    if _inverse_count(name):
        return [(d, configs.inverse_design_case(d)[1]) for d in range(_inverse_count(name))]
    return []


def main():
    p = argparse.ArgumentParser()
    p.add_argument("workload")
    p.add_argument("--precision", default="f32")
    p.add_argument("--schedule", default=None)
    p.add_argument("--zseg", type=int, default=8)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--diag", default=None, choices=["energy", "phases"])
    p.add_argument("--adjoint", action="store_true")
    a = p.parse_args()
    f = Fields(instances(a.workload), a.precision, a.schedule)
    for q, des in designs(a.workload):
        f.set_design(des, q)
    if f.schedule_name() == "fused":
        f.set_tiling(8, 0, a.zseg)
    if a.adjoint:
        f.adjoint_gradient(objectives(a.workload), a.steps, a.steps)
    else:
        f.step(a.steps)
    f.synchronize()
    print(f"{a.workload} {a.precision} {f.schedule_name()} steps={f.steps_done} voxels={f.voxels()} "
          f"launches_per_step={f.launches_per_step()}", flush=True)
    if a.diag == "energy":
        for _ in range(3):
            print("energy", f.energy(0), flush=True)
    elif a.diag == "phases":
        import numpy as np
        from .phases import extract_phases
        mon = f.monitors(0)
        t = np.arange(mon.shape[1]) * (f.instances[0].grid.dt * f.instances[0].save_span)
        res = extract_phases(t, np.tile(mon, (48, 1)), 2.0)
        print("phases", len(res), sum(r["status"] == 0 for r in res), flush=True)
    f.close()


if __name__ == "__main__":
    main()
