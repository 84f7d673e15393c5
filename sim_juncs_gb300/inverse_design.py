"""Batched adjoint inverse design (16 designs at 192^3); prints one JSON line.

    python -m sim_juncs_gb300.inverse_design [--designs 16] [--n 192]
        [--steps 5000] [--iters 50] [--checkpoint 200] [--lr 0.05]

Every design (configs.inverse_design_case, seed = design index) is one
instance of a single batched simulation.  Each iteration runs forward and
adjoint for all designs at once (sj_adjoint_gradient, FP32 fields with FP64
DFT sums) and takes a normalised gradient-ascent step on eps, clipped to
[1, 4].  At the iterations in --check (default 0, 25 and --iters, the last
being one more evaluation after the final step) the FP32 objective and
gradient of design 0 are compared with an FP64 run of the same eps.

--state FILE.npz saves the designs, history and iteration reached after
every iteration and resumes from them when the file exists, so that a long
loop can run as several shorter processes; --stop-after N ends a process
after N iterations of this run.
"""
import argparse
import json
import os
import time

import numpy as np

from . import configs
from .fields import Fields
from .spec import Design


def fp64_check(inst, design, objective, steps, checkpoint, F32, g32):
    f = Fields(inst, "f64")
    f.set_design(design)
    F, g = f.adjoint_gradient(objective, steps, checkpoint)
    f.close()
    return {"objective_rel_err": float(abs(F32 - F[0]) / abs(F[0])),
            "gradient_rel_err": float(np.max(np.abs(g32 - g[0])) / np.max(np.abs(g[0])))}


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--designs", type=int, default=16)
    p.add_argument("--n", type=int, default=192)
    p.add_argument("--steps", type=int, default=5000)
    p.add_argument("--iters", type=int, default=50)
    p.add_argument("--checkpoint", type=int, default=200)
    p.add_argument("--lr", type=float, default=0.05)
    p.add_argument("--check", default=None, help="comma-separated iterations checked against FP64")
    p.add_argument("--state", default=None)
    p.add_argument("--stop-after", type=int, default=None)
    a = p.parse_args()
    check_at = ({0, 25, a.iters} if a.check is None else {int(x) for x in a.check.split(",") if x})
    res = 30.0 * a.n / 192
    cases = [configs.inverse_design_case(d, n=a.n, res=res) for d in range(a.designs)]
    insts = [c[0] for c in cases]
    eps = [c[1].eps.copy() for c in cases]
    lo = cases[0][1].lo
    objs = [c[2] for c in cases]
    f = Fields(insts, "f32")
    hist, secs, checks, start = [], [], {}, 0
    if a.state and os.path.exists(a.state):
        with np.load(a.state, allow_pickle=False) as z:
            eps = [z[f"eps{q}"] for q in range(a.designs)]
            hist = z["hist"].tolist()
            secs = z["secs"].tolist()
            start = int(z["next_iter"])
            checks = json.loads(str(z["checks"]))
    done_here = 0
    # iterations 0 .. iters-1 step the designs; iteration `iters` only evaluates
    for it in range(start, a.iters + 1):
        if a.stop_after is not None and done_here >= a.stop_after:
            break
        if it == a.iters and it not in check_at:
            break
        for q in range(a.designs):
            f.set_design(Design(lo, eps[q]), q)
        f.synchronize()
        t0 = time.perf_counter()
        F, grads = f.adjoint_gradient(objs, a.steps, a.checkpoint)
        f.synchronize()
        secs.append(time.perf_counter() - t0)
        hist.append([float(x) for x in F])
        if it in check_at:
            checks[str(it)] = fp64_check(insts[0], Design(lo, eps[0]), objs[0], a.steps, a.checkpoint, F[0], grads[0])
        if it < a.iters:
            for q in range(a.designs):
                g = grads[q]
                eps[q] = np.clip(eps[q] + a.lr * g / max(np.max(np.abs(g)), 1e-300), 1.0, 4.0)
        done_here += 1
        if a.state:
            np.savez(a.state, **{f"eps{q}": eps[q] for q in range(a.designs)}, hist=np.asarray(hist),
                     secs=np.asarray(secs), next_iter=it + 1, checks=json.dumps(checks))
    voxels = a.designs * a.n ** 3
    out = {"config": {"designs": a.designs, "grid": f"{a.n}^3", "px_per_um": res,
                      "design_voxels": int(eps[0].size), "steps": a.steps, "iterations": a.iters,
                      "checkpoint_every": a.checkpoint, "evaluations_so_far": len(hist)},
           "objective_mean": [float(np.mean(h)) for h in hist],
           "objective_first_last": [hist[0], hist[-1]],
           "seconds_per_iteration": secs,
           "design_voxel_steps_per_s": voxels * a.steps / float(np.median(secs)),  # forward, re-runs and adjoint
           "fp32_vs_fp64": checks}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
