"""Batched adjoint inverse design (16 designs at 192^3); prints one JSON line.

    python -m sim_juncs_gb300.inverse_design [--designs 16] [--n 192]
        [--steps 5000] [--iters 50] [--checkpoint 200] [--lr 0.05]

Every design (configs.inverse_design_case, seed = design index) is one
instance of a single batched simulation.  Each iteration runs forward and
adjoint for all designs at once (sj_adjoint_gradient, FP32 fields with FP64
DFT sums) and takes a normalised gradient-ascent step on eps, clipped to
[1, 4].  At the first and last iteration the FP32 objective and gradient of
design 0 are compared with an FP64 run of the same eps.
"""
import argparse
import json
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
    a = p.parse_args()
    res = 30.0 * a.n / 192
    cases = [configs.inverse_design_case(d, n=a.n, res=res) for d in range(a.designs)]
    insts = [c[0] for c in cases]
    eps = [c[1].eps.copy() for c in cases]
    lo = cases[0][1].lo
    objs = [c[2] for c in cases]
    f = Fields(insts, "f32")
    hist, secs, checks = [], [], {}
    for it in range(a.iters):
        for q in range(a.designs):
            f.set_design(Design(lo, eps[q]), q)
        f.synchronize()
        t0 = time.perf_counter()
        F, grads = f.adjoint_gradient(objs, a.steps, a.checkpoint)
        f.synchronize()
        secs.append(time.perf_counter() - t0)
        hist.append([float(x) for x in F])
        if it == 0 or it == a.iters - 1:
            checks[str(it)] = fp64_check(insts[0], Design(lo, eps[0]), objs[0], a.steps, a.checkpoint, F[0], grads[0])
        for q in range(a.designs):
            g = grads[q]
            eps[q] = np.clip(eps[q] + a.lr * g / max(np.max(np.abs(g)), 1e-300), 1.0, 4.0)
    voxels = a.designs * a.n ** 3
    out = {"config": {"designs": a.designs, "grid": f"{a.n}^3", "px_per_um": res,
                      "design_voxels": int(eps[0].size), "steps": a.steps, "iterations": a.iters,
                      "checkpoint_every": a.checkpoint},
           "objective_mean": [float(np.mean(h)) for h in hist],
           "objective_first_last": [hist[0], hist[-1]],
           "seconds_per_iteration": secs,
           "forward_voxel_steps_per_s": voxels * a.steps / float(np.median(secs)),
           "fp32_vs_fp64": checks}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
