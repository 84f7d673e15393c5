"""Check the adjoint gradient of a design problem against central finite
differences and against the FP64 adjoint; print one JSON line.

    python -m sim_juncs_gb300.adjoint_check [--n 160] [--steps 4000]
        [--checkpoint 200] [--voxels 16] [--h 1e-3]

Defaults are the adjoint case (configs.adjoint_case): 160^3 at
30 px/um, Au box pair, an 18 x 18 x 3 design region in the gap with
eps ~ U[1, 4] (seed 1), |E(fcen)|^2 over a 5 x 5 gap patch, 4000 steps,
checkpoints every 200 steps.  The finite differences use the FP64 forward
path (sj_objective) on `voxels` design voxels drawn from seed 2.
"""
import argparse
import json
import time

import numpy as np

from . import configs
from .fields import Fields
from .spec import Design


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--n", type=int, default=160)
    p.add_argument("--steps", type=int, default=4000)
    p.add_argument("--checkpoint", type=int, default=200)
    p.add_argument("--voxels", type=int, default=16)
    p.add_argument("--h", type=float, default=1e-3)
    a = p.parse_args()
    res = 30.0 * a.n / 160
    inst, des, obj = configs.adjoint_case(n=a.n, res=res)
    out = {"config": {"grid": f"{a.n}^3", "px_per_um": res, "design_voxels": int(des.eps.size),
                      "patch_cells": int(len(obj.cells)), "steps": a.steps, "checkpoint_every": a.checkpoint}}
    grads = {}
    for prec in ("f32", "f64"):
        f = Fields(inst, prec)
        f.set_design(des)
        f.synchronize()
        t0 = time.perf_counter()
        F, g = f.adjoint_gradient(obj, a.steps, a.checkpoint)
        f.synchronize()
        t1 = time.perf_counter()
        Ff = f.objective(obj, a.steps)
        f.synchronize()
        t2 = time.perf_counter()
        grads[prec] = g[0]
        out[prec] = {"F": float(F[0]), "adjoint_s": t1 - t0, "forward_s": t2 - t1,
                     "adjoint_over_forward": (t1 - t0) / (t2 - t1)}
        f.close()
    ref = grads["f64"]
    out["f32_vs_f64_grad_rel_err"] = float(np.max(np.abs(grads["f32"] - ref)) / np.max(np.abs(ref)))
    # central differences with the FP64 forward path
    rng = np.random.default_rng(2)
    flat = rng.choice(des.eps.size, size=min(a.voxels, des.eps.size), replace=False)
    f = Fields(inst, "f64")
    fd = []
    for q in flat:
        idx = np.unravel_index(q, des.eps.shape)
        vals = []
        for sgn in (1, -1):
            e2 = des.eps.copy()
            e2[idx] += sgn * a.h
            f.set_design(Design(des.lo, e2))
            vals.append(float(f.objective(obj, a.steps)[0]))
        fd.append((vals[0] - vals[1]) / (2 * a.h))
    fd = np.array(fd)
    scale = float(np.max(np.abs(fd)))
    for prec in ("f32", "f64"):
        g = grads[prec].reshape(-1)[flat]
        out[prec]["fd_max_abs_err_over_max_fd"] = float(np.max(np.abs(g - fd)) / scale)
        big = np.abs(fd) > 1e-2 * scale
        out[prec]["fd_max_rel_err_where_fd_gt_1pct"] = float(np.max(np.abs(g - fd)[big] / np.abs(fd[big])))
    out["fd"] = {"voxels": int(len(flat)), "h": a.h, "max_abs_fd": scale}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
