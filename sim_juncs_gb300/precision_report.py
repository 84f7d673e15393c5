"""FP32 against FP64 on the full-length workloads; prints one JSON line.

    python -m sim_juncs_gb300.precision_report [--parts sweep,bowtie,energy]
        [--sweep-steps 4000] [--bowtie-steps 20000]

  sweep   the first 192^3 member of the CEP/amplitude sweep (60 px/um, its
          seed-0 CEP and amplitude), 4000 steps: Ez at the 4 gap points and
          their spectra;
  bowtie  the 512 x 512 x 384 bowtie, 20000 steps: the 32 x 32 Ez monitor
          plane, the 50-frequency DFTs of Ex, Ey, Hx, Hy on it and the flux
          spectrum through it;
  energy  a closed 512 x 512 x 384 cavity with the bowtie's SiO2 slab (eps
          2.13, no PML, no source, random initial E), 20000 steps: the drift
          of the discrete energy, which the leapfrog conserves exactly, in
          each precision.

Each error is max |FP32 - FP64| / max |FP64| over the output.
"""
import argparse
import json
import time

import numpy as np

from . import configs
from .fields import Fields
from .spec import PML, ClassMaterial, Grid, Instance


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def run(inst, prec, steps):
    f = Fields(inst, prec)
    f.synchronize()
    t0 = time.perf_counter()
    f.step(steps)
    f.synchronize()
    return f, time.perf_counter() - t0


def sweep_part(steps):
    inst = configs.sweep_instances()[64]
    out = {"workload": "sweep member 192^3 at 60 px/um", "steps": steps}
    res = {}
    for prec in ("f64", "f32"):
        f, sec = run(inst, prec, steps)
        res[prec] = (f.monitors(), f.monitor_spectrum())
        out[f"{prec}_s"] = sec
        f.close()
    out["gap_ez_rel_err"] = rel(res["f32"][0], res["f64"][0])
    out["spectrum_rel_err"] = rel(res["f32"][1], res["f64"][1])
    return out


def bowtie_part(steps):
    inst = configs.bowtie_instance()
    rows = configs.bowtie_flux_rows()
    dA = inst.grid.dx ** 2
    out = {"workload": "bowtie 512x512x384", "steps": steps}
    res = {}
    for prec in ("f64", "f32"):
        f, sec = run(inst, prec, steps)
        res[prec] = (f.monitors(), f.dft(), f.flux(rows, dA))
        out[f"{prec}_s"] = sec
        f.close()
    out["ez_plane_rel_err"] = rel(res["f32"][0], res["f64"][0])
    out["dft_rel_err"] = rel(res["f32"][1], res["f64"][1])
    out["flux_rel_err"] = rel(res["f32"][2], res["f64"][2])
    return out


def energy_part(steps, nx=512, ny=512, nz=384, res=40.0):
    dx = 1.0 / res
    cm = np.zeros((3, nz, ny, nx), dtype=np.uint8)
    cz = nz // 2
    cm[:, cz - 41:cz - 1, :, :] = 1       # the bowtie's 1 um SiO2 slab below the prisms
    inst = Instance(Grid(nx, ny, nz, dx, configs.stable_courant(res) * dx), ClassMaterial(cm, [1.0, 2.13]),
                    PML(0.0), save_span=20)
    rng = np.random.default_rng(4)
    init = [rng.standard_normal((nz, ny, nx)) for _ in range(3)]
    out = {"workload": "closed 512x512x384 cavity with the SiO2 slab, random E", "steps": steps}
    for prec in ("f64", "f32"):
        f = Fields(inst, prec)
        for c in range(3):
            f.set_array(c, init[c])
        f.step(1)
        w0 = f.energy()
        f.synchronize()
        t0 = time.perf_counter()
        f.step(steps)
        f.synchronize()
        out[f"{prec}_s"] = time.perf_counter() - t0
        w1 = f.energy()
        out[f"{prec}_energy_drift"] = abs(w1 - w0) / w0
        f.close()
    return out


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--parts", default="sweep,bowtie,energy")
    p.add_argument("--sweep-steps", type=int, default=4000)
    p.add_argument("--bowtie-steps", type=int, default=20000)
    p.add_argument("--energy-steps", type=int, default=20000)
    a = p.parse_args()
    out = {}
    parts = a.parts.split(",")
    if "sweep" in parts:
        out["sweep"] = sweep_part(a.sweep_steps)
    if "bowtie" in parts:
        out["bowtie"] = bowtie_part(a.bowtie_steps)
    if "energy" in parts:
        out["energy"] = energy_part(a.energy_steps)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
