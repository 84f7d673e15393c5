"""Benchmark of the GB300 FDTD stepper (one JSON line on rank 0).

Workload (default "sweep"): the batched CEP/amplitude sweep — 96 junction
instances on uneven grids (32 x 96^3, 32 x 128^3, 32 x 192^3), FP32 fields,
the instances of one grid size sharing every tile launch (12 launches per
step, replayed from CUDA graphs).  A bench step is one FDTD time
step of the whole batch.  The metric is voxel-steps/s = sum of instance
voxels x steps / device time.  Also reported: the plain FP64 path on a grid
whose state is well above L2 (512 x 512 x 384), its roofline fraction, and
the FP32/FP64 gap-field error.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload sweep|bowtie|junction] [--schedule auto|fused|tma|split]

--schedule auto (default) autotunes both single-pass schedules (fused
column-march kernels; TMA shared-memory tiles) on the workload and times
the faster.

Under torchrun each rank runs its own full batch (weak scaling, no
collective on the data path); value = all ranks' voxel-steps / max time.
`--impl reference` times the CPU restatement (the reference's stepper,
meep, cannot run here) on the host cores with a bounded sample per step.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "voxel-steps/s & %HBM peak: FP32 batched vs FP64 plain at <=1e-4 rel gap-field err"
UNIT = "voxel-steps/s"


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="sweep", choices=["sweep", "bowtie", "junction"])
    p.add_argument("--schedule", default="auto", choices=["auto", "fused", "tma", "split"])
    p.add_argument("--e2e-steps", type=int, default=None,
                   help="steps of the end-to-end job (default: the workload's steps per run)")
    p.add_argument("--no-extras", action="store_true", help="skip the FP64 and error legs")
    return p.parse_args(argv)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(secs, torch):
    """The slowest rank's time (every rank gets it); identity on one rank.
    The tensor lives where the process group's backend wants it (NCCL: the
    GPU, gloo: the host)."""
    dist = torch.distributed
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(secs)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(secs)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(voxels_per_rank, steps, ws, secs):
    """Whole-job voxel-steps/s: every rank steps its own batch (weak
    scaling, replicas), timed by the slowest rank."""
    return voxels_per_rank * steps * ws / secs


def workload_instances(name, rank=0):
    from sim_juncs_gb300 import configs
    if name == "sweep":
        return configs.sweep_instances(seed=rank), {
            "workload": "cep_amplitude_sweep", "instances": 96,
            "grids": "32x96^3 + 32x128^3 + 32x192^3", "px_per_um": [30, 40, 60],
            "cell_um": 3.2, "pml_um": 0.5, "steps_per_run": 4000, "seed": rank}
    if name == "bowtie":
        return [configs.bowtie_instance()], {"workload": "bowtie", "grid": "512x512x384",
                                             "px_per_um": 40, "pml_um": 1.0, "steps_per_run": 20000}
    return [configs.junction_instance()], {"workload": "junction", "grid": "64^3", "px_per_um": 20,
                                           "pml_um": 0.5, "steps_per_run": 2000}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        # the raw samples: SJ_CLOCKS_DIR when set (to keep them), else the temp directory
        base = os.environ.get("SJ_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(base, f"clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        self.proc.wait()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def time_steps(f, torch, steps, warmup, graph_chunk=0):
    """Device time of `steps` steps on f's stream (CUDA events), after warmup;
    graph_chunk > 0: the steps replay CUDA graphs of that many steps
    (sj_step_graph; the graphs are captured during the warm-up)."""
    run = (lambda n: f.step_graph(n, graph_chunk)) if graph_chunk > 0 else f.step
    run(warmup)
    f.synchronize()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if torch.distributed.is_initialized():
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    run(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    return ms / 1000.0, steps * f.launches_per_step()


def tuned_fields(insts, schedule, torch):
    """Fields on the current torch stream with the schedule's tiling picked by
    the library's autotuner; schedule "auto" keeps the faster of the two
    single-pass schedules.  Returns (fields, schedule, tiling, ms/step)."""
    from sim_juncs_gb300.fields import Fields
    cands = ("fused", "tma") if schedule == "auto" else (schedule,)
    best = None
    for sch in cands:
        f = Fields(insts, "f32", sch, stream=torch.cuda.current_stream())
        if sch == "split":
            til, ms = None, None
        else:
            ty, ring, zs, ms = f.autotune(steps=2)
            til = (ty, ring, zs)
        if best is None or (ms is not None and ms < best[3]):
            if best is not None:
                best[0].close()
            best = (f, sch, til, ms)
        else:
            f.close()
    return best


def run_ours(args):
    import torch
    from sim_juncs_gb300 import build

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    # a real (non-legacy) stream shared by torch's events and the library
    torch.cuda.set_stream(torch.cuda.Stream())
    if ws > 1:
        torch.distributed.init_process_group("nccl")
    if rank == 0:
        build.build()
    if ws > 1:
        torch.distributed.barrier()

    insts, cfg = workload_instances(args.workload, rank)
    f, schedule, til, tune_ms = tuned_fields(insts, args.schedule, torch)
    if til is not None:
        cfg = dict(cfg, tile=f"32x{til[0]}", tma_ring=til[1], zseg=til[2], tiling="autotuned",
                   autotune_dry_ms_per_step=tune_ms)  # the tuner's launches load but do not store
        if schedule == "fused":
            cfg["launch_mode"] = f.fused_launch()  # grouped launches or one queued launch, as the tuner kept
    voxels = f.voxels()
    bytes_step = f.bytes_per_step()

    # the headline replays CUDA graphs of `chunk` steps (sj_step_graph): an odd
    # chunk alternates the two ping-pong parities, and the warm-up (>= 2
    # chunks) captures both graphs before the timed region
    chunk = max(1, (args.warmup // 2) | 1) if args.warmup >= 2 else 0
    if chunk and 2 * chunk > args.warmup:
        chunk -= 2
    clocks = ClockSampler(local)
    clocks.start()
    secs, launches = time_steps(f, torch, args.steps, args.warmup, graph_chunk=max(chunk, 0))
    clk = clocks.stop()
    secs_launch, _ = time_steps(f, torch, args.steps, args.warmup)
    secs = max_over_ranks(secs, torch)
    secs_launch = max_over_ranks(secs_launch, torch)
    value = job_value(voxels, args.steps, ws, secs)
    peak, peak_kind = measured_peak()
    achieved = bytes_step / (secs / args.steps) / 1e9
    kernel = {"fused": "fused step: plain, slab and multi tile launches per instance group and one general "
                       "launch, concurrent (one HBM pass)",
              "tma": "k_fused (TMA shared-memory tiles), one launch per step",
              "split": "k_split_h + k_split_e"}[schedule]
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(cfg, schedule=schedule, l2="state larger than L2 (no flush needed)",
                       voxels_per_step=voxels, parallelism=f"replicas{ws}",
                       timed=f"CUDA graph replays of {max(chunk, 0)} step(s) (sj_step_graph)" if chunk > 0
                       else "sj_step launches",
                       ms_per_step_plain_launches=secs_launch / args.steps * 1e3),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "frac_of_nominal_7900": achieved / 7900.0,
                     "traffic": traffic_per_step(schedule, voxels),
                     "peak_kind": peak_kind, "algorithmic_bytes_per_step": bytes_step, "kernel": kernel},
        "gpu_launches": launches,
        "clocks": clk,
    }
    f.close()
    del f

    if rank == 0 and not args.no_extras:
        out["fp64_plain"] = fp64_leg(torch, args)
        out["fp64_same_workload"] = fp64_same_workload(torch, args, insts, value / ws)
        out["fp32_vs_fp64"] = error_leg(schedule)
    if rank == 0:
        out["e2e"] = e2e_leg(args, insts, schedule, til, args.e2e_steps or cfg["steps_per_run"])
        out["cpu_baseline"] = cpu_baseline()
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def traffic_per_step(schedule, voxels):
    """DRAM bytes per step from the committed ncu summary of the schedule's
    kernels (bytes per voxel-step of the captured case x this step's voxels),
    or None when there is none."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            per = json.load(fh)[schedule]["dram_bytes_per_voxel_step"]
        return float(per) * voxels
    except Exception:
        return None


def fp64_leg(torch, args):
    """Plain FP64 path (the library's FP64 default schedule) on the
    512 x 512 x 384 bowtie grid (state >> L2)."""
    from sim_juncs_gb300 import configs
    from sim_juncs_gb300.fields import Fields
    inst = configs.bowtie_instance()
    f = Fields(inst, "f64", stream=torch.cuda.current_stream())
    steps = max(5, args.steps // 4)
    secs, launches = time_steps(f, torch, steps, 3)
    peak, kind = measured_peak()
    b = f.bytes_per_step()
    ach = b / (secs / steps) / 1e9
    res = {"workload": "bowtie 512x512x384 f64", "schedule": f.schedule_name(),
           "value": inst.grid.voxels * steps / secs, "unit": UNIT,
           "ms_per_step": secs / steps * 1e3, "steps": steps, "gpu_launches": launches,
           "roofline": {"achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                        "peak_kind": kind, "algorithmic_bytes_per_step": b}}
    f.close()
    return res


def fp64_same_workload(torch, args, insts, fp32_value):
    """FP64 (the library's default schedule) on the headline workload itself:
    plain = one instance at a time (each distinct grid timed alone, weighted
    by how many instances share it), batched = all instances in one
    simulation.  fp32_over_fp64_* = the FP32 headline value over each."""
    from sim_juncs_gb300.fields import Fields
    steps = max(3, args.steps // 8)
    shapes = {}
    for inst in insts:
        g = inst.grid
        shapes.setdefault((g.nx, g.ny, g.nz, g.dx), []).append(inst)
    total_vox, total_s = 0, 0.0
    for members in shapes.values():
        f = Fields(members[0], "f64", stream=torch.cuda.current_stream())
        secs, _ = time_steps(f, torch, steps, 2)
        total_vox += len(members) * f.voxels() * steps
        total_s += len(members) * secs
        f.close()
    plain = total_vox / total_s
    f = Fields(insts, "f64", stream=torch.cuda.current_stream())
    secs, launches = time_steps(f, torch, steps, 2)
    batched = f.voxels() * steps / secs
    res = {"schedule": f.schedule_name(), "unit": UNIT, "steps": steps,
           "plain_value": plain, "batched_value": batched, "batched_gpu_launches": launches,
           "fp32_over_fp64_plain": fp32_value / plain, "fp32_over_fp64_batched": fp32_value / batched}
    f.close()
    return res


def error_leg(schedule):
    """FP32 (timed schedule) vs FP64 (default schedule) relative gap-field
    error on the 64^3 junction, 2000 steps."""
    from sim_juncs_gb300 import configs
    from sim_juncs_gb300.fields import Fields
    inst = configs.junction_instance()
    a = Fields(inst, "f64")
    b = Fields(inst, "f32", schedule)
    a.step(2000)
    b.step(2000)
    m64, m32 = a.monitors()[:4], b.monitors()[:4]
    d64, d32 = a.dft()[:4], b.dft()[:4]
    a.close()
    b.close()
    return {"workload": "junction 64^3, 2000 steps, Ex at 4 gap points",
            "monitor_rel_err": float(np.max(np.abs(m32 - m64)) / np.max(np.abs(m64))),
            "dft_rel_err": float(np.max(np.abs(d32 - d64)) / np.max(np.abs(d64)))}


def e2e_leg(args, insts, schedule, til, steps):
    """Whole job through the public API from host descriptors: create
    (uploads the scene and the per-step source tables, rasterises on the
    device), set the tuned tiling, `steps` steps (by default the workload's
    whole run), then monitors + DFT back to host buffers.  Wall clock, host
    to host."""
    from sim_juncs_gb300.fields import Fields
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    f = Fields(insts, "f32", schedule)
    if til is not None:
        f.set_tiling(*til)
    f.step(steps)
    outs = [(f.monitors(q), f.dft(q)) for q in range(f.n_instances)]
    t1 = time.perf_counter()
    voxels = f.voxels()
    h2d, d2h = f.transfer_bytes()
    f.close()
    return {"value": voxels * steps / (t1 - t0), "unit": UNIT,
            "steps": steps, "seconds": t1 - t0,
            "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": d2h / steps,
            "includes": "create + device rasterise + steps + monitor/DFT read-back"}


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the platform)."""
    import platform
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.machine()


def cpu_sample():
    """Bounded CPU sample: one 96^3 sweep member, FP64 restatement."""
    from sim_juncs_gb300 import configs
    return configs.junction_instance(n=96, res=30.0, probe_components=("Ez",), dft=False)


def cpu_baseline(target_s=10.0):
    """The oracle on one 96^3 sweep member, as many steps as take ~target_s."""
    from oracle import oracle
    oracle.build()
    inst = cpu_sample()
    o = oracle.OracleFields(inst)
    t0 = time.perf_counter()
    o.step(10)
    probe = time.perf_counter() - t0
    steps = int(min(4000, max(10, target_s / max(probe / 10, 1e-6))))
    t0 = time.perf_counter()
    o.step(steps)
    secs = time.perf_counter() - t0
    return {"value": inst.grid.voxels * steps / secs, "unit": UNIT, "cores": oracle.threads(),
            "kind": "port", "cpu": cpu_model(), "mpi_ranks": 1,
            "sample": f"one 96^3 sweep member, {steps} FP64 steps in {secs:.1f} s "
                      "(OpenMP restatement; meep v1.24 is not available to run)"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle
    oracle.build()
    inst = cpu_sample()
    o = oracle.OracleFields(inst)
    per = 10
    for _ in range(args.warmup):
        o.step(per)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step(per)
    secs = time.perf_counter() - t0
    value = inst.grid.voxels * per * args.steps / secs
    _, cfg = workload_instances(args.workload)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference", "config": cfg,
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.threads(), "kind": "port",
                            "cpu": cpu_model(), "mpi_ranks": 1,
                            "sample": f"{per} FP64 steps of one 96^3 sweep member per bench step "
                                      "(CPU restatement; meep v1.24 is not available to run)"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
