"""Build the CUDA library libsj_gb300.so in-tree with nvcc for sm_103a.

Each translation unit compiles in its own nvcc process (in parallel), then
one link step produces the shared library next to this file.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libsj_gb300.so")
OBJ = os.path.join(HERE, "_build")
SOURCES = ["sj_host.cu", "sj_step.cu", "sj_lean.cu", "sj_fused.cu", "sj_raster.cu", "sj_adjoint.cu", "sj_spectrum.cu",
           "sj_diag.cu", "sj_phases.cu"]
HEADERS = ["sj_internal.h", "sj_physics.cuh", os.path.join("..", "..", "include", "sj.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# the fused stepper writes every fused multiply-add explicitly (results must
# not depend on which of its kernels updated a voxel); host tables and the
# smoothing offsets are computed without contraction on every host CPU
FILE_FLAGS = {"sj_lean.cu": ["-fmad=false"], "sj_host.cu": ["-Xcompiler", "-ffp-contract=off"]}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, extra_flags=()):
    """Compile and link; returns the path of the shared library."""
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS]
    jobs = []
    objs = []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        op = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(op)
        if force or _stale(op, [sp] + hdrs):
            jobs.append([nvcc, *ARCH, *FLAGS, *FILE_FLAGS.get(src, []), *extra_flags, "-c", sp, "-o", op])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(OUT, objs):
        run([nvcc, *ARCH, "-shared", "-o", OUT, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
