"""Generate cgs_reference.json: golden vectors from the reference's own CGS code.

Run where the reference checkout exists (argument: its root):

    make -C oracle ref
    python tests/golden/make_golden.py <reference root>

oracle/_ref/libsjref.so is the reference's src/cgs_read.cpp, cgs_data.cpp and
cgs.cpp compiled unmodified, plus oracle/ref_shim.cpp.  For every .geom file
of the reference's tests/ and junctions/ that parses, and every root
composite of it, the file records:

  * the postfix program (sj_csg_node list) the integration walk flattens the
    root into,
  * the root's eps metadata and susceptibilities (parse_susceptibilities,
    src/disp.cpp:418-454),
  * composite_object::in (src/cgs.cpp:431-456) at the E-component Yee points
    of a 32^3 grid (x: origin + (i + 1/2) dx, i.e. the points the rasteriser
    samples), packed one bit per point and zlib-compressed,
  * for tests/test.geom, in() at the six points src/main_test.cpp:1555-1564
    checks.

fft_reference.json holds the reference's fft (src/data_utils.cpp:413-427) of
seeded series of several lengths.

volume_reference.json holds, for the sphere, cylinder and plane of the
reference's volume test (src/main_test.cpp:1448-1489), the reference's own
in() (the primitives built with its constructors) at the test's 10000 sample
points: the Numerical Recipes LCG of src/main_test.hpp:17-33 from TEST_SEED,
one point per four draws.

The parser executes snapshot(...) statements (it draws an image file), so
each file is parsed from a copy without them, written to a temporary
directory; snapshots do not change the geometry.  The
junction files read their parameters from the context bound_geom builds
(src/disp.cpp:28-50) and the --opts string scripts/run.sh passes; the values
used are in OPTS below.
"""
import base64
import ctypes as C
import glob
import json
import os
import re
import sys
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from sim_juncs_gb300 import _abi  # noqa: E402

LIB = os.path.join(REPO, "oracle", "_ref", "libsjref.so")
OUT = os.path.join(HERE, "cgs_reference.json")
GRID_N = 32
# scripts/run.sh passes width, thick, inf_thick, wavelen and n_cycles
OPTS = "width=0.1;thick=0.2;inf_thick=0;wavelen=0.7;n_cycles=0.5;snap_file=\"unused.pgm\""
TEST_POINTS = [[.45, .45, .45], [.45, .41, .6], [.65, .45, .41], [.71, .51, .51], [.55, .45, .45],
               [.55, .41, .85]]
NODE_FIELDS = ("op", "invert", "m", "t", "c", "p")


def load_lib():
    lib = C.CDLL(LIB)
    lib.sjref_load.argtypes = [C.c_char_p]
    lib.sjref_load_ctx.argtypes = [C.c_char_p, C.c_double, C.c_double, C.c_double, C.c_char_p]
    lib.sjref_n_roots.argtypes = [C.c_int]
    lib.sjref_flatten.argtypes = [C.c_int, C.c_int, C.POINTER(_abi.CsgNode), C.c_int]
    lib.sjref_root_eps.argtypes = [C.c_int, C.c_int, C.c_double]
    lib.sjref_root_eps.restype = C.c_double
    D = C.POINTER(C.c_double)
    lib.sjref_root_poles.argtypes = [C.c_int, C.c_int, D, D, D, C.POINTER(C.c_int), C.c_int]
    lib.sjref_in.argtypes = [C.c_int, C.c_int, D, C.c_int64, C.POINTER(C.c_uint8)]
    return lib


def strip_snapshots(src, dst):
    text = open(src).read()
    text = re.sub(r"^\s*snapshot\(.*$", "", text, flags=re.M)
    with open(dst, "w") as fh:
        fh.write(text)


def conf_values(path):
    vals = {}
    if os.path.exists(path):
        for line in open(path):
            m = re.match(r"\s*(\w+)\s*=\s*([-0-9.eE+]+)\s*$", line)
            if m:
                vals[m.group(1)] = float(m.group(2))
    return vals


def node_to_json(n):
    return {"op": n.op, "invert": n.invert, "m": list(n.m), "t": list(n.t), "c": list(n.c), "p": list(n.p)}


def yee_points(origin, dx, n):
    """E-component sample points of an n^3 grid, ordered [c][k][j][i]."""
    idx = np.arange(n, dtype=np.float64)
    pts = []
    for c in range(3):
        ax = [origin[a] + (idx + (0.5 if c == a else 0.0)) * dx for a in range(3)]
        z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
        pts.append(np.stack([x, y, z], axis=-1).reshape(-1, 3))
    return np.concatenate(pts)


def ref_in(lib, h, r, pts):
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros(len(pts), dtype=np.uint8)
    rc = lib.sjref_in(h, r, pts.ctypes.data_as(C.POINTER(C.c_double)), len(pts),
                      out.ctypes.data_as(C.POINTER(C.c_uint8)))
    assert rc == 0
    return out


def pack_bits(bits):
    return base64.b64encode(zlib.compress(np.packbits(bits).tobytes(), 9)).decode()


def record(lib, h, name, origin, dx, ambient):
    roots = []
    for r in range(lib.sjref_n_roots(h)):
        cap = 4096
        nodes = (_abi.CsgNode * cap)()
        n = lib.sjref_flatten(h, r, nodes, cap)
        assert 0 < n <= cap, (name, r, n)
        w0, ga, sg = (C.c_double * 16)(), (C.c_double * 16)(), (C.c_double * 16)()
        dr = (C.c_int * 16)()
        npl = lib.sjref_root_poles(h, r, w0, ga, sg, dr, 16)
        poles = [{"omega_0": w0[q], "gamma": ga[q], "sigma": sg[q], "drude": bool(dr[q])}
                 for q in range(max(npl, 0))]
        inside = ref_in(lib, h, r, yee_points(origin, dx, GRID_N))
        roots.append({"nodes": [node_to_json(nodes[q]) for q in range(n)],
                      "eps": lib.sjref_root_eps(h, r, ambient), "poles": poles,
                      "inside_bits": pack_bits(inside), "n_inside": int(inside.sum())})
    return {"grid": {"n": GRID_N, "origin": list(origin), "dx": dx}, "ambient_eps": ambient, "roots": roots}


FFT_OUT = os.path.join(HERE, "fft_reference.json")
FFT_SIZES = (1, 2, 3, 7, 8, 16, 33, 64, 100, 128, 257, 1000)


def write_fft(lib):
    """The reference's fft (src/data_utils.cpp:413-427) on seeded real and
    complex series of several lengths, powers of two included."""
    lib.sjref_fft.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_double),
                              C.c_int64]
    lib.sjref_fft.restype = C.c_int64
    rng = np.random.default_rng(7)
    cases = []
    for n in FFT_SIZES:
        for cplx in (False, True):
            re = rng.standard_normal(n)
            im = rng.standard_normal(n) if cplx else np.zeros(n)
            out = np.zeros(2 * n)
            m = lib.sjref_fft(re.ctypes.data_as(C.POINTER(C.c_double)), im.ctypes.data_as(C.POINTER(C.c_double)), n,
                              out.ctypes.data_as(C.POINTER(C.c_double)), n)
            cases.append({"n": n, "re": re.tolist(), "im": im.tolist(), "out_len": int(m),
                          "out": out[:2 * m].tolist()})
    with open(FFT_OUT, "w") as fh:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": cases}, fh)


VOLUME_OUT = os.path.join(HERE, "volume_reference.json")
TEST_SEED = 31415926
TEST_N = 10000
# the primitives of src/main_test.cpp:1452-1459 (kind, constructor arguments)
VOLUME_PRIMITIVES = {"sphere": (0, [0.5, 0.5, 0.5, 0.5]),
                     "cylinder": (1, [0.5, 0.5, 0.5, 0.5, 0.5, 0.5]),
                     "plane": (2, [1.0, 1.0, 0.0, 0.0, 1.0, 1.0, 1.0, 0.0, 1.0])}


def lcg_points(n=TEST_N, seed=TEST_SEED):
    """The volume test's samples: state = lcg(lcg(seed)); per point three
    draws for x, y, z and one more (src/main_test.cpp:1449-1469)."""
    def lcg(v):
        return (v * 1664525 + 1013904223) & 0xFFFFFFFF
    state = lcg(lcg(seed))
    pts = np.zeros((n, 3))
    for q in range(n):
        for a in range(3):
            state = lcg(state)
            pts[q, a] = state / 4294967295.0
        state = lcg(state)
    return pts


def write_volumes(lib):
    lib.sjref_primitive_in.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int64,
                                       C.POINTER(C.c_uint8)]
    pts = np.ascontiguousarray(lcg_points())
    prims = {}
    for name, (kind, args) in VOLUME_PRIMITIVES.items():
        a = (C.c_double * len(args))(*args)
        out = np.zeros(len(pts), dtype=np.uint8)
        rc = lib.sjref_primitive_in(kind, a, pts.ctypes.data_as(C.POINTER(C.c_double)), len(pts),
                                    out.ctypes.data_as(C.POINTER(C.c_uint8)))
        assert rc == 0
        prims[name] = {"kind": kind, "args": args, "inside_bits": pack_bits(out), "n_inside": int(out.sum())}
    with open(VOLUME_OUT, "w") as fh:
        json.dump({"generator": "tests/golden/make_golden.py", "seed": TEST_SEED, "n": TEST_N,
                   "primitives": prims}, fh, indent=1)


def main(ref_root):
    lib = load_lib()
    scratch = tempfile.TemporaryDirectory()
    SCRATCH = scratch.name
    out = {"generator": "tests/golden/make_golden.py", "files": {}}
    for path in sorted(glob.glob(os.path.join(ref_root, "tests", "*.geom"))):
        name = os.path.relpath(path, ref_root)
        tmp = os.path.join(SCRATCH, name.replace(os.sep, "__"))
        strip_snapshots(path, tmp)
        h = lib.sjref_load(tmp.encode())
        if h < 0 or lib.sjref_n_roots(h) < 1:
            continue
        entry = record(lib, h, name, (0.0, 0.0, 0.0), 1.0 / GRID_N, 1.0)
        if name == os.path.join("tests", "test.geom"):
            pts = np.array(TEST_POINTS)
            entry["test_points"] = {"points": TEST_POINTS, "inside": ref_in(lib, h, 0, pts).tolist()}
        out["files"][name] = entry
    for path in sorted(glob.glob(os.path.join(ref_root, "junctions", "*", "junc.geom"))):
        name = os.path.relpath(path, ref_root)
        conf = conf_values(os.path.join(os.path.dirname(path), "params.conf"))
        pml, length, ums = conf.get("pml_thickness", 1.0), conf.get("length", 16.0), conf.get("um_scale", 1.0)
        tmp = os.path.join(SCRATCH, name.replace(os.sep, "__"))
        strip_snapshots(path, tmp)
        h = lib.sjref_load_ctx(tmp.encode(), pml, length, ums, OPTS.encode())
        if h < 0 or lib.sjref_n_roots(h) < 1:
            print("skip", name, h)
            continue
        # a 32^3 window around the cell centre, one micron across
        mid = pml + length / 2
        half = 0.5 * ums
        entry = record(lib, h, name, (mid - half, mid - half, mid - half), 2 * half / GRID_N,
                       conf.get("ambient_eps", 1.0))
        entry["context"] = {"pml_thickness": pml, "length": length, "um_scale": ums, "opts": OPTS}
        out["files"][name] = entry
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=1)
    write_fft(lib)
    write_volumes(lib)
    for name, e in out["files"].items():
        print(name, [(len(r["nodes"]), r["n_inside"], r["eps"], len(r["poles"])) for r in e["roots"]])


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SJ_REFERENCE")
    if not root:
        sys.exit(f"usage: python {sys.argv[0]} <reference checkout root>  (or set SJ_REFERENCE)")
    main(root)
