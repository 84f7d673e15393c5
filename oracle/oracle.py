"""TEST INFRASTRUCTURE ONLY: ctypes binding of the CPU oracle
(oracle/_build/libsj_oracle.so).  Imported by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg, never by the
product package.

``OracleFields`` mirrors sim_juncs_gb300.fields.Fields for one instance so
that a parity test can run the same Instance through both.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from sim_juncs_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libsj_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libsjref.so")

_lib = None


def build(force=False):
    """Compile the oracle with the committed Makefile (g++, OpenMP)."""
    args = ["make", "-s", "-C", HERE]
    if force:
        args.insert(1, "-B")
    subprocess.run(args + ["all"], check=True)
    return LIB


def threads():
    """OpenMP threads the oracle's stepping loops use."""
    return int(load().sjo_threads())


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        build()
    lib = C.CDLL(LIB)
    P = C.c_void_p
    D = C.POINTER(C.c_double)
    lib.sjo_last_error.restype = C.c_char_p
    lib.sjo_threads.restype = C.c_int
    lib.sjo_create.argtypes = [C.POINTER(_abi.InstanceDesc), C.POINTER(P)]
    lib.sjo_destroy.argtypes = [P]
    lib.sjo_step.argtypes = [P, C.c_int64]
    lib.sjo_steps_done.argtypes = [P]
    lib.sjo_steps_done.restype = C.c_int64
    lib.sjo_dt.argtypes = [P]
    lib.sjo_dt.restype = C.c_double
    lib.sjo_n_samples.argtypes = [P]
    lib.sjo_n_samples.restype = C.c_int64
    lib.sjo_read_monitors.argtypes = [P, D, C.c_size_t]
    lib.sjo_read_dft.argtypes = [P, D, C.c_size_t]
    lib.sjo_read_field.argtypes = [P, C.c_int, D, C.c_size_t]
    lib.sjo_write_field.argtypes = [P, C.c_int, D, C.c_size_t]
    lib.sjo_read_class_map.argtypes = [P, C.POINTER(C.c_uint8), C.c_size_t]
    lib.sjo_rasterize.argtypes = [C.POINTER(_abi.GridDesc), C.POINTER(_abi.SceneDesc),
                                  C.POINTER(C.c_uint8)]
    lib.sjo_csg_in.argtypes = [C.POINTER(_abi.CsgNode), C.c_int, D, C.c_int64, C.POINTER(C.c_uint8)]
    lib.sjo_rasterize_counts.argtypes = [C.POINTER(_abi.GridDesc), C.POINTER(_abi.SceneDesc),
                                         C.POINTER(C.c_uint8)]
    lib.sjo_smooth_points.argtypes = [C.c_int32, C.c_double, D]
    lib.sjo_in_bound.argtypes = [C.POINTER(_abi.SceneDesc), D, C.c_int64, D]
    lib.sjo_set_design.argtypes = [P, C.POINTER(_abi.DesignDesc)]
    lib.sjo_objective.argtypes = [P, C.POINTER(_abi.ObjectiveDesc), C.c_int64, D]
    lib.sjo_adjoint.argtypes = [P, C.POINTER(_abi.ObjectiveDesc), C.c_int64, D, D]
    lib.sjo_source_dipole.argtypes = [C.POINTER(_abi.SourceDesc), C.c_double, D, D]
    _lib = lib
    return lib


class OracleFields:
    """FP64 CPU restatement of the stepper for one Instance."""

    def __init__(self, instance):
        self.lib = load()
        self.instance = instance
        d, self._holder = instance.to_c()
        h = C.c_void_p()
        if self.lib.sjo_create(C.byref(d), C.byref(h)) != 0:
            raise RuntimeError("oracle create failed: " + self.lib.sjo_last_error().decode())
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self.lib.sjo_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n=1):
        self.lib.sjo_step(self.handle, int(n))

    def set_design(self, design):
        d, self._design = design.to_c()
        if self.lib.sjo_set_design(self.handle, C.byref(d)) != 0:
            raise RuntimeError(self.lib.sjo_last_error().decode())

    def objective(self, objective, n_steps):
        """F after n_steps from rest."""
        o, keep = objective.to_c()
        F = C.c_double()
        self.lib.sjo_objective(self.handle, C.byref(o), int(n_steps), C.byref(F))
        return F.value

    def adjoint(self, objective, n_steps):
        """(F, dF/d eps over the design voxels [k][j][i]) after n_steps from rest."""
        o, keep = objective.to_c()
        shape = self._design.shape
        g = np.zeros(shape, dtype=np.float64)
        F = C.c_double()
        if self.lib.sjo_adjoint(self.handle, C.byref(o), int(n_steps), g.ctypes.data_as(C.POINTER(C.c_double)),
                                C.byref(F)) != 0:
            raise RuntimeError(self.lib.sjo_last_error().decode())
        return F.value, g

    @property
    def steps_done(self):
        return self.lib.sjo_steps_done(self.handle)

    def dt(self):
        return self.lib.sjo_dt(self.handle)

    def monitors(self):
        ns = self.lib.sjo_n_samples(self.handle)
        out = np.zeros((self.instance.n_monitors, ns))
        assert self.lib.sjo_read_monitors(self.handle, out.ctypes.data_as(C.POINTER(C.c_double)), out.size) == 0
        return out

    def dft(self):
        out = np.zeros((self.instance.n_dft, len(self.instance.freqs), 2))
        assert self.lib.sjo_read_dft(self.handle, out.ctypes.data_as(C.POINTER(C.c_double)), out.size) == 0
        return out[..., 0] + 1j * out[..., 1]

    def get_array(self, comp):
        g = self.instance.grid
        out = np.zeros((g.nz, g.ny, g.nx))
        assert self.lib.sjo_read_field(self.handle, comp, out.ctypes.data_as(C.POINTER(C.c_double)), out.size) == 0
        return out

    def set_array(self, comp, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        assert self.lib.sjo_write_field(self.handle, comp, v.ctypes.data_as(C.POINTER(C.c_double)), v.size) == 0

    def class_map(self):
        g = self.instance.grid
        out = np.zeros((3, g.nz, g.ny, g.nx), dtype=np.uint8)
        assert self.lib.sjo_read_class_map(self.handle, out.ctypes.data_as(C.POINTER(C.c_uint8)), out.size) == 0
        return out


def rasterize(grid, scene):
    from sim_juncs_gb300.spec import scene_to_c
    lib = load()
    sc, h = scene_to_c(scene)
    out = np.zeros((3, grid.nz, grid.ny, grid.nx), dtype=np.uint8)
    g = grid.to_c()
    lib.sjo_rasterize(C.byref(g), sc, out.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out


def rasterize_counts(grid, scene):
    """in_bound's per-region counts: [3][n_regions][nz][ny][nx]."""
    from sim_juncs_gb300.spec import scene_to_c
    lib = load()
    sc, h = scene_to_c(scene)
    out = np.zeros((3, len(scene.regions), grid.nz, grid.ny, grid.nx), dtype=np.uint8)
    g = grid.to_c()
    rc = lib.sjo_rasterize_counts(C.byref(g), sc, out.ctypes.data_as(C.POINTER(C.c_uint8)))
    if rc:
        raise RuntimeError(lib.sjo_last_error().decode())
    return out


def smooth_points(n, rad):
    """The smoothing offsets: [8 n][3]."""
    lib = load()
    out = np.zeros((8 * n, 3), dtype=np.float64)
    lib.sjo_smooth_points(n, rad, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def in_bound(scene, points):
    """cgs_material_function::in_bound of the scene's eps at each point."""
    from sim_juncs_gb300.spec import scene_to_c
    lib = load()
    sc, h = scene_to_c(scene)
    pts = np.ascontiguousarray(points, dtype=np.float64)
    out = np.zeros(len(pts), dtype=np.float64)
    rc = lib.sjo_in_bound(sc, pts.ctypes.data_as(C.POINTER(C.c_double)), len(pts),
                          out.ctypes.data_as(C.POINTER(C.c_double)))
    if rc:
        raise RuntimeError(lib.sjo_last_error().decode())
    return out


def csg_in(program, points):
    """in_root(point) for each point (program = list of CsgNode)."""
    lib = load()
    arr = (_abi.CsgNode * len(program))(*program)
    pts = np.ascontiguousarray(points, dtype=np.float64)
    out = np.zeros(len(pts), dtype=np.uint8)
    lib.sjo_csg_in(arr, len(program), pts.ctypes.data_as(C.POINTER(C.c_double)), len(pts),
                   out.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out


def source_dipole(src, t):
    lib = load()
    s = src.to_c()
    re, im = C.c_double(), C.c_double()
    lib.sjo_source_dipole(C.byref(s), t, C.byref(re), C.byref(im))
    return complex(re.value, im.value)
