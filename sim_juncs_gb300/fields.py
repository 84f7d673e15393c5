"""``Fields``: the Python handle on the C ABI, standing where the reference
holds its ``meep::fields`` member (src/disp.hpp:175-177).

Method names follow the calls the reference makes on that object
(src/disp.cpp:557-749): ``step``, ``time``, ``dt``, ``last_source_time``,
``get_field`` (monitor read-back) and ``output`` of a raw component.
"""
import ctypes as C

import numpy as np

from . import _abi
from .spec import Instance

_PREC = {"f64": _abi.F64, "f32": _abi.F32, _abi.F64: _abi.F64, _abi.F32: _abi.F32}
_SCHED = {"fused": _abi.SCHED_FUSED, "split": _abi.SCHED_SPLIT, "tma": _abi.SCHED_TMA,
          _abi.SCHED_FUSED: _abi.SCHED_FUSED, _abi.SCHED_SPLIT: _abi.SCHED_SPLIT,
          _abi.SCHED_TMA: _abi.SCHED_TMA}


class Fields:
    """One or many simulation instances stepped by the CUDA library."""

    def __init__(self, instances, precision="f64", schedule=None, stream=None):
        self.lib = _abi.load_library()
        if isinstance(instances, Instance):
            instances = [instances]
        self.instances = list(instances)
        n = len(self.instances)
        descs = (_abi.InstanceDesc * n)()
        self._holders = []
        for q, inst in enumerate(self.instances):
            d, h = inst.to_c()
            descs[q] = d
            self._holders.append(h)
        self.precision = _PREC[precision]
        handle = C.c_void_p()
        _abi.check(self.lib, self.lib.sj_batch_create(n, descs, self.precision, C.byref(handle)))
        self.handle = handle
        self._holders = None  # the library copied everything it needs
        self._designs = {}    # instance -> design eps shape
        if schedule is not None:  # default: fused for f32, split for f64
            self.set_schedule(schedule)
        if stream is not None:
            self.set_stream(stream)

    # ------------------------------------------------------------ lifecycle
    def close(self):
        if getattr(self, "handle", None):
            self.lib.sj_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, code):
        return _abi.check(self.lib, code, self.handle)

    def set_stream(self, stream):
        """Run on `stream` (a cudaStream_t as int, or a torch.cuda.Stream)."""
        ptr = getattr(stream, "cuda_stream", stream)
        self._ck(self.lib.sj_set_stream(self.handle, C.c_void_p(ptr)))

    def set_schedule(self, schedule):
        self._ck(self.lib.sj_set_schedule(self.handle, _SCHED[schedule]))

    def set_tiling(self, tile_y, ring, zseg):
        """Tiling of the selected single-pass schedule (fused: only zseg; tma:
        32 x tile_y tiles, TMA ring depth, z segments)."""
        self._ck(self.lib.sj_set_tiling(self.handle, int(tile_y), int(ring), int(zseg)))

    def set_fused_columns(self, columns):
        """Fused schedule: 0 = two columns per thread where rows are whole
        (default), 1 = one column per thread everywhere (same results)."""
        self._ck(self.lib.sj_set_fused_columns(self.handle, int(columns)))

    def set_fused_launch(self, mode):
        """"grouped" (one launch per group and tile class) or "queue" (one
        launch of resident blocks claiming every group's tiles)."""
        self._ck(self.lib.sj_set_fused_launch(self.handle, {"grouped": 0, "queue": 1}[mode]))

    def fused_launch(self):
        return {0: "grouped", 1: "queue"}[int(self.lib.sj_get_fused_launch(self.handle))]

    def tiling(self):
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        self._ck(self.lib.sj_get_tiling(self.handle, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def autotune(self, steps=3):
        """Pick the fused tiling by timing state-preserving launches.
        Returns (tile_y, ring, zseg, ms_per_step)."""
        a, b, c, ms = C.c_int32(), C.c_int32(), C.c_int32(), C.c_float()
        self._ck(self.lib.sj_autotune(self.handle, int(steps), C.byref(a), C.byref(b), C.byref(c),
                                      C.byref(ms)))
        return a.value, b.value, c.value, ms.value

    def synchronize(self):
        self._ck(self.lib.sj_synchronize(self.handle))

    # ------------------------------------------------------------ stepping
    def step(self, n=1):
        """n iterations of the reference loop body (asynchronous)."""
        self._ck(self.lib.sj_step(self.handle, int(n)))

    def step_graph(self, n, chunk=50):
        self._ck(self.lib.sj_step_graph(self.handle, int(n), int(chunk)))

    # ------------------------------------------------------------ queries
    @property
    def n_instances(self):
        return len(self.instances)

    @property
    def steps_done(self):
        return self.lib.sj_steps_done(self.handle)

    def transfer_bytes(self):
        """(host->device, device->host) bytes this sim has copied so far."""
        a, b = C.c_int64(), C.c_int64()
        self._ck(self.lib.sj_transfer_bytes(self.handle, C.byref(a), C.byref(b)))
        return a.value, b.value

    def dt(self, inst=0):
        return self.lib.sj_dt(self.handle, inst)

    def time(self, inst=0):
        return self.lib.sj_time(self.handle, inst)

    def last_source_time(self, inst=0):
        return self.lib.sj_last_source_time(self.handle, inst)

    def voxels(self, inst=None):
        if inst is None:
            return sum(self.lib.sj_voxels(self.handle, q) for q in range(self.n_instances))
        return self.lib.sj_voxels(self.handle, inst)

    def bytes_per_step(self, inst=None):
        if inst is None:
            return sum(self.lib.sj_bytes_per_step(self.handle, q) for q in range(self.n_instances))
        return self.lib.sj_bytes_per_step(self.handle, inst)

    # ------------------------------------------------------------ adjoint
    def set_design(self, design, inst=0):
        """Per-voxel eps on a box (spec.Design), or None to remove it.  An
        instance with a design region steps with the split schedule."""
        if design is None:
            self._ck(self.lib.sj_set_design(self.handle, inst, None))
            self._designs.pop(inst, None)
            return
        d, keep = design.to_c()
        self._ck(self.lib.sj_set_design(self.handle, inst, C.byref(d)))
        self._designs[inst] = keep.shape

    def adjoint_gradient(self, objectives, n_steps, checkpoint_every=200):
        """Run n_steps from rest and the discrete adjoint back.  objectives:
        one spec.Objective per instance (or one for a single instance).
        Returns (F per instance, dF/d eps per instance shaped like its design
        eps, None where it has no design region)."""
        if not isinstance(objectives, (list, tuple)):
            objectives = [objectives]
        assert len(objectives) == self.n_instances
        arr = (_abi.ObjectiveDesc * self.n_instances)()
        keep = []
        for q, ob in enumerate(objectives):
            o, k = ob.to_c()
            arr[q] = o
            keep.append(k)
        sizes = [int(np.prod(self._designs[q])) if q in self._designs else 0 for q in range(self.n_instances)]
        g = np.zeros(max(1, sum(sizes)), dtype=np.float64)
        F = np.zeros(self.n_instances, dtype=np.float64)
        self._ck(self.lib.sj_adjoint_gradient(self.handle, arr, int(n_steps), int(checkpoint_every),
                                              g.ctypes.data_as(C.POINTER(C.c_double)), g.size,
                                              F.ctypes.data_as(C.POINTER(C.c_double))))
        out, off = [], 0
        for q, n in enumerate(sizes):
            out.append(g[off:off + n].reshape(self._designs[q]).copy() if n else None)
            off += n
        return F, out

    def objective(self, objectives, n_steps):
        """F per instance after n_steps from rest (the forward half of
        adjoint_gradient)."""
        if not isinstance(objectives, (list, tuple)):
            objectives = [objectives]
        assert len(objectives) == self.n_instances
        arr = (_abi.ObjectiveDesc * self.n_instances)()
        keep = []
        for q, ob in enumerate(objectives):
            o, k = ob.to_c()
            arr[q] = o
            keep.append(k)
        F = np.zeros(self.n_instances, dtype=np.float64)
        self._ck(self.lib.sj_objective(self.handle, arr, int(n_steps), F.ctypes.data_as(C.POINTER(C.c_double))))
        return F

    def schedule_name(self):
        """The schedule in use: "fused", "split" or "tma"."""
        return {_abi.SCHED_FUSED: "fused", _abi.SCHED_SPLIT: "split", _abi.SCHED_TMA: "tma"}[
            int(self.lib.sj_get_schedule(self.handle))]

    def launches_per_step(self):
        """Kernel launches one step issues under the current schedule."""
        return int(self.lib.sj_launches_per_step(self.handle))

    def n_samples(self, inst=0):
        return self.lib.sj_n_samples(self.handle, inst)

    # ------------------------------------------------------------ read-back
    def monitors(self, inst=0):
        """field_times: [monitor][sample] (float64)."""
        nm = self.instances[inst].n_monitors
        ns = self.n_samples(inst)
        out = np.zeros((nm, ns), dtype=np.float64)
        self._ck(self.lib.sj_read_monitors(self.handle, inst,
                                           out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out

    def monitor_spectrum(self, inst=0):
        """The per-monitor spectrum save_field_times writes: [monitor][N']
        complex, N' = 2^floor(log2 samples)."""
        nm = self.instances[inst].n_monitors
        npts = int(self.lib.sj_monitor_spectrum_length(self.handle, inst))
        out = np.zeros((nm, max(npts, 0), 2), dtype=np.float64)
        self._ck(self.lib.sj_monitor_spectrum(self.handle, inst, out.ctypes.data_as(C.POINTER(C.c_double)),
                                              out.size))
        return out[..., 0] + 1j * out[..., 1]

    def dft(self, inst=0):
        """Running DFT sums: complex [dft_probe][freq]."""
        nd = self.instances[inst].n_dft
        nf = len(self.instances[inst].freqs)
        out = np.zeros((nd, nf, 2), dtype=np.float64)
        self._ck(self.lib.sj_read_dft(self.handle, inst,
                                      out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out[..., 0] + 1j * out[..., 1]

    def get_array(self, component, inst=0):
        """Full component array [nz][ny][nx] as float64 (dump_raw)."""
        g = self.instances[inst].grid
        out = np.zeros((g.nz, g.ny, g.nx), dtype=np.float64)
        self._ck(self.lib.sj_read_field(self.handle, inst, component,
                                        out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out

    def set_snapshots(self, component, every, depth=2, inst=0):
        """Stream `component` to host memory every `every` steps (dump_raw),
        overlapped with stepping; `depth` snapshots may wait to be taken.
        every = 0 switches it off."""
        self._ck(self.lib.sj_set_snapshots(self.handle, inst, component, int(every), int(depth)))

    def take_snapshot(self, inst=0, out=None):
        """The oldest snapshot not yet taken as (step, [nz][ny][nx] float64),
        or None; `out` (a C-contiguous float64 array of that shape) is
        filled instead of a new array."""
        g = self.instances[inst].grid
        if out is None:
            out = np.empty((g.nz, g.ny, g.nx), dtype=np.float64)
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == g.nx * g.ny * g.nz
        step = C.c_int64(-1)
        self._ck(self.lib.sj_take_snapshot(self.handle, inst, C.byref(step),
                                           out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return None if step.value < 0 else (step.value, out)

    def snapshots_pending(self, inst=0):
        return int(self.lib.sj_snapshots_pending(self.handle, inst))

    def set_array(self, component, values, inst=0):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._ck(self.lib.sj_write_field(self.handle, inst, component,
                                         v.ctypes.data_as(C.POINTER(C.c_double)), v.size))

    def class_map(self, inst=0):
        g = self.instances[inst].grid
        out = np.zeros((3, g.nz, g.ny, g.nx), dtype=np.uint8)
        self._ck(self.lib.sj_read_class_map(self.handle, inst,
                                            out.ctypes.data_as(C.POINTER(C.c_uint8)), out.size))
        return out

    def max_abs_e(self, inst=0):
        v = C.c_double()
        self._ck(self.lib.sj_max_abs_e(self.handle, inst, C.byref(v)))
        return v.value

    # ------------------------------------------------------------ diagnostics
    def energy(self, inst=0):
        """Discrete leapfrog energy (FP64 sums; conserved by a closed,
        source-free, non-dispersive cavity)."""
        v = C.c_double()
        self._ck(self.lib.sj_energy(self.handle, inst, C.byref(v)))
        return v.value

    def flux(self, rows, dA, inst=0):
        """Flux spectrum through the points whose DFT rows (E1, E2, H1, H2)
        are the rows of `rows` ([n_points][4]); one value per DFT frequency."""
        r = np.ascontiguousarray(rows, dtype=np.int32).reshape(-1, 4)
        out = np.zeros(len(self.instances[inst].freqs), dtype=np.float64)
        self._ck(self.lib.sj_flux(self.handle, inst, len(r), r.ctypes.data_as(C.POINTER(C.c_int32)),
                                  float(dA), out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out

    # ------------------------------------------------------------ bounded waits
    def set_wait_limit(self, ns):
        """Limit of a TMA-schedule wait on a tile copy (0 = the default 100 ms)."""
        self._ck(self.lib.sj_set_wait_limit(self.handle, int(ns)))

    def set_test_stall(self, on):
        """Test hook: the TMA schedule's first tile block skips a plane's
        copy, so its wait runs out and SJ_E_TIMEOUT is reported."""
        self._ck(self.lib.sj_set_test_stall(self.handle, 1 if on else 0))

    # ------------------------------------------------------------ divergence guard
    def set_divergence_guard(self, bound):
        """Monitor samples with |value| > bound (or not finite) stop the loop
        (src/disp.cpp:727-729 flags samples above 1000); 0 = off."""
        self._ck(self.lib.sj_set_divergence_guard(self.handle, float(bound)))

    def divergence(self):
        """(step, instance, monitor, value) of the sample that tripped the
        guard, or None."""
        s, q, m, v = C.c_int64(), C.c_int32(), C.c_int32(), C.c_double()
        r = self.lib.sj_divergence(self.handle, C.byref(s), C.byref(q), C.byref(m), C.byref(v))
        return (s.value, q.value, m.value, v.value) if r == 1 else None


def rasterize(grid, scene):
    """Region bitmasks at the Ex/Ey/Ez points of `grid` ([3][nz][ny][nx] uint8)."""
    from .spec import scene_to_c
    lib = _abi.load_library()
    sc, h = scene_to_c(scene)
    out = np.zeros((3, grid.nz, grid.ny, grid.nx), dtype=np.uint8)
    g = grid.to_c()
    _abi.check(lib, lib.sj_rasterize(C.byref(g), sc, out.ctypes.data_as(C.POINTER(C.c_uint8))))
    return out


def rasterize_counts(grid, scene):
    """Per-region fill counts at the Ex/Ey/Ez points of `grid` under the scene's
    stochastic smoothing ([3][n_regions][nz][ny][nx] uint8, 0 .. 8 smooth_n + 1)."""
    from .spec import scene_to_c
    lib = _abi.load_library()
    sc, h = scene_to_c(scene)
    out = np.zeros((3, len(scene.regions), grid.nz, grid.ny, grid.nx), dtype=np.uint8)
    g = grid.to_c()
    _abi.check(lib, lib.sj_rasterize_counts(C.byref(g), sc, out.ctypes.data_as(C.POINTER(C.c_uint8))))
    return out


def smooth_points(smooth_n, smooth_rad):
    """The smoothing offsets d_j of cgs_material_function ([8 smooth_n][3])."""
    lib = _abi.load_library()
    out = np.zeros((8 * smooth_n, 3), dtype=np.float64)
    _abi.check(lib, lib.sj_smooth_points(smooth_n, smooth_rad, out.ctypes.data_as(C.POINTER(C.c_double)),
                                         out.size))
    return out
