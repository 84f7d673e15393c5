"""ctypes mirror of include/sj.h and the loader of libsj_gb300.so.

The structures below must match include/sj.h field for field; the library
exports ``sj_abi_struct_size`` so the tests can check every layout.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsj_gb300.so")

SJ_OK = 0
SJ_E_INVALID = -1
SJ_E_CUDA = -2
SJ_E_NOMEM = -3
SJ_E_RANGE = -4
SJ_E_DIVERGED = -5
SJ_E_TIMEOUT = -6

EX, EY, EZ, HX, HY, HZ = range(6)
COMPONENTS = {"Ex": EX, "Ey": EY, "Ez": EZ, "Hx": HX, "Hy": HY, "Hz": HZ}
F64, F32 = 0, 1
SCHED_FUSED, SCHED_SPLIT, SCHED_TMA = 0, 1, 2
LAUNCH_GROUPED, LAUNCH_QUEUE = 0, 1
SRC_GAUSSIAN, SRC_CONTINUOUS = 0, 1
PROBE_MONITOR, PROBE_DFT = 1, 2
CSG_BOX, CSG_SPHERE, CSG_CYLINDER, CSG_PLANE = 0, 1, 2, 3
CSG_UNION, CSG_INTERSECT, CSG_PASS, CSG_CONST, CSG_NOOP = 4, 5, 6, 7, 8
MAX_POLES, MAX_SOURCES, MAX_REGIONS = 8, 4, 8
RASTER_STATIC_NODES = 512
EPS_SUM, EPS_FIRST = 0, 1


class GridDesc(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("dx", C.c_double), ("dt", C.c_double), ("origin", C.c_double * 3)]


class Pole(C.Structure):
    _fields_ = [("omega_0", C.c_double), ("gamma", C.c_double), ("drude", C.c_int32),
                ("_pad", C.c_int32)]


class CsgNode(C.Structure):
    _fields_ = [("op", C.c_int32), ("invert", C.c_int32), ("m", C.c_double * 9),
                ("t", C.c_double * 9), ("c", C.c_double * 3), ("p", C.c_double * 4)]


class RegionDesc(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("nodes", C.POINTER(CsgNode)), ("eps", C.c_double),
                ("n_poles", C.c_int32), ("poles", C.POINTER(Pole)),
                ("sigma", C.POINTER(C.c_double))]


class SceneDesc(C.Structure):
    _fields_ = [("ambient_eps", C.c_double), ("n_regions", C.c_int32), ("combine", C.c_int32),
                ("regions", C.POINTER(RegionDesc)), ("smooth_n", C.c_int32), ("smooth_rad", C.c_double)]


class MaterialDesc(C.Structure):
    _fields_ = [("n_classes", C.c_int32), ("eps_inf", C.POINTER(C.c_double)),
                ("n_poles", C.c_int32), ("poles", C.POINTER(Pole)),
                ("sigma", C.POINTER(C.c_double)), ("class_map", C.POINTER(C.c_uint8)),
                ("scene", C.POINTER(SceneDesc))]


class PmlDesc(C.Structure):
    _fields_ = [("thickness", (C.c_double * 2) * 3), ("r_asymptotic", C.c_double),
                ("power", C.c_double), ("alpha", C.c_double)]


class SourceDesc(C.Structure):
    _fields_ = [("component", C.c_int32), ("kind", C.c_int32), ("frequency", C.c_double),
                ("width", C.c_double), ("phase", C.c_double), ("start_time", C.c_double),
                ("end_time", C.c_double), ("amplitude", C.c_double * 2),
                ("lo", C.c_double * 3), ("hi", C.c_double * 3)]


class ProbeDesc(C.Structure):
    _fields_ = [("component", C.c_int32), ("flags", C.c_int32), ("pos", C.c_double * 3)]


class InstanceDesc(C.Structure):
    _fields_ = [("grid", GridDesc), ("material", MaterialDesc), ("pml", PmlDesc),
                ("n_sources", C.c_int32), ("sources", C.POINTER(SourceDesc)),
                ("n_probes", C.c_int32), ("probes", C.POINTER(ProbeDesc)),
                ("n_freqs", C.c_int32), ("freqs", C.POINTER(C.c_double)),
                ("save_span", C.c_int32)]


class DesignDesc(C.Structure):
    _fields_ = [("lo", C.c_int32 * 3), ("n", C.c_int32 * 3), ("eps", C.POINTER(C.c_double))]


class ObjectiveDesc(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("cells", C.POINTER(C.c_int32)), ("comp_mask", C.c_int32),
                ("_pad", C.c_int32), ("frequency", C.c_double)]


class PhaseResult(C.Structure):
    _fields_ = [("f0", C.c_double), ("phi", C.c_double), ("t0_corr", C.c_double), ("t0", C.c_double),
                ("amp", C.c_double * 2), ("mu", C.c_double), ("sig", C.c_double), ("skew", C.c_double),
                ("f0_ind", C.c_int32), ("band_lo", C.c_int32), ("band_hi", C.c_int32),
                ("lowpass_steps", C.c_int32), ("status", C.c_int32), ("_pad", C.c_int32)]


PHASE_OK, PHASE_NARROW_BAND, PHASE_EMPTY_BAND, PHASE_BAD_F0, PHASE_BAD_T0, PHASE_WIDE_BAND = range(6)

STRUCTS = {0: GridDesc, 1: Pole, 2: CsgNode, 3: RegionDesc, 4: SceneDesc, 5: MaterialDesc,
           6: PmlDesc, 7: SourceDesc, 8: ProbeDesc, 9: InstanceDesc, 10: DesignDesc, 11: ObjectiveDesc,
           12: PhaseResult}

_P = C.c_void_p
_D = C.POINTER(C.c_double)
_U8 = C.POINTER(C.c_uint8)

# name -> (restype, argtypes)
SIGNATURES = {
    "sj_abi_version": (C.c_int, []),
    "sj_abi_struct_size": (C.c_int64, [C.c_int32]),
    "sj_last_error": (C.c_char_p, [_P]),
    "sj_create": (C.c_int, [C.POINTER(InstanceDesc), C.c_int32, C.POINTER(_P)]),
    "sj_batch_create": (C.c_int, [C.c_int32, C.POINTER(InstanceDesc), C.c_int32, C.POINTER(_P)]),
    "sj_destroy": (C.c_int, [_P]),
    "sj_set_stream": (C.c_int, [_P, _P]),
    "sj_set_schedule": (C.c_int, [_P, C.c_int32]),
    "sj_synchronize": (C.c_int, [_P]),
    "sj_set_tiling": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "sj_get_tiling": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "sj_autotune": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                              C.POINTER(C.c_int32), C.POINTER(C.c_float)]),
    "sj_step": (C.c_int, [_P, C.c_int64]),
    "sj_step_graph": (C.c_int, [_P, C.c_int64, C.c_int32]),
    "sj_steps_done": (C.c_int64, [_P]),
    "sj_n_instances": (C.c_int32, [_P]),
    "sj_transfer_bytes": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "sj_time": (C.c_double, [_P, C.c_int32]),
    "sj_dt": (C.c_double, [_P, C.c_int32]),
    "sj_last_source_time": (C.c_double, [_P, C.c_int32]),
    "sj_n_samples": (C.c_int64, [_P, C.c_int32]),
    "sj_voxels": (C.c_int64, [_P, C.c_int32]),
    "sj_bytes_per_step": (C.c_double, [_P, C.c_int32]),
    "sj_launches_per_step": (C.c_int32, [_P]),
    "sj_get_schedule": (C.c_int32, [_P]),
    "sj_set_design": (C.c_int, [_P, C.c_int32, C.POINTER(DesignDesc)]),
    "sj_adjoint_gradient": (C.c_int, [_P, C.POINTER(ObjectiveDesc), C.c_int64, C.c_int32, _D, C.c_size_t, _D]),
    "sj_objective": (C.c_int, [_P, C.POINTER(ObjectiveDesc), C.c_int64, _D]),
    "sj_monitor_spectrum_length": (C.c_int64, [_P, C.c_int32]),
    "sj_monitor_spectrum": (C.c_int, [_P, C.c_int32, _D, C.c_size_t]),
    "sj_read_monitors": (C.c_int, [_P, C.c_int32, _D, C.c_size_t]),
    "sj_read_dft": (C.c_int, [_P, C.c_int32, _D, C.c_size_t]),
    "sj_read_field": (C.c_int, [_P, C.c_int32, C.c_int32, _D, C.c_size_t]),
    "sj_set_snapshots": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "sj_set_fused_columns": (C.c_int, [_P, C.c_int32]),
    "sj_set_fused_launch": (C.c_int, [_P, C.c_int32]),
    "sj_get_fused_launch": (C.c_int32, [_P]),
    "sj_take_snapshot": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_int64), _D, C.c_size_t]),
    "sj_snapshots_pending": (C.c_int32, [_P, C.c_int32]),
    "sj_write_field": (C.c_int, [_P, C.c_int32, C.c_int32, _D, C.c_size_t]),
    "sj_read_class_map": (C.c_int, [_P, C.c_int32, _U8, C.c_size_t]),
    "sj_max_abs_e": (C.c_int, [_P, C.c_int32, _D]),
    "sj_set_divergence_guard": (C.c_int, [_P, C.c_double]),
    "sj_energy": (C.c_int, [_P, C.c_int32, _D]),
    "sj_extract_phases": (C.c_int, [C.c_int32, C.c_int32, _D, _D, C.c_double, C.POINTER(PhaseResult)]),
    "sj_extract_monitor_phases": (C.c_int, [_P, C.c_double, C.POINTER(PhaseResult), C.c_size_t]),
    "sj_flux": (C.c_int, [_P, C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.c_double, _D, C.c_size_t]),
    "sj_set_wait_limit": (C.c_int, [_P, C.c_int64]),
    "sj_set_test_stall": (C.c_int, [_P, C.c_int32]),
    "sj_divergence": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int32), _D]),
    "sj_rasterize": (C.c_int, [C.POINTER(GridDesc), C.POINTER(SceneDesc), _U8]),
    "sj_rasterize_counts": (C.c_int, [C.POINTER(GridDesc), C.POINTER(SceneDesc), _U8]),
    "sj_smooth_points": (C.c_int, [C.c_int32, C.c_double, C.POINTER(C.c_double), C.c_size_t]),
    "sj_rasterize_static": (C.c_int, [C.POINTER(GridDesc), C.POINTER(SceneDesc), _P, _P]),
    "sj_source_dipole": (C.c_int, [C.POINTER(SourceDesc), C.c_double, _D, _D]),
    "sj_source_current": (C.c_int, [C.POINTER(SourceDesc), C.c_double, C.c_double, _D, _D]),
    "sj_source_last_time": (C.c_double, [C.POINTER(SourceDesc)]),
}

_lib = None


class SJError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"sj error {code}: {msg}")
        self.code = code


# SJ_ABI_VERSION of include/sj.h that these ctypes mirrors follow
ABI_VERSION = 3


def load_library(path=LIB_PATH):
    """Load the CUDA library; raises if it was not built (no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build it with `python -m sim_juncs_gb300.build` "
            "(the stepper has no CPU fallback)")
    lib = C.CDLL(path)
    # the version first: a library of another ABI may lack later symbols
    lib.sj_abi_version.restype = C.c_int
    lib.sj_abi_version.argtypes = []
    if lib.sj_abi_version() != ABI_VERSION:
        raise ImportError(f"{path} implements ABI {lib.sj_abi_version()}, these bindings ABI {ABI_VERSION}: "
                          "rebuild it with `python -m sim_juncs_gb300.build`")
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(lib, code, handle=None):
    if code != SJ_OK:
        msg = lib.sj_last_error(handle)
        raise SJError(code, msg.decode() if msg else "")
    return code
