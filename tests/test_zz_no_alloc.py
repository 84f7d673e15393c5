"""The allocation-free rasteriser entry point, through the C ABI.

sj_rasterize_static serves callers that cannot call cudaMalloc (hosts that
hand out device memory from their own pool or caching allocator, loops that
must not stall on the device-synchronising cudaMalloc/cudaFree): it writes
into a device buffer the caller owns and stages the CSG program in a static
device array.  Two calls in a row, on two
different scenes, must each give exactly what the allocating sj_rasterize
gives (integer masks: bit-exact).  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from sim_juncs_gb300 import _abi
from sim_juncs_gb300.configs import bowtie_instance, junction_instance
from sim_juncs_gb300.fields import rasterize
from sim_juncs_gb300.spec import Grid, scene_to_c

pytestmark = pytest.mark.gpu


def static_rasterize(lib, torch, grid, scene):
    sc, holder = scene_to_c(scene)
    out = torch.zeros(3 * grid.voxels, dtype=torch.uint8, device="cuda")
    g = grid.to_c()
    stream = torch.cuda.current_stream()
    rc = lib.sj_rasterize_static(C.byref(g), sc, C.c_void_p(out.data_ptr()),
                                 C.c_void_p(stream.cuda_stream))
    _abi.check(lib, rc)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(3, grid.nz, grid.ny, grid.nx)


def test_static_rasterize_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    lib = _abi.load_library()
    a = junction_instance(n=48, res=15.0)
    b = bowtie_instance(nx=96, ny=80, nz=64, res=8.0)
    ga = Grid(48, 48, 48, 1.0 / 15.0)
    first = static_rasterize(lib, torch, ga, a.material)
    second = static_rasterize(lib, torch, b.grid, b.material)
    np.testing.assert_array_equal(first, rasterize(ga, a.material))
    np.testing.assert_array_equal(second, rasterize(b.grid, b.material))
    assert first.any() and (second & 2).any()


def test_static_rasterize_rejects_oversized_program():
    torch = pytest.importorskip("torch")
    lib = _abi.load_library()
    from sim_juncs_gb300.geometry import Box, Union
    from sim_juncs_gb300.spec import Region, Scene
    boxes = [Box((0.1 * q, 0, 0), (0.1 * q + 0.05, 1, 1)) for q in range(_abi.RASTER_STATIC_NODES)]
    scene = Scene([Region(Union(*boxes))])
    g = Grid(8, 8, 8, 0.1)
    sc, holder = scene_to_c(scene)
    out = torch.zeros(3 * g.voxels, dtype=torch.uint8, device="cuda")
    rc = lib.sj_rasterize_static(C.byref(g.to_c()), sc, C.c_void_p(out.data_ptr()), None)
    assert rc == _abi.SJ_E_RANGE
    assert b"SJ_RASTER_STATIC_NODES" in lib.sj_last_error(None)
