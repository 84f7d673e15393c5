"""The C-ABI library loads here (no GPU) and exports every entry point that
include/sj.h declares, with struct layouts matching the ctypes mirror."""
import ctypes as C
import os
import re

import pytest

from sim_juncs_gb300 import _abi

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "sj.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^[A-Za-z_][\w \*]*?\b(sj_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "sj_create" in names and "sj_step" in names and "sj_destroy" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in sj.h but not exported"
        assert name in _abi.SIGNATURES, f"{name} has no ctypes signature"


def test_struct_layouts_match(lib):
    for idx, st in _abi.STRUCTS.items():
        assert lib.sj_abi_struct_size(idx) == C.sizeof(st), st.__name__
    assert lib.sj_abi_struct_size(99) == -1


def test_abi_version(lib):
    text = open(HEADER).read()
    declared = int(re.search(r"#define SJ_ABI_VERSION (\d+)", text).group(1))
    assert lib.sj_abi_version() == declared == _abi.ABI_VERSION


def test_source_helpers_run_on_host(lib):
    from sim_juncs_gb300.spec import Source
    s = Source(_abi.EX, 1.0, 2.0, 0.0, 20.0, (0, 0, 0), (1, 1, 0)).to_c()
    re_, im_ = C.c_double(), C.c_double()
    assert lib.sj_source_dipole(C.byref(s), 10.0, C.byref(re_), C.byref(im_)) == 0
    # at the peak: |d| = 1/omega
    assert abs(complex(re_.value, im_.value)) == pytest.approx(1 / (2 * 3.141592653589793), rel=1e-12)
    assert lib.sj_source_last_time(C.byref(s)) == pytest.approx(20.0)


def test_create_rejects_bad_descriptor_without_gpu_work(lib):
    d = _abi.InstanceDesc()
    d.grid.nx = 0
    h = C.c_void_p()
    rc = lib.sj_create(C.byref(d), 0, C.byref(h))
    assert rc != 0
    assert not h.value
