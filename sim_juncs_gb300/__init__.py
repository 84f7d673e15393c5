"""sim_juncs_gb300: a GB300-native FDTD stepper standing in for the
meep::fields::step() loop of rachel-stromswold/sim_juncs.

The CUDA library (libsj_gb300.so, C ABI in include/sj.h) does all stepping;
this package builds the descriptors and reads results back.  There is no
CPU fallback: importing ``Fields`` without the built library raises.
"""
from . import _abi
from .spec import (PML, ClassMaterial, Grid, Instance, Probe, Region, Scene, Source,
                   Susceptibility)
from .geometry import Box, Cylinder, Difference, Intersect, Plane, Sphere, Union

__all__ = ["_abi", "PML", "ClassMaterial", "Grid", "Instance", "Probe", "Region", "Scene",
           "Source", "Susceptibility", "Box", "Cylinder", "Difference", "Intersect", "Plane",
           "Sphere", "Union", "Fields"]


def __getattr__(name):
    if name == "Fields":
        from .fields import Fields
        return Fields
    raise AttributeError(name)
