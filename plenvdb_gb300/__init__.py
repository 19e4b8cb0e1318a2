"""plenvdb_gb300 — GB300-native (sm_103a) implementation of PlenVDB's
differentiable sparse-grid ray-marching path behind the reference's
``plenvdb`` plugin API (DensityVDB, ColorVDB, DensityOpt, ColorOpt,
MGRenderer).

The compute lives in libpvdb.so (CUDA, C ABI in include/pvdb.h); this package
is the host-side mirror of the reference interface.
"""
from . import _lib  # noqa: F401
from .plenvdb import ColorOpt, ColorVDB, DensityOpt, DensityVDB  # noqa: F401

__all__ = ["DensityVDB", "ColorVDB", "DensityOpt", "ColorOpt", "MGRenderer"]


def __getattr__(name):
    if name == "MGRenderer":
        from .renderer import MGRenderer
        return MGRenderer
    raise AttributeError(name)
