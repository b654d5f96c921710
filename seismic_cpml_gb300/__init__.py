"""GB300-native staggered-grid velocity-stress elastic solver with C-PML.

A drop-in for seismic_CPML_2D_isotropic_second_order.f90 and
seismic_CPML_3D_isotropic_MPI_OpenMP.f90: the reference's parameter block
becomes ``CpmlParams``, its time loop runs as CUDA kernels for sm_103a behind
the C ABI of include/cpml.h (libcpml.so), and its output files are written by
the same library.
"""
from .params import (CpmlParams, default_2d, default_3d, config_2d_plain, config_3d_plain,
                     reference_receivers_2d, FIELDS, STF_DGAUSSIAN, STF_GAUSSIAN, STF_RICKER,
                     FLAG_ENERGY, FLAG_EP_PHYSICAL, FLAG_NO_STABILITY)

__all__ = ["CpmlParams", "default_2d", "default_3d", "config_2d_plain", "config_3d_plain",
           "reference_receivers_2d", "FIELDS", "STF_DGAUSSIAN", "STF_GAUSSIAN", "STF_RICKER",
           "FLAG_ENERGY", "FLAG_EP_PHYSICAL", "FLAG_NO_STABILITY", "Solver", "build"]


def __getattr__(name):
    if name == "Solver":
        from .solver import Solver
        return Solver
    if name == "build":
        from .build import build
        return build
    raise AttributeError(name)
