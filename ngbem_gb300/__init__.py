"""ngbem_gb300: GB300-native boundary-element operator assembly and H-matrix application.

Drop-in for ngbem's operator path: the factory functions below keep the reference names
and keywords (reference src/python_bem.cpp).  Assembly and application run as hand-written
CUDA kernels for sm_103a behind the C-ABI of include/ngbem_gb300.h.
"""
from .meshes import Mesh, Region, icosphere, ellipsoid, perturbed_icosphere
from .bem import *  # noqa: F401,F403
from .bem import __all__ as _bem_all
from .krylov import BlockMatrix, BlockVector

__all__ = ["Mesh", "Region", "icosphere", "ellipsoid", "perturbed_icosphere", "BlockMatrix",
           "BlockVector"] + list(_bem_all)
