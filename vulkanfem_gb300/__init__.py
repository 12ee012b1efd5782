"""vulkanfem_gb300 -- GB300-native matrix-free voxel elasticity MG-PCG.

The solver itself is the C-ABI CUDA library ``libvfem.so`` (``csrc/``, declared
in ``include/vfem.h``); this package builds it in-tree and mirrors the
reference's solve-path interface on top of it (``api``), plus the seeded
synthetic domains (``domains``) and the reference's ``.dat`` readers and
writers (``inout``; ``python -m vulkanfem_gb300 <model>.dat`` is the reference's
command-line driver).
"""
from .api import (  # noqa: F401
    MatrixFreeSparse, MultigridPreconditioner, VfemError, applyBoundaryConditions, assembleSystemMatrix,
    assemble_system_matrix, hex8_stiffness, kernel_launch_count, load_library, make_options, solve,
    solveWithKompute,
)
from . import domains  # noqa: F401
