"""parafem_gb300 -- GB300-native element-by-element PCG solve of ParaFEM's p121.

The compute path is libpfgpu.so (hand-written sm_103a kernels behind a C-ABI,
include/pfgpu.h); this package builds it in-tree and binds it with ctypes.
"""
from .pfgpu import (Batch, MODE_MIXED, MODE_MIXED_RESTART, MODE_FP64_RES, MODE_P121, PfError, Solver, cube_problem,
                    cube_restraints, cube_top_pressure, last_error, lib, library_path, mesh_cube,
                    number_equations, p121_run, p12meshgen, random_material, random_top_loads,
                    top_face_z_equations)

__all__ = ["Batch", "MODE_MIXED", "MODE_MIXED_RESTART", "MODE_FP64_RES", "MODE_P121", "PfError", "Solver", "cube_problem",
           "cube_restraints", "cube_top_pressure", "last_error", "lib", "library_path", "mesh_cube",
           "number_equations", "p121_run", "p12meshgen", "random_material", "random_top_loads",
           "top_face_z_equations"]
