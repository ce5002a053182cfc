"""parafem_gb300 -- GB300-native element-by-element PCG solves of ParaFEM's
p121 (3-D elasticity, 20-node bricks), p122 (Mohr-Coulomb viscoplasticity,
20-node bricks) and p123 (3-D Laplace, 8-node bricks).

The compute path is libpfgpu.so (hand-written sm_103a kernels behind a C-ABI,
include/pfgpu.h); this package builds it in-tree and binds it with ctypes.
"""
from .pfgpu import (Batch, MODE_MIXED, MODE_MIXED16, MODE_MIXED_RESTART, MODE_FP64_RES, MODE_P121, PfError, Solver, box8_problem,
                    box8_restraints, cube_problem, cube_restraints, cube_top_pressure, last_error, lib, library_path,
                    mesh_box8, mesh_cube, number_equations, number_equations1, p121_run, p122_run, p123_run, p12meshgen,
                    patch_loads,
                    random_material, random_top_loads, top_face_z_equations)

__all__ = ["Batch", "MODE_MIXED", "MODE_MIXED16", "MODE_MIXED_RESTART", "MODE_FP64_RES", "MODE_P121", "PfError", "Solver",
           "box8_problem", "box8_restraints", "cube_problem", "cube_restraints", "cube_top_pressure", "last_error",
           "lib", "library_path", "mesh_box8", "mesh_cube", "number_equations", "number_equations1", "p121_run",
           "p122_run", "p123_run", "p12meshgen", "patch_loads", "random_material", "random_top_loads", "top_face_z_equations"]
