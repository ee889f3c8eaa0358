"""GB300-native FoilCFD solver step: D3Q19 TRT + Smagorinsky stream-collide,
iMEM wall model, 2:1 refinement coupling and momentum-exchange forces as
hand-written sm_103a CUDA kernels behind a C ABI (include/foilcfd_step.h)."""
from .solver import (FLAG, Box, LBMSolver, SolverError, boundary_flags, build_wall_list, close_trailing_edge_gaps,
                     compute_scaling, derive_patch_box, fine_anchor, fine_dims_for, force_to_coefficient,
                     layout_anchor, naca4, refined_scaling, scaling_direct, scaling_for_nu, stamp_interface_shell,
                     voxelize_airfoil)

__all__ = ["FLAG", "Box", "LBMSolver", "SolverError", "boundary_flags", "build_wall_list",
           "close_trailing_edge_gaps", "compute_scaling", "derive_patch_box", "fine_anchor", "fine_dims_for",
           "force_to_coefficient", "layout_anchor", "naca4", "refined_scaling", "scaling_direct", "scaling_for_nu",
           "stamp_interface_shell", "voxelize_airfoil"]
