"""GB300-native (sm_103a) MPM step with the capabilities of the HybridSolver step of
2iw31Zhv/AnisotropicElastoplasticity: APIC transfers with cubic B-spline weights,
fixed-corotated snow, Drucker-Prager sand, level-set collision with friction.

The compute path is libaep.so (CUDA kernels behind the C-ABI of include/aep.h);
this package is its host-side binding and the reference-shaped classes.
"""
from . import capi, scenes
from .capi import AepError
from .solver import HybridSolver, LagrangianMesh, LevelSet, ParticleSystem, RegularGrid, make_params

__all__ = ["capi", "scenes", "AepError", "HybridSolver", "LagrangianMesh", "LevelSet", "ParticleSystem",
           "RegularGrid", "make_params"]
