"""GB300-native bonded-DEM Newton solver: a drop-in for the reference's
``bonded_dem_newton`` path (``NewtonBonds`` and its fused binder).

Import as ``dpf_gb300``.  The solver classes need ``libdpf_gb300.so``
(``python dynamic-powerfoam_gb300/build.py``) and a CUDA device; there is no
CPU fallback.
"""
from .foam import jittered_lattice_foam, gravity_load, regular_edges, morton_order
from .newton import (LinearBonds, FiniteBonds, NewtonBonds, FastNewtonBonds, MixedNewtonBonds, AdaptiveIntervals,
                     SubdivideError, fgmres, incidence, guard_error)
from .adjoint import DifferentiableBonds
from .energy import EnergyFoam, EnergyNewton
from .core import ParallelBonds
from .static import reference_stiffness, solve_prescribed

# Reference class names (experiments/bonded_dem_linear_gpu.py, bonded_dem_finite_gpu.py).
LinearBondsGPU = LinearBonds
FiniteBondsGPU = FiniteBonds

__all__ = ['jittered_lattice_foam', 'gravity_load', 'regular_edges', 'morton_order', 'LinearBonds',
           'FiniteBonds', 'NewtonBonds', 'FastNewtonBonds', 'MixedNewtonBonds', 'LinearBondsGPU', 'FiniteBondsGPU',
           'AdaptiveIntervals', 'SubdivideError', 'fgmres', 'incidence', 'guard_error', 'DifferentiableBonds',
           'EnergyFoam', 'EnergyNewton', 'ParallelBonds', 'reference_stiffness', 'solve_prescribed']
