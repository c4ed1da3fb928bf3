"""beastgpu -- GB300 (sm_103a) Galerkin BEM assembly and dense solve with BEAST.jl's API.

The compute lives in libbeastgpu.so (C ABI, include/beastgpu.h); this package is the host
mirror of the reference's interface: meshes, spaces, operators, quadrature strategies,
`assemble`, `solve`, `gmres` and far-field post-processing.
"""
from . import lib
from .lib import FP64, MIXED, MIXED_ACCURATE, MIXED_BALANCED, C128, C64, BeastError
from .mesh import Mesh, readmesh, icosphere, ellipsoid, refines
from .spaces import raviartthomas, lagrangecxd0, lagrangec0d1, P0, P1, RT
from .operators import (Maxwell3D, Helmholtz3D, nxdoublelayer, Identity, NCross,
                        DoubleNumWiltonSauterQStrat, DoubleNumSauterQstrat, DoubleNumQStrat,
                        TestRefinesTrialQStrat, TrialRefinesTestQStrat, defaultquadstrat, tangential_trace, cross_trace_H, dirichlet_trace)
from .api import (Context, get_context, assemble, assemble_rhs, solve, gmres, farfield,
                  solve_job, blockassembler, assemblerow, assemblecol)
from .serve import Server, run_job, job_footprint
from .batch import Batch
from .refine import barycentric_refinement, buffachristiansen, refined
from . import tune

__all__ = [n for n in dir() if not n.startswith("_")]
