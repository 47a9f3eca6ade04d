"""pypde_gb300: the pypde spectral-Galerkin time-step path on GB300 (sm_103a), FP64.

Mirrors pypde's public names (``from pypde import *``) on float64 CUDA tensors:
bases, fields, field operations, solver plans and templates.  Every transform
and solve runs in the hand-written kernels of libpypde_gb300.so (C ABI in
include/pgx.h); there is no CPU fallback.
"""
from .bases import Base, MetaBase, Chebyshev, GalerkinChebyshev, ChebDirichlet, ChebNeumann, DirichletC, NeumannC
from .spectralspace import SpectralSpace, SpectralSpaceBC
from .field import Field, FieldBC, MultiField, zero_pad, zero_unpad
from .field_operations import (grad, cheby_to_galerkin, galerkin_to_cheby, conv_term, convective_term, avg_x,
                               avg_vol, interpolate)
from .solver import (Flags, MetaPlan, MatrixBase, PlanRHS, PlanLHS, Plan_numpy, Plan_twodma, Plan_fdma,
                     Plan_Poisson, SolverPlan, Integrator)
from .templates import (solverplan_hholtz1d, solverplan_hholtz2d_adi, solverplan_hholtz2d_fd, solverplan_poisson1d,
                        solverplan_poisson2d)
from ._lib import PgxError

__version__ = "0.1.0"
