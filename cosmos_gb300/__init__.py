"""cosmos_gb300: GB300 (sm_103a) implementation of the Cosmos SLIC/FORCE finite-volume path.

The compute path is libcosmos_gb300.so (hand-written CUDA kernels behind the C ABI in
include/cosmos_gb300.h).  This package provides the Python host side: a ctypes binding
(``_lib``), device grids (``Grid``) and reference-named solver classes (``solvers``).
"""
from ._lib import (BC_PERIODIC, BC_TRANSMISSIVE, FP32, FP64, GR, MINBEE, NEWTONIAN, SR, SUPERBEE, VANLEER,  # noqa
                   CosmosError, load)
from .solvers import (BlackHoleEulerFirstOrderSolver, BlackHoleEulerForcingSolver,  # noqa: F401
                      BlackHoleEulerSecondOrderSolver, BlackHoleEulerSolvers, BlackHoleSpacetime, Context,
                      EulerFirstOrderSolver, EulerMaterialParameters, EulerSecondOrderSolver, EulerSolvers, Grid,
                      RelativisticEulerFirstOrderSolver, RelativisticEulerSecondOrderSolver, RelativisticEulerSolvers,
                      default_context, set_tensor_maps, solve_with_steps)
from .solvers import (AMR, Batch, EulerAMR, EulerEquationOfState, RelativisticEulerAMR,  # noqa: F401
                      RelativisticEulerEquationOfState, SlopeLimiters, interface_eval, state_eval)

__all__ = [n for n in dir() if not n.startswith("_")]
