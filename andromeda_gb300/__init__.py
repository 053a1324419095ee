"""GB300-native BEM hot path of Andromeda: Laplace/Stokes influence-matrix
assembly and LSQR solve as hand-written sm_103a CUDA kernels behind a C ABI
(include/andromeda_gb300.h)."""
from . import mesh  # noqa: F401
from ._lib import AgbError, LIB_PATH, load  # noqa: F401
from .api import (BC_CONTACT, BC_FLUX, BC_FUNCTION, ERR_ARG, ERR_CUDA, ERR_NUMERIC, ERR_STATE,  # noqa: F401
                  ERR_UNSUPPORTED, FP64, OK, LAPLACE, MATRIX_FREE, MIXED, SOLVER_BICGSTAB,  # noqa: F401
                  SOLVER_GMRES, SOLVER_HYBRID, SOLVER_LSQR, SOLVER_LSQR_BLOCK, STOKES, Context, batch_resistance, dirichlet_known, form_pre_fm, lsqr_precon, lsqr_solve, solv_eqn_fm,
                  version)
