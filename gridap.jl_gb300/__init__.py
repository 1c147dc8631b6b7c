"""gridap_gb300 -- GB300-native finite-element assembly and linear solve behind Gridap.jl's
API (assemble_matrix/assemble_vector, SparseMatrixAssembler, AffineFEOperator, LinearSolver).

All numerical work runs in libgfe (hand-written sm_103a CUDA, C ABI in include/gfe.h); this
package is the host-side mirror of Gridap's interface for Python callers. There is no CPU
fallback: importing works without a GPU, but every assembly or solve needs libgfe and a GPU.

The directory name is not a Python identifier; load it with `load_package()` from
`__graft_entry__` or add the repository root to sys.path and import `gridap_gb300` via
`importlib` (see `__graft_entry__.load_package`).
"""
from . import _lib
from ._lib import GfeError
from .assembly import (AffineFEOperator, Context, DeviceMatrix, SparseMatrixAssembler,
                       assemble_matrix, assemble_matrix_, assemble_matrix_and_vector,
                       assemble_matrix_and_vector_, assemble_vector, assemble_vector_,
                       default_context, numeric_loop_matrix, numeric_loop_vector,
                       prepare_problem, symbolic_loop_matrix)
from .celldata import (CellField, DomainContribution, NodalField, SinSum, div, divergence, dot,
                       get_fe_basis, get_normal_vector, get_trial_fe_basis, grad, gradient,
                       inner, integrate, isotropic_stress, PolynomialCoefficient, PowerLawFlux,
                       symmetric_gradient, ε)
from .fespaces import (FEFunction, FESpace, ReferenceFE, TrialFESpace, get_cell_dof_ids,
                       lagrangian, num_free_dofs)
from .geometry import (Boundary, BoundaryTriangulation, CartesianDiscreteModel, FaceLabeling,
                       Measure, SimplexDiscreteModel, Triangulation, simplexify)
from .batch import BatchedPoissonProblems
from .multifield import (BlockDeviceMatrix, BlockMultiFieldStyle, ConsecutiveMultiFieldStyle,
                         MultiFieldFEFunction, MultiFieldFESpace, compute_field_offsets,
                         num_fields)
from .reindexing import compute_dof_permutation, reindex_free_dof_ids
from .nonlinear import (FEOperator, NewtonRaphsonSolver, NLSolver, NonlinearFESolver,
                        solve_nonlinear_)
from .learned import LearnedBlockPreconditioner
from .solvers import (AffineOperator, BiCGStabSolver, CGSolver, FCGSolver, IRCGSolver,
                      LinearFESolver,
                      LinearSolver, MixedCGSolver, solve_matrix_,
                      SolveReport, solve,
                      solve_, numerical_setup, numerical_setup_, symbolic_setup)

__all__ = [n for n in dir() if not n.startswith("_")]
