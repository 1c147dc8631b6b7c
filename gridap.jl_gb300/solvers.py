"""LinearSolver protocol (Algebra/LinearSolvers.jl:58-129,202-209) with GPU CG solvers.

Gridap ships no Krylov solver; a user plugs one in through
symbolic_setup -> numerical_setup -> solve!(x, ns, b). These classes are that plug-in:

  - CGSolver(rtol, maxiter, precond="jacobi"): FP64 preconditioned CG;
  - IRCGSolver(rtol, inner_rtol, ...): FP32 PCG inside FP64 iterative refinement: the outer
    loop forms r = b - A x and updates x in FP64, the inner solves A d = r in FP32;
  - MixedCGSolver(rtol, ...): FP32 PCG with FP64 reliable updates (no restarts);
  - BiCGStabSolver(rtol, ...): FP64 Jacobi-preconditioned BiCGStab (non-symmetric matrices).

Both stop on the FP64 relative residual ||b - A x|| <= rtol ||b|| and report it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .assembly import AffineFEOperator, DeviceMatrix
from .fespaces import FEFunction


class SolveReport:
    def __init__(self, r: _lib.SolveReport):
        self.iterations = r.iterations
        self.refinements = r.refinements
        self.converged = bool(r.converged)
        self.status = r.status
        self.relres = r.relres
        self.operator_format = ("sliced-ELL", "diagonal", "matrix-free lattice")[
            r.operator_format]
        self.ndiag = r.ndiag
        self.fallback = bool(r.fallback)

    def __repr__(self):
        return (f"SolveReport(iterations={self.iterations}, refinements={self.refinements}, "
                f"converged={self.converged}, relres={self.relres:.3e})")


class LinearSolver:
    method = _lib.GFE_SOLVER_CG

    def __init__(self, rtol: float = 1e-8, maxiter: int = 100000, precond: str = "jacobi",
                 inner_rtol: float = 1e-4, check_every: int = 0, initial_guess: bool = False):
        self.rtol = rtol
        self.maxiter = maxiter
        self.precond = {"jacobi": _lib.GFE_PC_JACOBI, "none": _lib.GFE_PC_NONE}[precond]
        self.inner_rtol = inner_rtol
        self.check_every = check_every
        # True: solve!(x, ns, b) starts from the values in x (restart from a saved solution)
        self.initial_guess = initial_guess

    def opts(self) -> _lib.SolverOpts:
        return _lib.SolverOpts(self.method, self.precond, self.rtol, self.maxiter,
                               self.inner_rtol, self.check_every, int(self.initial_guess))


class CGSolver(LinearSolver):
    method = _lib.GFE_SOLVER_CG


class IRCGSolver(LinearSolver):
    method = _lib.GFE_SOLVER_IR_CG


class MixedCGSolver(LinearSolver):
    """FP32 PCG with FP64 reliable updates: x accumulates in FP64 and the FP32 residual is
    replaced by the FP64 true residual b - A x every time it has dropped by `inner_rtol`
    (default 0.01); the search direction is re-orthogonalised and kept."""
    method = _lib.GFE_SOLVER_MIXED_CG

    def __init__(self, rtol: float = 1e-8, maxiter: int = 100000, precond: str = "jacobi",
                 inner_rtol: float = 0.01, check_every: int = 0, initial_guess: bool = False):
        super().__init__(rtol, maxiter, precond, inner_rtol, check_every, initial_guess)


class BiCGStabSolver(LinearSolver):
    """FP64 BiCGStab with a Jacobi (right) preconditioner, for non-symmetric matrices such as
    the Jacobians of quasilinear forms whose coefficient depends on u."""
    method = _lib.GFE_SOLVER_BICGSTAB


class FCGSolver(LinearSolver):
    """Flexible CG with FP32 vectors and FP64 reliable updates, preconditioned by a
    LearnedBlockPreconditioner (`pc`), by a geometric multigrid V-cycle (pc="mg": on the
    lattice operator of uniform Cartesian Q1 in 3-D, or p-multigrid for 3-D Cartesian Q2),
    by the V-cycle with the learned preconditioner as its fine-level smoother (pc=learned,
    multigrid=True) or by Jacobi (pc=None); a stagnating learned preconditioner hands over
    to Jacobi (report.fallback)."""

    def __init__(self, rtol: float = 1e-8, maxiter: int = 100000, pc=None,
                 inner_rtol: float = 0.0, check_every: int = 0, initial_guess: bool = False,
                 multigrid: bool = False):
        # inner_rtol 0: the library's reliable-update threshold (0.1; 1e-4 with multigrid)
        super().__init__(rtol, maxiter, "jacobi", inner_rtol, check_every, initial_guess)
        if isinstance(pc, str):
            if pc != "mg":
                raise ValueError(f"unknown preconditioner {pc!r}")
            self.precond, pc = _lib.GFE_PC_MG, None
        if multigrid:
            if pc is None:
                raise ValueError("multigrid=True takes the learned smoother as pc (or pc=\"mg\")")
            self.precond = _lib.GFE_PC_MG
        self.pc = pc


class SymbolicSetup:
    def __init__(self, solver: LinearSolver):
        self.solver = solver


class NumericalSetup:
    def __init__(self, solver: LinearSolver, A: DeviceMatrix):
        self.solver = solver
        self.A = A
        self.report: SolveReport | None = None


def symbolic_setup(solver: LinearSolver, A: DeviceMatrix) -> SymbolicSetup:
    return SymbolicSetup(solver)


def numerical_setup(ss: SymbolicSetup, A: DeviceMatrix) -> NumericalSetup:
    return NumericalSetup(ss.solver, A)


def numerical_setup_(ns: NumericalSetup, A: DeviceMatrix) -> NumericalSetup:
    ns.A = A
    return ns


def solve_(x, ns: NumericalSetup, b):
    """solve!(x, ns, b): x (numpy or CUDA tensor) receives the solution."""
    rep = _lib.SolveReport()
    o = ns.solver.opts()
    if isinstance(ns.solver, FCGSolver):
        pc = ns.solver.pc.handle if ns.solver.pc is not None else None
        _lib.check(_lib.load().gfe_solve_fcg(ns.A.ctx.handle, ns.A.handle, pc, C.byref(o),
                                             _lib.ptr(b), _lib.ptr(x), C.byref(rep)))
    else:
        _lib.check(_lib.load().gfe_solve(ns.A.ctx.handle, ns.A.handle, C.byref(o), _lib.ptr(b),
                                         _lib.ptr(x), C.byref(rep)))
    ns.report = SolveReport(rep)
    return x


class AffineOperator:
    """AffineOperator(A, b): the algebraic operator x -> A x - b (Algebra/LinearSolvers.jl:8-33)."""

    def __init__(self, A: DeviceMatrix, b):
        self.matrix = A
        self.vector = b

    def get_matrix(self) -> DeviceMatrix:
        return self.matrix

    def get_vector(self):
        return self.vector

    def residual(self, x):
        """A x - b (host arrays)."""
        return self.matrix.matvec(x) - np.asarray(self.vector)


def solve_matrix_(x, ls: LinearSolver, A: DeviceMatrix, b):
    """solve!(x, ls, A, b) (Algebra/LinearSolvers.jl:202-209): one-shot setup and solve."""
    return solve_(x, numerical_setup(symbolic_setup(ls, A), A), b)


class LinearFESolver:
    def __init__(self, ls: LinearSolver | None = None):
        self.ls = ls or CGSolver()


def solve(solver, op, b=None):
    """solve(solver, op) with op an AffineFEOperator returns an FEFunction of the trial space
    (the solver's report attached as `uh.report`); solve(ls, op) with an AffineOperator and
    solve(ls, A, b) with a matrix return the solution vector (Algebra/LinearSolvers.jl)."""
    if getattr(op, "is_nonlinear", False):
        from .nonlinear import solve_nonlinear
        return solve_nonlinear(solver, op)
    ls = solver.ls if isinstance(solver, LinearFESolver) else solver
    if b is not None or isinstance(op, AffineOperator):
        A = op.get_matrix() if isinstance(op, AffineOperator) else op
        rhs = op.get_vector() if isinstance(op, AffineOperator) else b
        x = np.empty_like(rhs) if isinstance(rhs, np.ndarray) else rhs.new_empty(rhs.shape)
        return solve_matrix_(x, ls, A, rhs)
    A, b = op.get_matrix(), op.get_vector()
    x = np.empty_like(b) if isinstance(b, np.ndarray) else b.new_empty(b.shape)
    from .multifield import MultiFieldFESpace, MultiFieldFEFunction
    U = op.get_trial()
    if isinstance(U, MultiFieldFESpace) and U.is_block():
        raise NotImplementedError("solve a block-assembled system through its blocks (or use "
                                  "the consecutive style for one matrix)")
    ns = numerical_setup(symbolic_setup(ls, A), A)
    solve_(x, ns, b)
    uh = MultiFieldFEFunction(U, x) if isinstance(U, MultiFieldFESpace) else FEFunction(U, x)
    uh.report = ns.report
    return uh
