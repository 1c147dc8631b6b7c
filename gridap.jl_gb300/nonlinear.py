"""Nonlinear FE operators and Newton solvers over libgfe, mirroring Gridap's
FEOperator(res, jac, U, V) (FESpaces/FEOperatorsFromWeakForm.jl), its algebraic operator
(FESpaces/FEOperators.jl:140-200), NewtonRaphsonSolver and NLSolver (Algebra/NLSolvers.jl) and
NonlinearFESolver (FESpaces/FESolvers.jl).

Every Newton step re-assembles the Jacobian into the pattern of the first one
(`jacobian_`: fillstored + the device numeric loop) and the residual into the same vector.
The residual and Jacobian integrands are recognised from expression trees
(celldata.classify_residual / check_jacobian): quasilinear diffusion
`∫ κ ∇v⋅flux(∇u) - f v` with the p-Laplacian flux, or `∫ κ α(u) ∇v⋅∇u - f v` with a
polynomial α, evaluated at the state on the device (GFE_FORM_QUASILINEAR).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .assembly import (SparseMatrixAssembler, _Prepared, _dirichlet_to_problem, _qpoints,
                       symbolic_loop_matrix)
from .celldata import (CellField, PolynomialCoefficient, PowerLawFlux, _FEState,
                       check_jacobian, classify_residual, get_fe_basis, get_trial_fe_basis)
from .fespaces import FEFunction, TrialFESpace, _space
from .solvers import BiCGStabSolver, numerical_setup, numerical_setup_, solve_, symbolic_setup


class FEOperator:
    """FEOperator(res, jac, U, V) or FEOperator(res, U, V): res(u, v) and jac(u, du, v) return
    DomainContributions. Without jac the Jacobian is the exact derivative of the recognised
    law (Gridap differentiates res automatically in that case)."""

    is_nonlinear = True

    def __init__(self, res, *args, assem: SparseMatrixAssembler | None = None):
        if len(args) == 3:
            jac, U, V = args
        elif len(args) == 2:
            jac, (U, V) = None, args
        else:
            raise TypeError("FEOperator(res, jac, U, V) or FEOperator(res, U, V)")
        self.res, self.jac = res, jac
        self.trial, self.test = U, V
        self.assem = assem or SparseMatrixAssembler(U, V)
        Vs = _space(V)
        v = get_fe_basis(V)
        probe = _FEState(None)
        dc = res(probe, v)
        if len(dc.terms) != 1:
            raise NotImplementedError("one residual term (one measure) is provided")
        expr, self.measure = dc.terms[0]
        self.form = classify_residual(expr)
        if jac is not None:
            djc = jac(probe, get_trial_fe_basis(U), v)
            if len(djc.terms) != 1 or djc.terms[0][1].degree != self.measure.degree:
                raise NotImplementedError("residual and Jacobian on one measure are provided")
            check_jacobian(djc.terms[0][0], self.form)
        model = Vs.model
        if Vs.reffe.ncomp != 1 or Vs.reffe.order not in (1, 2):
            raise NotImplementedError("quasilinear forms on scalar Q1/Q2 spaces are provided")
        self._source = None
        self._src_kind = _lib.GFE_SRC_NONE
        if self.form.source is not None:
            s, d = self.form.source
            if callable(d):
                xq = _qpoints(model, self.measure)
                self._source = np.ascontiguousarray(
                    s * np.asarray(d(xq.reshape(-1, model.dim)), np.float64).reshape(-1))
                self._src_kind = _lib.GFE_SRC_QPOINT
            else:
                self._source = np.array([s * float(d)])
                self._src_kind = _lib.GFE_SRC_CONST
        self._coef = None
        if self.form.cells:
            self._coef = np.ascontiguousarray(self.form.scale * np.asarray(
                self.form.cells[0].values, np.float64))
        self._A = None

    def get_trial(self):
        return self.trial

    def get_test(self):
        return self.test

    # -- device calls -----------------------------------------------------------------------
    def _problem(self, x) -> _Prepared:
        V = _space(self.test)
        model = V.model
        prep = _Prepared()
        p = prep.p
        D = model.dim
        p.dim, p.ncomp, p.degree = D, 1, self.measure.degree
        p.reffe = _lib.GFE_REFFE_Q2 if V.reffe.order == 2 else _lib.GFE_REFFE_Q1
        p.ncells = model.num_cells()
        p.nd = V.ndofs_per_cell()
        prep.keep += [V.cell_dof_ids, model.node_coords, model.cell_node_ids]
        p.cell_dof_ids = _lib.ptr(V.cell_dof_ids)
        p.nfree = V.num_free_dofs()
        for d in range(D):
            p.partition[d] = model.partition[d]
            p.domain[2 * d] = model.domain[2 * d]
            p.domain[2 * d + 1] = model.domain[2 * d + 1]
        p.nnodes = model.num_nodes()
        # undistorted Cartesian Q1 cells take the table-driven kernel; coordinates go along
        p.geometry = (_lib.GFE_GEOM_CARTESIAN if model.cartesian and V.reffe.order == 1
                      else _lib.GFE_GEOM_NODAL)
        p.node_coords = _lib.ptr(model.node_coords)
        p.cell_node_ids = _lib.ptr(model.cell_node_ids)
        p.form = _lib.GFE_FORM_QUASILINEAR
        law = self.form.law
        if self._coef is not None:
            p.coef_kind, p.coef = _lib.GFE_COEF_CELL, _lib.ptr(self._coef)
        elif self.form.scale != 1.0:
            k = np.array([self.form.scale])
            prep.keep.append(k)
            p.coef_kind, p.coef = _lib.GFE_COEF_CONST, _lib.ptr(k)
        else:
            p.coef_kind = _lib.GFE_COEF_ONE
        if isinstance(law, PowerLawFlux):
            p.law = _lib.GFE_LAW_POWER
            p.law_params[0], p.law_params[1] = law.p, law.eps2
        elif isinstance(law, PolynomialCoefficient):
            p.law = _lib.GFE_LAW_POLY
            p.law_params[0], p.law_params[1], p.law_params[2] = law.c
        else:
            raise NotImplementedError(f"law {type(law).__name__}")
        if self._source is not None:
            p.source_kind, p.source, p.source_len = (self._src_kind, _lib.ptr(self._source),
                                                     self._source.size)
        if hasattr(x, "free_values"):
            x = x.free_values
        if isinstance(x, np.ndarray):
            x = np.ascontiguousarray(x, np.float64)
        prep.keep.append(x)
        p.state = _lib.ptr(x)
        uD = self.trial.dirichlet_values if isinstance(self.trial, TrialFESpace) else None
        _dirichlet_to_problem(prep, uD)
        return prep

    def _assemble(self, x, A, b):
        prep = self._problem(x)
        ctx = A.ctx if A is not None else self.assem.ctx
        _lib.check(_lib.load().gfe_assemble_matrix_and_vector(
            ctx.handle, C.byref(prep.p), A.handle if A is not None else None,
            _lib.ptr(b) if b is not None else None))

    def allocate_jacobian(self):
        ids = _space(self.test).cell_dof_ids
        return symbolic_loop_matrix(self.assem, (None, ids, ids))

    def residual_(self, b, uh):
        """residual!(b, op, uh): b (host array or CUDA tensor) is overwritten."""
        self._assemble(uh, None, b)
        return b

    def _new_vector(self, like):
        n = _space(self.test).num_free_dofs()
        if hasattr(like, "free_values"):
            like = like.free_values
        return np.empty(n) if isinstance(like, np.ndarray) else like.new_empty((n,))

    def residual(self, uh):
        return self.residual_(self._new_vector(uh), uh)

    def jacobian_(self, A, uh):
        """jacobian!(A, op, uh): re-assembly into A's pattern."""
        A.fillstored_zero()
        self._assemble(uh, A, None)
        return A

    def jacobian(self, uh):
        return self.jacobian_(self.allocate_jacobian(), uh)

    def residual_and_jacobian_(self, b, A, uh):
        A.fillstored_zero()
        self._assemble(uh, A, b)
        return b, A

    def residual_and_jacobian(self, uh):
        return self.residual_and_jacobian_(self._new_vector(uh), self.allocate_jacobian(), uh)

    def get_algebraic_operator(self) -> "AlgebraicOpFromFEOp":
        return AlgebraicOpFromFEOp(self)


class AlgebraicOpFromFEOp:
    """The NonlinearOperator over free values x (FESpaces/FEOperators.jl:140-200)."""

    def __init__(self, feop: FEOperator):
        self.feop = feop

    def residual_(self, b, x):
        return self.feop.residual_(b, x)

    def residual(self, x):
        return self.feop.residual(x)

    def jacobian_(self, A, x):
        return self.feop.jacobian_(A, x)

    def jacobian(self, x):
        return self.feop.jacobian(x)

    def zero_initial_guess(self):
        return np.zeros(_space(self.feop.test).num_free_dofs())

    def allocate_jacobian(self):
        return self.feop.allocate_jacobian()


# ---- Newton solvers ----------------------------------------------------------------------------
def _empty_like(b):
    return np.empty_like(b) if isinstance(b, np.ndarray) else b.new_empty(b.shape)


def _maxabs(b) -> float:
    return float(b.abs().max()) if hasattr(b, "abs") and not isinstance(b, np.ndarray) \
        else float(np.max(np.abs(b))) if len(b) else 0.0


class NewtonRaphsonSolver:
    """NewtonRaphsonSolver(ls, tol, max_nliters) (Algebra/NLSolvers.jl:1-87): converged when
    max|r| < tol at the start, or max|r| < tol * max|r0| after a step; the Jacobian is
    re-assembled in place (jacobian!) and the linear solver re-set-up (numerical_setup!) every
    step."""

    def __init__(self, ls, tol: float, max_nliters: int):
        self.ls, self.tol, self.max_nliters = ls, float(tol), int(max_nliters)
        self.iterations = 0

    def solve_(self, x, op, cache=None):
        if cache is None:
            b = op.residual(x)
            A = op.jacobian(x)
            dx = _empty_like(b)
            ns = numerical_setup(symbolic_setup(self.ls, A), A)
        else:
            A, b, dx, ns = cache
            op.residual_(b, x)
            op.jacobian_(A, x)
            numerical_setup_(ns, A)
        self._solve_nr(x, A, b, dx, ns, op)
        return (A, b, dx, ns)

    def _solve_nr(self, x, A, b, dx, ns, op):
        self.iterations = 0
        m0 = _maxabs(b)
        if m0 < self.tol:
            return
        for it in range(1, self.max_nliters + 1):
            b *= -1
            solve_(dx, ns, b)
            x += dx
            self.iterations = it
            op.residual_(b, x)
            if _maxabs(b) < self.tol * m0:
                return
            if it == self.max_nliters:
                raise RuntimeError(f"NewtonRaphsonSolver failed to converge in {it} iterations. "
                                   f"Final residual: {_maxabs(b)}")
            op.jacobian_(A, x)
            numerical_setup_(ns, A)


class NLSolver:
    """NLSolver(ls; method="newton", ftol, xtol, iterations) (Algebra/NLSolvers.jl:89-170),
    which hands the problem to NLsolve.jl (4.5) — absent here. Its trust-region default is not
    restated; method "newton" is, with the static line search NLsolve uses by default:
    x_{k+1} = x_k - J(x_k)⁻¹ F(x_k), converged when ‖F‖∞ <= ftol (checked at x0 too) or
    ‖x_{k+1} - x_k‖∞ <= xtol, at most `iterations` steps. The default linear solver is
    BiCGStab (Gridap's default is LU)."""

    def __init__(self, ls=None, method: str = "newton", ftol: float = 1e-8, xtol: float = 0.0,
                 iterations: int = 1000, show_trace: bool = False):
        if method != "newton":
            raise NotImplementedError("method='newton' is provided")
        self.ls = ls or BiCGStabSolver(rtol=1e-12)
        self.ftol, self.xtol, self.max_iterations = float(ftol), float(xtol), int(iterations)
        self.show_trace = show_trace
        self.iterations = 0
        self.residual_norm = float("nan")

    def solve_(self, x, op, cache=None):
        if cache is None:
            F = op.residual(x)
            A = op.allocate_jacobian() if hasattr(op, "allocate_jacobian") else op.jacobian(x)
            ns = None
        else:
            A, F, ns = cache
            op.residual_(F, x)
        p = _empty_like(F)
        self.iterations = 0
        fnorm = _maxabs(F)
        converged = fnorm <= self.ftol
        it = 0
        while not converged and it < self.max_iterations and np.isfinite(fnorm):
            it += 1
            op.jacobian_(A, x)
            ns = numerical_setup(symbolic_setup(self.ls, A), A) if ns is None \
                else numerical_setup_(ns, A)
            solve_(p, ns, -F)
            x += p
            op.residual_(F, x)
            fnorm = _maxabs(F)
            xstep = _maxabs(p)
            if self.show_trace:
                print(f"iter {it:4d}  |F|inf {fnorm:.6e}  |dx|inf {xstep:.6e}")
            converged = fnorm <= self.ftol or xstep <= self.xtol
        self.iterations, self.residual_norm = it, fnorm
        if not converged:
            raise RuntimeError(f"Newton solver did not converge after {it} iterations. "
                               f"Final residual norm: {fnorm}")
        return (A, F, ns)


class NonlinearFESolver:
    """NonlinearFESolver(nls) (FESpaces/FESolvers.jl): solves an FEOperator on free values."""

    def __init__(self, nls):
        self.nls = nls


def solve_nonlinear_(uh, solver, op: FEOperator, cache=None):
    """solve!(uh, solver, op[, cache]) -> (uh, cache): uh's free values are the initial guess
    and receive the solution."""
    nls = solver.nls if isinstance(solver, NonlinearFESolver) else solver
    x = uh.free_values
    cache = nls.solve_(x, op.get_algebraic_operator(), cache)
    return uh, cache


def solve_nonlinear(solver, op: FEOperator):
    """solve(nls, op): from a zero initial guess."""
    uh = FEFunction(op.get_trial(), np.zeros(_space(op.get_trial()).num_free_dofs()))
    return solve_nonlinear_(uh, solver, op)[0]
