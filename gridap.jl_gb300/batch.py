"""Many independent Q1 diffusion problems assembled and solved in one call (libgfe
`gfe_batch_*`).

Each problem is -div(kappa grad u) = f on the unit cube with an (n, n, n) Cartesian partition,
per-cell kappa (Gridap's cell order), constant f and homogeneous Dirichlet data on the
boundary; the free dofs follow Gridap's CLagrangian numbering of a space with
dirichlet_tags="boundary" (interior nodes in node order). One persistent kernel launch solves
them all: thread-block clusters take the large problems largest first from a work counter and
solve each together, then every CTA takes the small ones alone from a second counter; each
problem runs a Jacobi-PCG, the operator applied matrix-free in FP32 from the cell
coefficients, with FP64 reliable updates whose FP64 true residual decides convergence
(||b - A x|| <= rtol ||b||). Gridap has no batched driver: the per-problem result equals
AffineFEOperator + solve with a Jacobi-preconditioned CG to the same tolerance.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .assembly import default_context


class BatchedPoissonProblems:
    def __init__(self, sizes, kappas, ctx=None):
        lib = _lib.load()
        self.ctx = ctx or default_context()
        self.sizes = [int(n) for n in sizes]
        if len(kappas) != len(self.sizes):
            raise ValueError("one kappa array per problem")
        for n, k in zip(self.sizes, kappas):
            if np.asarray(k).size != n ** 3:
                raise ValueError("kappa of a problem must have n^3 entries")
        parts = np.ascontiguousarray(np.repeat(np.asarray(self.sizes, np.int64), 3))
        kap = np.ascontiguousarray(np.concatenate([np.asarray(k, np.float64).ravel()
                                                   for k in kappas]))
        h = C.c_void_p()
        _lib.check(lib.gfe_batch_create(self.ctx.handle, len(self.sizes), _lib.ptr(parts),
                                        _lib.ptr(kap), C.byref(h)))
        self.handle = h
        self.ctx._own(self)
        nrows, nfree, ncells = C.c_int64(), C.c_int64(), C.c_int64()
        _lib.check(lib.gfe_batch_info(h, C.byref(nrows), C.byref(nfree), C.byref(ncells)))
        self.nrows, self.nfree, self.ncells = nrows.value, nfree.value, ncells.value
        self.offsets = np.concatenate([[0], np.cumsum([(n - 1) ** 3 for n in self.sizes])])
        self.iterations = np.zeros(len(self.sizes), np.int32)
        self.nconverged = 0

    def assemble_solve(self, source=1.0, rtol=1e-8, maxiter=0, x=None):
        """Returns the concatenated free-dof solutions (host array, or fills device `x`)."""
        out = np.empty(self.nfree) if x is None else x
        nconv = C.c_int32()
        _lib.check(_lib.load().gfe_batch_assemble_solve(
            self.handle, float(source), float(rtol), int(maxiter), _lib.ptr(out),
            _lib.ptr(self.iterations), C.byref(nconv)))
        self.nconverged = nconv.value
        return out

    def shape(self):
        """(threads per CTA, CTAs per cluster, cluster threshold) the autotuner chose;
        (0, 0, 0.0) before a solve."""
        t, c, g = C.c_int32(), C.c_int32(), C.c_double()
        _lib.check(_lib.load().gfe_batch_shape(self.handle, C.byref(t), C.byref(c), C.byref(g)))
        return t.value, c.value, round(g.value, 6)

    def set_shape(self, threads, ctas_per_problem, cluster_threshold=0.0):
        """Fixes the schedule (one of the candidates); (0, 0) re-enables autotuning."""
        _lib.check(_lib.load().gfe_batch_set_shape(self.handle, int(threads),
                                                   int(ctas_per_problem),
                                                   float(cluster_threshold)))

    def split(self, x):
        return [x[self.offsets[i]:self.offsets[i + 1]] for i in range(len(self.sizes))]

    def _release(self):
        h, self.handle = self.handle, None
        if h and self.ctx.handle:
            _lib.load().gfe_batch_destroy(h)

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass
