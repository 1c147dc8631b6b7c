"""Parity with the oracle at the benchmark configurations' own sizes, through the public API.

Sizes (stated here, as the oracle's cost sets them):
  - 256^2 Q1 Poisson with the sinusoid-sum source (65,025 free dofs): the whole configuration;
  - 128^3 Q1 lognormal diffusion (2,048,383 free dofs, nnz 54,439,939): the whole
    configuration, assembled by the closed-form Cartesian pattern and the fused row gather,
    solved by the multigrid-preconditioned mixed-precision FCG;
  - 64^3 jittered Q2 Poisson (2,048,383 free dofs, nnz 127,263,527): the whole configuration,
    FP64 cells and tensor-core cells (FP16 operands with TF32's 11 significant bits);
  - simplexify(24^3) vector P2 elasticity (345,744 free dofs): the oracle restates Gridap's
    per-point steps and needs about half a minute here; the 48^3 configuration runs the same
    kernels on a larger grid (the benchmark compares it at full size).

Tolerances:
  - CSR pattern: bit-exact (the oracle's CSC arrays are the CSR arrays of these symmetric
    matrices);
  - FP64 matrix values: |a - a_ref| <= 1e-12 * max |row of a_ref|; vectors: 1e-12 * max |b_ref|;
  - tensor-core Q2 cells: 2e-3 of the row maximum (matrix) and of max |b_ref| (vector);
  - solutions: the FP64 relative residual of the device solution in the oracle's own system
    <= rtol (1 + 1e-3), and the distance to the oracle's solution <= 1e3 * rtol relative.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_VAL = 1e-12


def _rowscaled(cp, zv, nz):
    lens = np.diff(cp)
    rowmax = np.maximum.reduceat(np.abs(zv), cp[:-1] - 1)
    return float(np.max(np.abs(nz - zv) / np.repeat(np.maximum(rowmax, 1e-300), lens)))


def _check_system(A, b, ref, tol=TOL_VAL):
    rp, cv, nz = A.export_csr(1)
    cp, rv, zv = ref["csc"]
    assert np.array_equal(rp, cp), "row pointers differ from the oracle"
    assert np.array_equal(cv, rv), "column ids differ from the oracle"
    assert _rowscaled(cp, zv, nz) <= tol
    if b is not None:  # TF32 cells carry FP32 cell vectors: the same tolerance as the matrix
        assert np.abs(b - ref["b"]).max() <= tol * np.abs(ref["b"]).max()


def _relres_in(orc, ref, x):
    r = ref["b"] - orc.csc_mul(*ref["csc"], x)
    return np.linalg.norm(r) / np.linalg.norm(ref["b"])


def test_poisson_2d_256_full_size(gg, orc):
    from gridap_gb300 import workloads
    w = workloads.poisson_2d(256)
    V = w.space
    U = gg.TrialFESpace(V)
    dO = w.measure
    op = gg.AffineFEOperator(lambda u, v: gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dO),
                             lambda v: gg.integrate(w.source * v, dO), U, V)
    ref = orc.poisson_q1((0, 1, 0, 1), (256, 256), ("boundary",), f_callable=w.source)
    assert V.num_free_dofs() == ref["nfree"] == 65025
    _check_system(op.A, op.b, ref)
    uh = gg.solve(gg.LinearFESolver(gg.CGSolver(rtol=w.rtol)), op)
    assert uh.report.converged
    x = np.asarray(uh.free_values)
    assert _relres_in(orc, ref, x) <= w.rtol * (1 + 1e-3)
    xr, _, _ = orc.pcg(*ref["csc"], ref["b"], w.rtol)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) <= 1e3 * w.rtol


def test_lognormal_128_full_size(gg, orc):
    from gridap_gb300 import workloads
    w = workloads.lognormal_3d(128)
    V = w.space
    U = gg.TrialFESpace(V)
    dO = w.measure
    kap, f = gg.CellField(w.kappa), w.source
    op = gg.AffineFEOperator(
        lambda u, v: gg.integrate(kap * gg.inner(gg.grad(v), gg.grad(u)), dO),
        lambda v: gg.integrate(f * v, dO), U, V)
    with orc.cell_threads(os.cpu_count() or 1):
        ref = orc.poisson_q1((0, 1, 0, 1, 0, 1), (128, 128, 128), ("boundary",), kappa=w.kappa,
                             fkind=orc.F_NODAL, fdata=f.values)
    assert ref["nfree"] == 2048383 and ref["csc"][2].shape[0] == 54439939
    _check_system(op.A, op.b, ref)
    uh = gg.solve(gg.LinearFESolver(gg.FCGSolver(rtol=w.rtol, pc="mg")), op)
    assert uh.report.converged
    x = np.asarray(uh.free_values)
    assert _relres_in(orc, ref, x) <= w.rtol * (1 + 1e-3)
    xr, _, rr = orc.pcg(*ref["csc"], ref["b"], w.rtol, nthreads=os.cpu_count() or 1)
    assert rr <= w.rtol
    # two solutions that each meet 1e-8: their distance is bounded by cond(A) * 1e-8
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) <= 1e-4


@pytest.mark.parametrize("precision,tol", [("fp64", TOL_VAL), ("fp32", 2e-3)])
def test_jittered_q2_64_full_size(gg, orc, precision, tol):
    from gridap_gb300 import synthetic, workloads
    model, V, dO = workloads.jittered_q2_3d(64)
    U = gg.TrialFESpace(V)
    assem = gg.SparseMatrixAssembler(U, V, precision=precision)
    op = gg.AffineFEOperator(lambda u, v: gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dO),
                             lambda v: gg.integrate(1.0 * v, dO), U, V, assem)
    with orc.cell_threads(os.cpu_count() or 1):
        ref = orc.poisson_q2((0, 1, 0, 1, 0, 1), (64, 64, 64), ("boundary",), kappa=None,
                             fconst=1.0, degree=4, jitter=synthetic.q2_jitter(64))
    del ref["cellmats"]
    assert ref["nfree"] == 2048383
    _check_system(op.A, op.b, ref, tol)
    if precision == "fp64":
        uh = gg.solve(gg.LinearFESolver(gg.MixedCGSolver(rtol=1e-8)), op)
        assert uh.report.converged
        assert _relres_in(orc, ref, np.asarray(uh.free_values)) <= 1e-8 * (1 + 1e-3)


def test_elasticity_p2_24(gg, orc):
    from gridap_gb300 import workloads
    n = 24
    model, V, dO, lame, force = workloads.elasticity_3d(n)
    U = gg.TrialFESpace(V)
    sigma = gg.isotropic_stress(gg.CellField(lame[:, 0]), gg.CellField(lame[:, 1]))
    op = gg.AffineFEOperator(lambda u, v: gg.integrate(gg.inner(gg.ε(v), sigma(gg.ε(u))), dO),
                             lambda v: gg.integrate(gg.inner(tuple(force), v), dO), U, V)
    with orc.cell_threads(os.cpu_count() or 1):
        ref = orc.elasticity_p2((0, 1, 0, 1, 0, 1), (n, n, n), lame)
    assert np.array_equal(ref["cell_dofs"], V.cell_dof_ids)
    assert V.num_free_dofs() == ref["nfree"] == 345744
    _check_system(op.A, op.b, ref)
    uh = gg.solve(gg.LinearFESolver(gg.FCGSolver(rtol=1e-8)), op)
    assert uh.report.converged
    assert _relres_in(orc, ref, np.asarray(uh.free_values)) <= 1e-8 * (1 + 1e-3)
