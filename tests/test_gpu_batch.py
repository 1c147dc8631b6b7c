"""GPU tests of the batched problems path (`gfe_batch_*`): many independent Q1 diffusion
problems assembled and solved in one call.

Each problem's solution is compared with the oracle's assembly of the same problem (Gridap's
CLagrangian numbering, FP64 cell integrals, InserterCSC assembly) solved by the oracle's
Jacobi-PCG to the same rtol. The batched solver iterates in FP32 between FP64 reliable
updates, so its iteration counts track the FP64 ones within a few iterations (tolerance below:
15 % + 2), its FP64 true residual meets rtol against the oracle's matrix, and the solutions
agree within the CG tolerance (1e-10 relative residual -> 1e-7 relative solutions after the
conditioning of these small problems).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# the autotuner's candidate schedules: threads per CTA, CTAs per cluster, cluster threshold
SCHEDULES = {(256, 1, 0.0), (1024, 1, 0.0), (1024, 2, 0.0), (512, 4, 0.0), (512, 4, 0.3),
             (1024, 4, 0.3), (1024, 8, 0.0), (1024, 8, 0.3)}


def _oracle_problem(orc, n, kappa, f):
    P = orc.poisson_q1((0.0, 1.0) * 3, (n, n, n), kappa=kappa, fkind=orc.F_CONST,
                       fdata=np.array([f]))
    return P


def test_batch_matches_oracle_per_problem(gg, orc):
    rng = np.random.default_rng(11)
    sizes = [2, 3, 5, 8, 4, 9, 6, 12, 7, 3]
    kappas = [np.exp(rng.standard_normal(n ** 3)) for n in sizes]
    B = gg.BatchedPoissonProblems(sizes, kappas)
    assert B.nfree == sum((n - 1) ** 3 for n in sizes)
    assert B.nrows == B.nfree
    x = B.assemble_solve(source=2.5, rtol=1e-10)
    assert B.nconverged == len(sizes)
    for i, (n, k, xi) in enumerate(zip(sizes, kappas, B.split(x))):
        P = _oracle_problem(orc, n, k, 2.5)
        colptr, rowval, nzval = P["csc"]
        xr, it, relres = orc.pcg(colptr, rowval, nzval, P["b"], 1e-10)
        assert abs(int(B.iterations[i]) - it) <= 2 + 0.15 * it, (n, B.iterations[i], it)
        A = orc.to_scipy(colptr, rowval, nzval, P["nfree"], P["nfree"])
        rel = np.linalg.norm(P["b"] - A @ xi) / np.linalg.norm(P["b"])
        assert rel <= 1.01e-10, (n, rel)
        assert np.linalg.norm(xi - xr) <= 1e-7 * np.linalg.norm(xr), n


def test_batch_repeated_solves_are_identical(gg):
    rng = np.random.default_rng(12)
    sizes = [16] * 40 + [10] * 24
    kappas = [np.exp(rng.standard_normal(n ** 3)) for n in sizes]
    B = gg.BatchedPoissonProblems(sizes, kappas)
    x1 = B.assemble_solve(source=1.0, rtol=1e-8)
    it1 = B.iterations.copy()
    x2 = B.assemble_solve(source=1.0, rtol=1e-8)
    assert np.array_equal(x1, x2) and np.array_equal(it1, B.iterations)
    # the same problem posed twice in one batch gives the same answer both times
    a, b = B.split(x1)[0], B.split(x1)[1]
    assert not np.array_equal(a, b)  # different kappa
    B2 = gg.BatchedPoissonProblems([16, 16], [kappas[0], kappas[0]])
    y = B2.assemble_solve(source=1.0, rtol=1e-8)
    y0, y1 = B2.split(y)
    assert np.array_equal(y0, y1)
    # another batch may pick another launch shape (summation order): CG-tolerance agreement
    assert np.linalg.norm(y0 - a) <= 1e-6 * np.linalg.norm(a)


def test_batch_matches_single_problem_cg(gg):
    """Against the library's own single-problem path (AffineFEOperator + CG with Jacobi)."""
    rng = np.random.default_rng(13)
    n = 10
    kappa = np.exp(rng.standard_normal(n ** 3))
    B = gg.BatchedPoissonProblems([n, n - 3], [kappa, np.ones((n - 3) ** 3)])
    xb = B.split(B.assemble_solve(source=1.0, rtol=1e-10))[0]
    m = gg.CartesianDiscreteModel((0, 1) * 3, (n, n, n))
    V = gg.FESpace(m, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    dO = gg.Measure(gg.Triangulation(m), 2)
    kap = gg.CellField(kappa)
    A, b = gg.assemble_matrix_and_vector(
        lambda u, v: gg.integrate(kap * gg.inner(gg.grad(v), gg.grad(u)), dO),
        lambda v: gg.integrate(1.0 * v, dO), V, V)
    x = np.empty_like(b)
    ns = gg.numerical_setup(gg.symbolic_setup(gg.CGSolver(rtol=1e-10), A), A)
    gg.solve_(x, ns, b)
    it = ns.report.iterations
    assert abs(it - int(B.iterations[0])) <= 2 + 0.15 * it
    assert np.linalg.norm(xb - x) <= 1e-7 * np.linalg.norm(x)


def test_batch_rejects_non_cubic_partitions(gg):
    lib = gg._lib.load()
    import ctypes as C
    parts = np.array([4, 4, 5], np.int64)
    kap = np.ones(80)
    h = C.c_void_p()
    st = lib.gfe_batch_create(gg.default_context().handle, 1, gg._lib.ptr(parts),
                              gg._lib.ptr(kap), C.byref(h))
    assert st == gg._lib.GFE_ERR_UNSUPPORTED


def test_batch_one_launch_autotuned_shape_device_output(gg):
    """One kernel launch per solve after tuning, a tuned shape among the candidates, and the
    device-resident output equal to the host-output solve."""
    import torch
    rng = np.random.default_rng(14)
    sizes = [int(n) for n in rng.integers(4, 20, 48)]
    kappas = [np.exp(1.5 * rng.standard_normal(n ** 3)) for n in sizes]
    ctx = gg.default_context()
    B = gg.BatchedPoissonProblems(sizes, kappas, ctx)
    assert B.shape() == (0, 0, 0.0)
    xh = B.assemble_solve(source=1.0, rtol=1e-8)
    assert B.shape() in SCHEDULES
    xd = torch.empty(B.nfree, dtype=torch.float64, device="cuda")
    l0 = ctx.kernel_launches()
    B.assemble_solve(source=1.0, rtol=1e-8, x=xd)
    assert ctx.kernel_launches() - l0 == 1
    assert np.array_equal(xd.cpu().numpy(), xh)
    assert B.nconverged == len(sizes)


def test_batch_iteration_cap_reports_unconverged(gg):
    rng = np.random.default_rng(15)
    sizes = [12, 3, 9]
    kappas = [np.exp(2.0 * rng.standard_normal(n ** 3)) for n in sizes]
    B = gg.BatchedPoissonProblems(sizes, kappas)
    B.assemble_solve(source=1.0, rtol=1e-12, maxiter=3)
    assert B.nconverged < len(sizes)
    assert int(B.iterations.max()) <= 3
    # the 2^3-node problem (one free dof) converges in one iteration
    assert int(B.iterations[1]) <= 3


def test_batch_zero_source_and_single_cell(gg):
    """f = 0 gives x = 0 without iterating; n = 1 has no free dof."""
    B = gg.BatchedPoissonProblems([1, 5], [np.ones(1), np.ones(125)])
    x = B.assemble_solve(source=0.0, rtol=1e-8)
    assert x.shape == (64,) and np.all(x == 0.0)
    assert B.nconverged == 2 and int(B.iterations.max()) == 0


def test_batch_every_shape_agrees(gg):
    """Each candidate schedule (fixed by set_shape) converges every problem to rtol; the
    solutions agree within the CG tolerance."""
    rng = np.random.default_rng(16)
    sizes = [int(n) for n in rng.integers(3, 26, 20)]
    kappas = [np.exp(1.5 * rng.standard_normal(n ** 3)) for n in sizes]
    B = gg.BatchedPoissonProblems(sizes, kappas)
    ref = None
    for shape in sorted(SCHEDULES):
        try:
            B.set_shape(*shape)
        except gg._lib.GfeError:
            continue  # a cluster shape this device cannot co-schedule
        x = B.assemble_solve(source=1.0, rtol=1e-9)
        assert B.nconverged == len(sizes) and B.shape() == shape
        if ref is None:
            ref = x
        else:
            for a, b in zip(B.split(x), B.split(ref)):
                assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(b)
    assert ref is not None
