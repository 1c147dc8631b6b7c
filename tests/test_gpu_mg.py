"""Geometric multigrid on the lattice operator as the preconditioner of the flexible CG
(FCGSolver(pc="mg")): every solve must meet the FP64 relative residual (the report's relres
is b - A x in FP64) and agree with the FP64 Jacobi-CG solution to the solver tolerance; the
V-cycle must cut the iteration count far below Jacobi's on rough coefficients; odd cell
counts (fewer levels, down to smoothing only) still converge; a matrix without the lattice
form is refused.
"""
import numpy as np
import pytest

from test_gpu_q1 import _problem

pytestmark = pytest.mark.gpu


def _solve(gg, A, b, solver):
    x = np.empty_like(b)
    ns = gg.numerical_setup(gg.symbolic_setup(solver, A), A)
    gg.solve_(x, ns, b)
    return x, ns.report


@pytest.mark.parametrize("part,sigma", [((32, 32, 32), 1.5), ((48, 40, 32), 2.5),
                                        ((30, 28, 26), 1.0), ((21, 18, 16), 1.0)])
def test_mg_fcg_meets_fp64_tolerance(gg, orc, part, sigma):
    rng = np.random.default_rng(sum(part))
    kappa = np.exp(sigma * rng.standard_normal(int(np.prod(part))))
    fnod = rng.standard_normal(int(np.prod(np.array(part) + 1)))
    _, V, A, b = _problem(gg, (0, 1) * 3, part, ("boundary",), kappa, gg.NodalField(fnod))
    x64, r64 = _solve(gg, A, b, gg.CGSolver(rtol=1e-10))
    x, rep = _solve(gg, A, b, gg.FCGSolver(rtol=1e-8, pc="mg"))
    assert rep.converged and rep.relres <= 1e-8
    r = b - A.to_scipy() @ x
    assert np.linalg.norm(r) <= 1.01e-8 * np.linalg.norm(b)
    assert np.linalg.norm(x - x64) <= 1e-5 * np.linalg.norm(x64)
    # against the oracle's own system and its Jacobi-PCG solution (FP64, 1e-10)
    ref = orc.poisson_q1((0, 1) * 3, part, ("boundary",), kappa=kappa, fkind=orc.F_NODAL,
                         fdata=fnod)
    ro = ref["b"] - orc.csc_mul(*ref["csc"], x)
    assert np.linalg.norm(ro) <= 1.01e-8 * np.linalg.norm(ref["b"])
    xo, _, rro = orc.pcg(*ref["csc"], ref["b"], 1e-10)
    assert rro <= 1e-10
    assert np.linalg.norm(x - xo) <= 1e-5 * np.linalg.norm(xo)
    if part[0] % 4 == 0:  # at least three levels
        assert rep.iterations < 0.25 * r64.iterations


def test_mg_on_smooth_coefficient_converges_in_few_iterations(gg):
    part = (64, 64, 64)
    kappa = np.ones(int(np.prod(part)))
    fnod = np.random.default_rng(3).standard_normal(int(np.prod(np.array(part) + 1)))
    _, V, A, b = _problem(gg, (0, 1) * 3, part, ("boundary",), kappa, gg.NodalField(fnod))
    x, rep = _solve(gg, A, b, gg.FCGSolver(rtol=1e-8, pc="mg"))
    assert rep.converged and rep.relres <= 1e-8 and rep.iterations <= 30


def test_mg_without_lattice_form_is_refused(gg):
    part = (8, 8, 8)
    kappa = np.ones(int(np.prod(part)))
    _, V, A, b = _problem(gg, (0, 1) * 3, part, ("tag_21",), kappa, 1.0)
    with pytest.raises(gg._lib.GfeError):
        _solve(gg, A, b, gg.FCGSolver(rtol=1e-8, pc="mg"))


@pytest.mark.parametrize("part,jit", [((12, 10, 8), 0.2), ((16, 16, 16), 0.0)])
def test_q2_pmultigrid_fcg(gg, orc, part, jit):
    """Q2 on Cartesian hexahedra (nodes jittered by up to 0.2 h): flexible CG with the
    p-multigrid preconditioner (Jacobi-smoothed Q2 level, Q1 lattice V-cycle below) meets the
    FP64 relative residual in the oracle's own system, in far fewer iterations than
    Jacobi-preconditioned CG."""
    rng = np.random.default_rng(sum(part) + 7)
    nn = int(np.prod(np.array(part) + 1))
    h = 1.0 / np.array(part)
    jitter = rng.uniform(-jit, jit, (nn, 3)) * h
    model = gg.CartesianDiscreteModel((0, 1) * 3, part, node_jitter=jitter)
    V = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 2), dirichlet_tags="boundary")
    dO = gg.Measure(gg.Triangulation(model), 4)
    A, b = gg.assemble_matrix_and_vector(
        lambda u, v: gg.integrate(gg.inner(gg.grad(v), gg.grad(u)), dO),
        lambda v: gg.integrate(1.0 * v, dO), V, V)
    x, rep = _solve(gg, A, b, gg.FCGSolver(rtol=1e-8, pc="mg"))
    assert rep.converged and rep.relres <= 1e-8
    _, rj = _solve(gg, A, b, gg.CGSolver(rtol=1e-8))
    assert rep.iterations < 0.25 * rj.iterations
    ref = orc.poisson_q2((0, 1) * 3, part, ("boundary",), kappa=None, fconst=1.0, degree=4,
                         jitter=jitter)
    ro = ref["b"] - orc.csc_mul(*ref["csc"], x)
    assert np.linalg.norm(ro) <= 1.01e-8 * np.linalg.norm(ref["b"])


def test_mg_fcg_cached_loop_follows_new_kappa(gg):
    """The context keeps the multigrid hierarchy and the device loop graph between solves
    while the buffers they read stay the same: a solve after re-assembling with a new kappa,
    and after a solve of another size in between, must equal the same solve with the cache
    out of play (kernel timing on: a fresh hierarchy and the host-driven loop)."""
    rng = np.random.default_rng(77)
    part = (24, 24, 24)
    ncells = int(np.prod(part))
    fnod = rng.standard_normal(int(np.prod(np.array(part) + 1)))
    kaps = [np.exp(1.5 * rng.standard_normal(ncells)) for _ in range(2)]

    def run(kap, p=part, f=fnod):
        _, _, A, b = _problem(gg, (0, 1) * 3, p, ("boundary",), kap, gg.NodalField(f))
        return _solve(gg, A, b, gg.FCGSolver(rtol=1e-8, pc="mg"))

    x0, r0 = run(kaps[0])
    x1, r1 = run(kaps[1])           # same buffers, new kappa: the hierarchy is refreshed
    run(np.ones(8 ** 3), (8, 8, 8), np.ones(9 ** 3))  # another size in between
    x1b, r1b = run(kaps[1])
    ctx = gg.default_context()
    ctx.set_timing(True)
    try:
        x1ref, r1ref = run(kaps[1])
    finally:
        ctx.set_timing(False)
    for x, r in ((x1, r1), (x1b, r1b)):
        assert r.converged and r.iterations == r1ref.iterations
        assert np.linalg.norm(x - x1ref) <= 1e-12 * np.linalg.norm(x1ref)
    assert r0.converged and np.linalg.norm(x0 - x1) > 1e-3 * np.linalg.norm(x1)


def test_mg_fcg_device_loop_limits(gg):
    """The device-driven loop stops at maxiter (not converged, the FP64 residual of the
    iterate it reached, equal to the uncached host-driven loop's), solves b = 0 at once, and a
    NaN in b ends the solve with a non-finite residual instead of running on."""
    rng = np.random.default_rng(5)
    part = (16, 16, 16)
    kappa = np.exp(rng.standard_normal(int(np.prod(part))))
    fnod = rng.standard_normal(int(np.prod(np.array(part) + 1)))
    _, _, A, b = _problem(gg, (0, 1) * 3, part, ("boundary",), kappa, gg.NodalField(fnod))
    x, rep = _solve(gg, A, b, gg.FCGSolver(rtol=1e-12, pc="mg", maxiter=2))
    assert not rep.converged and rep.iterations == 2
    r = b - A.to_scipy() @ x
    assert abs(rep.relres - np.linalg.norm(r) / np.linalg.norm(b)) <= 1e-6 * rep.relres
    ctx = gg.default_context()
    ctx.set_timing(True)
    try:
        xh, reph = _solve(gg, A, b, gg.FCGSolver(rtol=1e-12, pc="mg", maxiter=2))
    finally:
        ctx.set_timing(False)
    assert reph.iterations == 2 and np.linalg.norm(x - xh) <= 1e-12 * np.linalg.norm(xh)
    x0, rep0 = _solve(gg, A, np.zeros_like(b), gg.FCGSolver(rtol=1e-8, pc="mg"))
    assert rep0.converged and rep0.iterations == 0 and not np.any(x0)
    bn = b.copy()
    bn[7] = np.nan
    xn, repn = _solve(gg, A, bn, gg.FCGSolver(rtol=1e-8, pc="mg", maxiter=50))
    assert not repn.converged and repn.iterations <= 50
    assert repn.status == gg._lib.GFE_ERR_NONFINITE or not np.isfinite(repn.relres)


def test_mg_fcg_pinned_host_x(gg):
    """A page-locked host x (the e2e route) must get what a device x gets: repeated solves
    into new buffers, a solve stopped by maxiter, and a NaN in b (reported from the error word
    that comes back with the solve's last wait)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    part = (24, 20, 16)
    kappa = np.exp(1.5 * rng.standard_normal(int(np.prod(part))))
    fnod = rng.standard_normal(int(np.prod(np.array(part) + 1)))
    _, _, A, b = _problem(gg, (0, 1) * 3, part, ("boundary",), kappa, gg.NodalField(fnod))
    n = b.size
    for maxiter, bb in ((100, b), (100, 2.0 * b), (3, b)):
        xd = torch.zeros(n, dtype=torch.float64, device="cuda")
        _, repd = _solve_into(gg, A, bb, xd, maxiter)
        for _ in range(2):
            xp = torch.full((n,), -1.0, dtype=torch.float64).pin_memory()
            _, repp = _solve_into(gg, A, bb, xp, maxiter)
            assert repp.iterations == repd.iterations and repp.converged == repd.converged
            assert np.array_equal(xp.numpy(), xd.cpu().numpy())
    bn = b.copy()
    bn[3] = np.nan
    xp = torch.zeros(n, dtype=torch.float64).pin_memory()
    _, repn = _solve_into(gg, A, bn, xp, 50)
    assert not repn.converged
    assert repn.status == gg._lib.GFE_ERR_NONFINITE or not np.isfinite(repn.relres)


def _solve_into(gg, A, b, x, maxiter):
    ns = gg.numerical_setup(gg.symbolic_setup(gg.FCGSolver(rtol=1e-8, pc="mg",
                                                             maxiter=maxiter), A), A)
    gg.solve_(x, ns, b)
    return x, ns.report


def test_mg_fcg_cached_graph_follows_settings(gg):
    """The cached solve graph bakes in its start's settings (rtol, maxiter): alternating them on
    one matrix must give each setting's own result, equal to a first solve with it."""
    rng = np.random.default_rng(23)
    part = (20, 16, 24)
    kappa = np.exp(1.2 * rng.standard_normal(int(np.prod(part))))
    fnod = rng.standard_normal(int(np.prod(np.array(part) + 1)))
    _, _, A, b = _problem(gg, (0, 1) * 3, part, ("boundary",), kappa, gg.NodalField(fnod))
    settings = [(1e-4, 1000), (1e-10, 1000), (1e-10, 3), (1e-4, 1000), (1e-10, 1000)]
    first = {}
    for rtol, maxiter in settings:
        x, rep = _solve(gg, A, b, gg.FCGSolver(rtol=rtol, pc="mg", maxiter=maxiter))
        if maxiter > 3:
            assert rep.converged and rep.relres <= rtol * (1 + 1e-6)
        else:
            assert not rep.converged and rep.iterations == 3
        key = (rtol, maxiter)
        if key in first:
            x0, rep0 = first[key]
            assert rep.iterations == rep0.iterations and np.array_equal(x, x0)
        else:
            first[key] = (x, rep)
