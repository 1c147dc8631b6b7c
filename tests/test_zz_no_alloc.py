"""The allocation-free solve entry point (gfe_cg_solve_noalloc), through the C ABI.

It exists for callers that cannot call cudaMalloc -- applications whose device memory
belongs to their own pool or arena and that must not have a library allocate while they
run. The test hands it a matrix and vectors that the test itself placed in device memory,
calls it twice in a row (the two calls share the library's fixed scratch array, so the
second must not see leftovers of the first), and compares both results with the regular
allocating solve (gfe_solve, FP64 Jacobi-PCG) within the solution tolerance the parity
tests use: ||x - x_ref|| / ||x_ref|| <= 1e3 * rtol. It lives in its own file, collected
last, and runs the same alone in a fresh process or after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _system(gg):
    rng = np.random.default_rng(77)
    part = (30, 28, 26)  # 29*27*25 = 19,575 free dofs
    model = gg.CartesianDiscreteModel((0, 1) * 3, part)
    V = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    kap = gg.CellField(np.exp(rng.standard_normal(model.num_cells())))
    f = gg.NodalField(rng.standard_normal(model.num_nodes()))
    dO = gg.Measure(gg.Triangulation(model), 2)
    op = gg.AffineFEOperator(lambda u, v: gg.integrate(kap * gg.inner(gg.grad(v), gg.grad(u)), dO),
                             lambda v: gg.integrate(f * v, dO), V, V)
    return op


def test_noalloc_solve_matches_allocating_solve(gg):
    torch = pytest.importorskip("torch")
    lib = gg._lib.load()
    op = _system(gg)
    A, b = op.A, op.b
    x_ref = np.empty_like(b)
    ns = gg.numerical_setup(gg.symbolic_setup(gg.CGSolver(rtol=RTOL), A), A)
    gg.solve_(x_ref, ns, b)
    assert ns.report.converged

    rp, cv, nz = A.export_csr(0)
    dev = torch.device("cuda:0")
    d_rp = torch.tensor(rp.astype(np.int32), device=dev)
    d_cv = torch.tensor(cv.astype(np.int32), device=dev)
    d_nz = torch.tensor(nz, device=dev)
    d_b = torch.tensor(b, device=dev)
    n = b.shape[0]
    for call in range(2):
        d_x = torch.full((n,), np.nan, dtype=torch.float64, device=dev)
        it = ctypes.c_int32()
        rr = ctypes.c_double()
        st = lib.gfe_cg_solve_noalloc(d_rp.data_ptr(), d_cv.data_ptr(), d_nz.data_ptr(), n,
                                      nz.shape[0], d_b.data_ptr(), d_x.data_ptr(), RTOL, 100000,
                                      None, ctypes.byref(it), ctypes.byref(rr))
        gg._lib.check(st)
        x = d_x.cpu().numpy()
        assert rr.value <= RTOL, (call, rr.value)
        assert it.value > 0
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) <= 1e3 * RTOL, call


def test_noalloc_rejects_oversized_and_host_inputs(gg):
    torch = pytest.importorskip("torch")
    lib = gg._lib.load()
    dev = torch.device("cuda:0")
    one = torch.zeros(4, dtype=torch.int32, device=dev)
    v = torch.zeros(4, dtype=torch.float64, device=dev)
    it, rr = ctypes.c_int32(), ctypes.c_double()
    st = lib.gfe_cg_solve_noalloc(one.data_ptr(), one.data_ptr(), v.data_ptr(), 1 << 20, 0,
                                  v.data_ptr(), v.data_ptr(), 1e-8, 10, None, ctypes.byref(it),
                                  ctypes.byref(rr))
    assert st == gg._lib.GFE_ERR_INVALID_ARGUMENT
    assert b"exceed" in lib.gfe_last_error()
    h = np.zeros(4)
    st = lib.gfe_cg_solve_noalloc(one.data_ptr(), one.data_ptr(), v.data_ptr(), 3, 0,
                                  h.ctypes.data, v.data_ptr(), 1e-8, 10, None, ctypes.byref(it),
                                  ctypes.byref(rr))
    assert st == gg._lib.GFE_ERR_INVALID_ARGUMENT
