"""The allocation-free solve entry point (gfe_cg_solve_noalloc), through the C ABI.

It exists for callers that cannot call cudaMalloc -- applications whose device memory
belongs to their own pool or arena and that must not have a library allocate while they
run. The test hands it a matrix and vectors that the test itself placed in device memory,
calls it twice in a row (the two calls share the library's fixed scratch array, so the
second must not see leftovers of the first), and compares both results with the regular
allocating solve (gfe_solve, FP64 Jacobi-PCG) and with the oracle's own Jacobi-PCG of the
oracle's matrix, within the solution tolerance the parity tests use:
||x - x_ref|| / ||x_ref|| <= 1e3 * rtol. The device's free memory (cudaMemGetInfo) must be
the same before and after each call. A NaN in b must come back as GFE_ERR_NONFINITE and a
solve cut off by maxiter as GFE_ERR_NOT_CONVERGED. It lives in its own file, collected last,
and runs the same alone in a fresh process or after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10


PART = (30, 28, 26)  # 29*27*25 = 19,575 free dofs


def _inputs():
    rng = np.random.default_rng(77)
    ncells = int(np.prod(PART))
    nnodes = int(np.prod(np.array(PART) + 1))
    return np.exp(rng.standard_normal(ncells)), rng.standard_normal(nnodes)


def _system(gg):
    kappa, fnod = _inputs()
    model = gg.CartesianDiscreteModel((0, 1) * 3, PART)
    V = gg.FESpace(model, gg.ReferenceFE(gg.lagrangian, float, 1), dirichlet_tags="boundary")
    kap = gg.CellField(kappa)
    f = gg.NodalField(fnod)
    dO = gg.Measure(gg.Triangulation(model), 2)
    op = gg.AffineFEOperator(lambda u, v: gg.integrate(kap * gg.inner(gg.grad(v), gg.grad(u)), dO),
                             lambda v: gg.integrate(f * v, dO), V, V)
    return op


def _device_system(torch, A, b):
    rp, cv, nz = A.export_csr(0)
    dev = torch.device("cuda:0")
    return (torch.tensor(rp.astype(np.int32), device=dev),
            torch.tensor(cv.astype(np.int32), device=dev), torch.tensor(nz, device=dev),
            torch.tensor(b, device=dev), nz.shape[0])


def _call(lib, d_rp, d_cv, d_nz, nnz, d_b, d_x, rtol, maxiter):
    it = ctypes.c_int32()
    rr = ctypes.c_double()
    st = lib.gfe_cg_solve_noalloc(d_rp.data_ptr(), d_cv.data_ptr(), d_nz.data_ptr(),
                                  d_b.shape[0], nnz, d_b.data_ptr(), d_x.data_ptr(), rtol,
                                  maxiter, None, ctypes.byref(it), ctypes.byref(rr))
    return st, it.value, rr.value


def test_noalloc_solve_matches_allocating_solve(gg, orc):
    torch = pytest.importorskip("torch")
    lib = gg._lib.load()
    op = _system(gg)
    A, b = op.A, op.b
    x_ref = np.empty_like(b)
    ns = gg.numerical_setup(gg.symbolic_setup(gg.CGSolver(rtol=RTOL), A), A)
    gg.solve_(x_ref, ns, b)
    assert ns.report.converged
    # the oracle's matrix and its own Jacobi-PCG on the same inputs
    kappa, fnod = _inputs()
    ref = orc.poisson_q1((0, 1) * 3, PART, ("boundary",), kappa=kappa, fkind=orc.F_NODAL,
                         fdata=fnod)
    x_orc, _, rr_orc = orc.pcg(*ref["csc"], ref["b"], RTOL)
    assert rr_orc <= RTOL

    d_rp, d_cv, d_nz, d_b, nnz = _device_system(torch, A, b)
    n = b.shape[0]
    for call in range(2):
        d_x = torch.full((n,), np.nan, dtype=torch.float64, device=dev_of(torch))
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(0)[0]
        st, it, rr = _call(lib, d_rp, d_cv, d_nz, nnz, d_b, d_x, RTOL, 100000)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info(0)[0]
        gg._lib.check(st)
        if call > 0:  # the first call may load the library's device code and its static array
            assert free1 == free0, f"device memory changed by {free0 - free1} bytes"
        x = d_x.cpu().numpy()
        assert rr <= RTOL, (call, rr)
        assert it > 0
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) <= 1e3 * RTOL, call
        assert np.linalg.norm(x - x_orc) / np.linalg.norm(x_orc) <= 1e3 * RTOL, call
        r = ref["b"] - orc.csc_mul(*ref["csc"], x)
        assert np.linalg.norm(r) / np.linalg.norm(ref["b"]) <= RTOL * (1 + 1e-3), call


def dev_of(torch):
    return torch.device("cuda:0")


def test_noalloc_reports_nonfinite_and_not_converged(gg):
    torch = pytest.importorskip("torch")
    lib = gg._lib.load()
    op = _system(gg)
    d_rp, d_cv, d_nz, d_b, nnz = _device_system(torch, op.A, op.b)
    n = op.b.shape[0]
    d_x = torch.zeros(n, dtype=torch.float64, device=dev_of(torch))
    # cut off after one iteration: the last iterate comes back with the status
    st, it, rr = _call(lib, d_rp, d_cv, d_nz, nnz, d_b, d_x, RTOL, 1)
    assert st == gg._lib.GFE_ERR_NOT_CONVERGED, lib.gfe_last_error()
    assert it == 1 and RTOL < rr < 1.0
    # a NaN in b
    d_bad = d_b.clone()
    d_bad[n // 2] = float("nan")
    st, it, rr = _call(lib, d_rp, d_cv, d_nz, nnz, d_bad, d_x, RTOL, 1000)
    assert st == gg._lib.GFE_ERR_NONFINITE, lib.gfe_last_error()
    # the shared array carries nothing over: the next solve is exact again
    st, it, rr = _call(lib, d_rp, d_cv, d_nz, nnz, d_b, d_x, RTOL, 100000)
    gg._lib.check(st)
    assert rr <= RTOL


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
