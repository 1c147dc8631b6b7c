"""Learned block preconditioner for flexible CG (libgfe `gfe_learned_pc_*`, `gfe_solve_fcg`).

The preconditioner groups the cells of a 3-D Cartesian Q1 problem in 2x2x2 blocks and maps
each block's residual patch (27 values, RMS-normalised) and log-kappa pattern (8 values)
through a 35 -> 64 -> 64 -> 27 MLP (BF16 weights, FP32 accumulation on the tensor cores) to
an estimate of the block's error; block results are averaged at shared nodes. It runs alone
inside flexible CG, or as the fine-level smoother of the multigrid V-cycle
(`FCGSolver(pc=learned, multigrid=True)`: pre-smoothing x = M(b), post-smoothing
x += M(b - A x), coarser levels damped Jacobi), with Jacobi as the fallback on stagnation.

Training (`train`) uses residual / error pairs of the method's own FP64 solves: for
independent kappa draws it assembles the system, solves it with FP64 CG to 1e-12 (x*), runs
FP64 CG again from x0 = x* + white noise for a few iteration counts k, and for random blocks
records the residual patch of r_k = b - A x_k (the input) and the error patch of
e_k = x* - x_k (the target). The MLP is fitted with hand-written FP32 kernels (Adam).
`train_local_solves` keeps the earlier targets (the block's local solve A_b^{-1} r_b).
"""
from __future__ import annotations

import ctypes as C
import pathlib

import numpy as np

from . import _lib
from .assembly import DeviceMatrix, default_context
from .fespaces import FESpace

N_IN, N_OUT = 48, 32
WEIGHTS_FILE = pathlib.Path(__file__).resolve().parent / "data" / "learned_pc_q1_lognormal.npy"


class LearnedBlockPreconditioner:
    def __init__(self, V: FESpace, kappa, ctx=None):
        lib = _lib.load()
        self.ctx = ctx or default_context()
        model = V.model
        if model.dim != 3 or V.reffe.order != 1 or V.reffe.ncomp != 1:
            raise NotImplementedError("the learned block preconditioner is for scalar 3-D Q1")
        part = np.asarray(model.partition, dtype=np.int64)
        dom = np.asarray(model.domain, dtype=np.float64)
        n2d = np.ascontiguousarray(V.node_comp_to_dof[:, 0], dtype=np.int32)
        kap = np.ascontiguousarray(np.asarray(kappa, dtype=np.float64))
        h = C.c_void_p()
        _lib.check(lib.gfe_learned_pc_create(self.ctx.handle, _lib.ptr(part), _lib.ptr(dom),
                                             _lib.ptr(n2d), V.num_free_dofs(), _lib.ptr(kap),
                                             C.byref(h)))
        self.handle = h
        self.ctx._own(self)
        self.nfree = V.num_free_dofs()
        self.nblocks = int(np.prod((part + 1) // 2))

    @staticmethod
    def num_params() -> int:
        return _lib.load().gfe_learned_pc_num_params()

    def set_weights(self, params: np.ndarray):
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != self.num_params():
            raise ValueError("wrong number of parameters")
        _lib.check(_lib.load().gfe_learned_pc_set_weights(self.handle, _lib.ptr(p)))

    def get_weights(self) -> np.ndarray:
        p = np.empty(self.num_params(), dtype=np.float32)
        _lib.check(_lib.load().gfe_learned_pc_get_weights(self.handle, _lib.ptr(p)))
        return p

    def load_default_weights(self):
        self.set_weights(np.load(WEIGHTS_FILE))

    def apply(self, r, z):
        """z = M(r) for FP32 CUDA tensors."""
        _lib.check(_lib.load().gfe_learned_pc_apply(self.handle, _lib.ptr(r), _lib.ptr(z)))
        return z

    def samples(self, A: DeviceMatrix, r, block_ids, X, T):
        ids = np.ascontiguousarray(block_ids, dtype=np.int64)
        rr = np.ascontiguousarray(r, dtype=np.float64) if isinstance(r, np.ndarray) else r
        _lib.check(_lib.load().gfe_learned_pc_samples(self.handle, A.handle, _lib.ptr(rr),
                                                      ids.shape[0], _lib.ptr(ids), _lib.ptr(X),
                                                      _lib.ptr(T)))

    def samples_error(self, r, e, block_ids, X, T):
        """Training rows from a residual / error pair (FP64, host or device)."""
        ids = np.ascontiguousarray(block_ids, dtype=np.int64)
        rr = np.ascontiguousarray(r, dtype=np.float64) if isinstance(r, np.ndarray) else r
        ee = np.ascontiguousarray(e, dtype=np.float64) if isinstance(e, np.ndarray) else e
        _lib.check(_lib.load().gfe_learned_pc_samples_error(
            self.handle, _lib.ptr(rr), _lib.ptr(ee), ids.shape[0], _lib.ptr(ids), _lib.ptr(X),
            _lib.ptr(T)))

    def fit(self, X, T, epochs=40, batch=2048, lr=2e-3, seed=0) -> float:
        loss = C.c_float()
        _lib.check(_lib.load().gfe_learned_pc_train(self.handle, _lib.ptr(X), _lib.ptr(T),
                                                    X.shape[0], epochs, batch, lr, seed,
                                                    C.byref(loss)))
        return loss.value

    def _release(self):
        h, self.handle = self.handle, None
        if h and self.ctx.handle:
            _lib.load().gfe_learned_pc_destroy(h)

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass


def train(n: int = 64, draws: int = 200, seed0: int = 5000, iterates=(0, 1, 2, 4),
          blocks_per_pair: int = 256, epochs: int = 40, batch: int = 2048, lr: float = 2e-3,
          log=print):
    """Trains the block MLP on residual / error pairs of FP64 CG iterations on `draws`
    independent lognormal kappa fields (seeds seed0, seed0+1, ...) on n^3 grids: x* from an
    FP64 CG solve to 1e-12, then FP64 CG from x0 = x* + noise (white noise, 0.1 times the
    RMS of x*) stopped after k iterations for each k in `iterates`; inputs from
    r_k = b - A x_k, targets e_k = x* - x_k. Returns the FP32 parameters and the final
    training loss."""
    import torch

    from . import workloads
    from .assembly import assemble_matrix_and_vector, SparseMatrixAssembler
    from .celldata import CellField, inner, grad, integrate
    from .solvers import CGSolver, numerical_setup, solve_, symbolic_setup

    ctx = default_context()
    dev = torch.device("cuda", ctx.device)
    rng = np.random.default_rng(seed0)
    nsamp = draws * len(iterates) * blocks_per_pair
    X = torch.empty((nsamp, N_IN), dtype=torch.float32, device=dev)
    T = torch.empty((nsamp, N_OUT), dtype=torch.float32, device=dev)
    row = 0
    pc = None
    for d in range(draws):
        w = workloads.lognormal_3d(n=n, seed=seed0 + d)
        V, dO = w.space, w.measure
        kap = CellField(w.kappa)
        A, b = assemble_matrix_and_vector(
            lambda u, v: integrate(kap * inner(grad(v), grad(u)), dO),
            lambda v: integrate(w.source * v, dO), V, V, SparseMatrixAssembler(V, V))
        pcd = LearnedBlockPreconditioner(V, w.kappa, ctx)
        xs = np.empty_like(b)
        ns = numerical_setup(symbolic_setup(CGSolver(rtol=1e-12), A), A)
        solve_(xs, ns, b)
        # start: the solution plus white noise, so that e_0 is the noise (every frequency at
        # the same amplitude) and the CG iterates damp it from the top of the spectrum down
        x0 = xs + 0.1 * np.sqrt(np.mean(xs * xs)) * rng.standard_normal(b.shape[0])
        for k in iterates:
            x = x0.copy()
            if k > 0:
                ns = numerical_setup(symbolic_setup(
                    CGSolver(rtol=1e-30, maxiter=k, initial_guess=True), A), A)
                solve_(x, ns, b)
            r = b - A.matvec(x)
            e = xs - x
            ids = rng.integers(0, pcd.nblocks, blocks_per_pair)
            pcd.samples_error(r, e, ids, X[row:row + len(ids)], T[row:row + len(ids)])
            row += len(ids)
        if pc is None:
            pc = pcd
        if log and (d + 1) % 50 == 0:
            log(f"samples from {d + 1} draws")
    perm = torch.randperm(nsamp, device=dev, generator=torch.Generator(device=dev).manual_seed(1))
    X, T = X[perm].contiguous(), T[perm].contiguous()
    loss = pc.fit(X, T, epochs=epochs, batch=batch, lr=lr, seed=seed0)
    return pc.get_weights(), loss


def train_local_solves(n: int = 64, draws: int = 200, seed0: int = 5000,
                       snapshots=(5, 20, 60, 150),
          blocks_per_snapshot: int = 256, epochs: int = 40, batch: int = 2048, lr: float = 2e-3,
          log=print):
    """The earlier targets: residual / local-solve pairs (A_b^{-1} r_b, FP64) from FP64
    Jacobi-PCG iterates of `draws` independent lognormal kappa fields on n^3 grids. Returns
    the FP32 parameters and the final training loss."""
    import torch

    from . import workloads
    from .assembly import assemble_matrix_and_vector, SparseMatrixAssembler
    from .celldata import CellField, inner, grad, integrate
    from .solvers import CGSolver, numerical_setup, solve_, symbolic_setup

    ctx = default_context()
    dev = torch.device("cuda", ctx.device)
    rng = np.random.default_rng(seed0)
    nsamp = draws * len(snapshots) * blocks_per_snapshot
    X = torch.empty((nsamp, N_IN), dtype=torch.float32, device=dev)
    T = torch.empty((nsamp, N_OUT), dtype=torch.float32, device=dev)
    row = 0
    pc = None
    for d in range(draws):
        w = workloads.lognormal_3d(n=n, seed=seed0 + d)
        V, dO = w.space, w.measure
        kap = CellField(w.kappa)
        A, b = assemble_matrix_and_vector(
            lambda u, v: integrate(kap * inner(grad(v), grad(u)), dO),
            lambda v: integrate(w.source * v, dO), V, V, SparseMatrixAssembler(V, V))
        pcd = LearnedBlockPreconditioner(V, w.kappa, ctx)
        for k in snapshots:
            x = np.empty_like(b)
            ns = numerical_setup(symbolic_setup(CGSolver(rtol=1e-30, maxiter=k), A), A)
            solve_(x, ns, b)
            r = b - A.matvec(x)
            ids = rng.integers(0, pcd.nblocks, blocks_per_snapshot)
            pcd.samples(A, r, ids, X[row:row + len(ids)], T[row:row + len(ids)])
            row += len(ids)
        if pc is None:
            pc = pcd
        if log and (d + 1) % 50 == 0:
            log(f"samples from {d + 1} draws")
    perm = torch.randperm(nsamp, device=dev, generator=torch.Generator(device=dev).manual_seed(1))
    X, T = X[perm].contiguous(), T[perm].contiguous()
    loss = pc.fit(X, T, epochs=epochs, batch=batch, lr=lr, seed=seed0)
    return pc.get_weights(), loss
