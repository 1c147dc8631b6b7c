"""Learned block preconditioner for flexible CG (libgfe `gfe_learned_pc_*`, `gfe_solve_fcg`).

The preconditioner groups the cells of a 3-D Cartesian Q1 problem in 2x2x2 blocks and maps
each block's residual patch (27 values, RMS-normalised) and log-kappa pattern (8 values)
through a 35 -> 64 -> 64 -> 27 MLP (BF16 weights, FP32 accumulation on the tensor cores) to
an approximation of the block's local solve; block results are averaged at shared nodes.

Training (`train`) uses only the method's own FP64 solves: for independent kappa draws it
assembles the system, runs FP64 Jacobi-PCG for a few iteration counts, takes the residuals
r_k = b - A x_k, and for random blocks records the input patch and the target A_b^{-1} r_b
(the block's local solve in FP64). The MLP is fitted with hand-written FP32 kernels (Adam).
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


def train(n: int = 64, draws: int = 200, seed0: int = 5000, snapshots=(5, 20, 60, 150),
          blocks_per_snapshot: int = 256, epochs: int = 40, batch: int = 2048, lr: float = 2e-3,
          log=print):
    """Trains the block MLP on residual / local-solve pairs from FP64 solves of `draws`
    independent lognormal kappa fields (seeds seed0, seed0+1, ...) on n^3 grids. Returns the
    FP32 parameters and the final training loss."""
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
