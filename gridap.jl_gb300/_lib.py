"""ctypes binding of libgfe (include/gfe.h).

The library is built in-tree by ``build.py`` into ``_build/libgfe.so``. Loading fails
loudly when it is missing: there is no CPU fallback for any operation of this package.
"""
from __future__ import annotations

import ctypes as C
import pathlib

import numpy as np

_HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = _HERE / "_build" / "libgfe.so"

# status codes (gfe.h)
GFE_OK = 0
GFE_ERR_INVALID_ARGUMENT = 1
GFE_ERR_CUDA = 2
GFE_ERR_OUT_OF_MEMORY = 3
GFE_ERR_DEGENERATE_CELL = 4
GFE_ERR_ROW_TOO_WIDE = 5
GFE_ERR_TIMEOUT = 6
GFE_ERR_UNSUPPORTED = 7
GFE_ERR_NONFINITE = 8
GFE_ERR_NOT_CONVERGED = 9

GFE_REFFE_Q1, GFE_REFFE_Q2 = 1, 2
GFE_GEOM_CARTESIAN, GFE_GEOM_NODAL = 0, 1
GFE_FORM_DIFFUSION, GFE_FORM_ELASTICITY, GFE_FORM_QUASILINEAR = 1, 2, 3
GFE_REFFE_Q1, GFE_REFFE_Q2, GFE_REFFE_P2_TET = 1, 2, 3
GFE_COEF_ONE, GFE_COEF_CONST, GFE_COEF_CELL = 0, 1, 2
GFE_SRC_NONE, GFE_SRC_CONST, GFE_SRC_NODAL, GFE_SRC_QPOINT, GFE_SRC_SINSUM = 0, 1, 2, 3, 4
GFE_BOP_VALUE, GFE_BOP_NORMAL_GRAD = 0, 1
GFE_LAW_POLY, GFE_LAW_POWER = 0, 1
GFE_REORDER_RCM, GFE_REORDER_SLOAN = 0, 1
GFE_PREC_FP64, GFE_PREC_FP32 = 0, 1
GFE_SOLVER_CG, GFE_SOLVER_IR_CG, GFE_SOLVER_MIXED_CG, GFE_SOLVER_BICGSTAB = 0, 1, 2, 3
GFE_PC_NONE, GFE_PC_JACOBI, GFE_PC_MG = 0, 1, 2
GFE_MOP_VALUE, GFE_MOP_GRAD, GFE_MOP_DIV = 0, 1, 2
GFE_KT_SPMV64, GFE_KT_SPMV32, GFE_KT_ASSEMBLE, GFE_KT_RESIDUAL64, GFE_KT_ELEMENT = 0, 1, 2, 3, 4
GFE_KT_PRECOND, GFE_KT_VECTOR = 5, 6


class GfeError(RuntimeError):
    """A libgfe call returned a non-zero status (Gridap would raise `error(...)`)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"libgfe error {code}: {msg}")
        self.code = code


class Problem(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("reffe", C.c_int32), ("ncomp", C.c_int32), ("degree", C.c_int32),
        ("ncells", C.c_int64), ("nd", C.c_int32), ("cell_dof_ids", C.c_void_p),
        ("nfree", C.c_int64),
        ("geometry", C.c_int32), ("partition", C.c_int64 * 3), ("domain", C.c_double * 6),
        ("nnodes", C.c_int64), ("node_coords", C.c_void_p), ("cell_node_ids", C.c_void_p),
        ("form", C.c_int32), ("coef_kind", C.c_int32), ("coef", C.c_void_p),
        ("source_kind", C.c_int32), ("source", C.c_void_p), ("source_len", C.c_int64),
        ("precision", C.c_int32), ("dirichlet_values", C.c_void_p), ("ndirichlet", C.c_int64),
        ("state", C.c_void_p), ("law", C.c_int32), ("law_params", C.c_double * 4),
    ]


class MfField(C.Structure):
    """gfe_mf_field."""
    _fields_ = [("ncomp", C.c_int32), ("nnodes", C.c_int32), ("shapes", C.c_void_p),
                ("grads", C.c_void_p)]


class MfTerm(C.Structure):
    """gfe_mf_term."""
    _fields_ = [("test_field", C.c_int32), ("trial_field", C.c_int32),
                ("test_op", C.c_int32), ("trial_op", C.c_int32), ("coef", C.c_double),
                ("cell_coef", C.c_void_p), ("qdata", C.c_void_p), ("qdata_ncomp", C.c_int32)]


class MfProblem(C.Structure):
    """gfe_mf_problem."""
    _fields_ = [("dim", C.c_int32), ("ncells", C.c_int64), ("nnodes", C.c_int64),
                ("node_coords", C.c_void_p), ("cell_node_ids", C.c_void_p), ("nq", C.c_int32),
                ("qweights", C.c_void_p), ("geo_grads", C.c_void_p), ("nfields", C.c_int32),
                ("fields", C.c_void_p), ("nterms", C.c_int32), ("terms", C.c_void_p)]


class SolverOpts(C.Structure):
    _fields_ = [("method", C.c_int32), ("precond", C.c_int32), ("rtol", C.c_double),
                ("maxiter", C.c_int32), ("inner_rtol", C.c_double), ("check_every", C.c_int32),
                ("initial_guess", C.c_int32)]


class SolveReport(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("refinements", C.c_int32), ("converged", C.c_int32),
                ("status", C.c_int32), ("relres", C.c_double), ("operator_format", C.c_int32),
                ("ndiag", C.c_int32), ("fallback", C.c_int32)]


_P = C.c_void_p
_I64P = C.POINTER(C.c_int64)

# name -> (restype, argtypes); every function in include/gfe.h
SIGNATURES = {
    "gfe_last_error": (C.c_char_p, []),
    "gfe_version": (C.c_char_p, []),
    "gfe_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "gfe_ctx_destroy": (C.c_int, [_P]),
    "gfe_ctx_stream": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
    "gfe_ctx_synchronize": (C.c_int, [_P]),
    "gfe_ctx_kernel_launches": (C.c_int, [_P, _I64P]),
    "gfe_ctx_set_timing": (C.c_int, [_P, C.c_int]),
    "gfe_ctx_set_wait_limit": (C.c_int, [_P, C.c_uint64]),
    "gfe_ctx_kernel_time": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double), _I64P]),
    "gfe_cartesian_model": (C.c_int, [C.c_int, _P, _P, _P, _P, _P]),
    "gfe_clagrangian_dofs": (C.c_int, [C.c_int64, _P, C.c_int, _P, C.c_int64, C.c_int, _P, _P,
                                       _P, _P, _P, _P]),
    "gfe_cartesian_conforming_dofs": (C.c_int, [C.c_int, C.c_int, _P, C.c_int, _P, _P, _P, _P,
                                                _P]),
    "gfe_symbolic_loop_matrix": (C.c_int, [_P, C.c_int64, C.c_int, _P, _P, C.c_int64,
                                           C.c_int64, C.POINTER(C.c_void_p)]),
    "gfe_symbolic_loop_matrix_rect": (C.c_int, [_P, C.c_int64, C.c_int, C.c_int, _P, _P,
                                                C.c_int64, C.c_int64, C.POINTER(C.c_void_p)]),
    "gfe_symbolic_loop_matrix_problem": (C.c_int, [_P, _P, C.POINTER(C.c_void_p)]),
    "gfe_symbolic_loop_matrix_masked": (C.c_int, [_P, C.c_int64, C.c_int, C.c_int, _P, _P, _P,
                                                  C.c_int64, C.c_int64,
                                                  C.POINTER(C.c_void_p)]),
    "gfe_multifield_assemble": (C.c_int, [_P, _P, C.c_int32, _P, C.c_int32, _P, _P, _P, _P,
                                          C.c_int64, _P, C.c_int64, _P]),
    "gfe_matrix_destroy": (C.c_int, [_P]),
    "gfe_matrix_info": (C.c_int, [_P, _I64P, _I64P, _I64P]),
    "gfe_matrix_export_csr": (C.c_int, [_P, C.c_int, _P, _P, _P]),
    "gfe_matrix_fillstored_zero": (C.c_int, [_P]),
    "gfe_numeric_loop_matrix": (C.c_int, [_P, _P, _P]),
    "gfe_numeric_loop_vector": (C.c_int, [_P, C.c_int64, C.c_int, _P, _P, C.c_int64, _P]),
    "gfe_assemble_matrix_and_vector": (C.c_int, [_P, C.POINTER(Problem), _P, _P]),
    "gfe_solve": (C.c_int, [_P, _P, C.POINTER(SolverOpts), _P, _P, C.POINTER(SolveReport)]),
    "gfe_matrix_mul": (C.c_int, [_P, _P, _P, _P]),
    "gfe_learned_pc_create": (C.c_int, [_P, _P, _P, _P, C.c_int64, _P, C.POINTER(C.c_void_p)]),
    "gfe_learned_pc_destroy": (C.c_int, [_P]),
    "gfe_learned_pc_num_params": (C.c_int, []),
    "gfe_learned_pc_set_weights": (C.c_int, [_P, _P]),
    "gfe_learned_pc_get_weights": (C.c_int, [_P, _P]),
    "gfe_learned_pc_apply": (C.c_int, [_P, _P, _P]),
    "gfe_learned_pc_samples": (C.c_int, [_P, _P, _P, C.c_int64, _P, _P, _P]),
    "gfe_learned_pc_samples_error": (C.c_int, [_P, _P, _P, C.c_int64, _P, _P, _P]),
    "gfe_learned_pc_train": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int32, C.c_int32, C.c_float,
                                       C.c_uint64, C.POINTER(C.c_float)]),
    "gfe_solve_fcg": (C.c_int, [_P, _P, _P, C.POINTER(SolverOpts), _P, _P,
                                C.POINTER(SolveReport)]),
    "gfe_simplex_model": (C.c_int, [_P, _P]),
    "gfe_assemble_boundary_vector": (C.c_int, [_P, C.POINTER(Problem), C.c_int64, _P, _P,
                                               C.c_int32, C.c_int32, C.c_int32, _P, C.c_int64,
                                               _P]),
    "gfe_dof_permutation": (C.c_int, [_P, C.c_int64, C.c_int32, _P, C.c_int64, C.c_int32,
                                      C.c_int32, C.c_int32, _P]),
    "gfe_assemble_boundary_matrix": (C.c_int, [_P, C.POINTER(Problem), _P, _P, C.c_int64, _P,
                                               _P, C.c_int32, _P]),
    "gfe_simplex_p2_dofs": (C.c_int, [_P, C.c_int32, _P, _P, _P, _P, _P]),
    "gfe_batch_create": (C.c_int, [_P, C.c_int32, _P, _P, C.POINTER(C.c_void_p)]),
    "gfe_batch_destroy": (C.c_int, [_P]),
    "gfe_batch_info": (C.c_int, [_P, _I64P, _I64P, _I64P]),
    "gfe_batch_shape": (C.c_int, [_P, _P, _P, _P]),
    "gfe_batch_set_shape": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_double]),
    "gfe_batch_assemble_solve": (C.c_int, [_P, C.c_double, C.c_double, C.c_int32, _P, _P,
                                           C.POINTER(C.c_int32)]),
    "gfe_cg_solve_noalloc": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, _P, _P, C.c_double,
                                       C.c_int32, _P, C.POINTER(C.c_int32),
                                       C.POINTER(C.c_double)]),
}

_lib = None


def load(path: pathlib.Path | str | None = None) -> C.CDLL:
    """Loads libgfe.so (once). Raises if the library has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = pathlib.Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"libgfe.so not found at {p}: build it with `python gridap.jl_gb300/build.py` "
            "(there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != GFE_OK:
        msg = _lib.gfe_last_error().decode() if _lib is not None else ""
        raise GfeError(status, msg)


def ptr(a) -> int | None:
    """Address of a numpy array, a torch tensor, or None."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags.c_contiguous:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr()
    raise TypeError(f"cannot take the address of {type(a)}")
