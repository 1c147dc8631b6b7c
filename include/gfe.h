/*
 * gfe.h -- C ABI of libgfe: GB300-native finite-element assembly and linear solve behind
 * Gridap.jl's assembler / linear-solver protocol.
 *
 * Every entry point replaces one step of Gridap's hot path; the comment above each one
 * names the Gridap function (path:line in Gridap.jl v0.20.8) whose behaviour it takes over.
 * A Julia shim reaches these with `ccall`; any C caller can use them directly.
 *
 * Conventions
 *   - Status: every function returns GFE_OK (0) or a GFE_ERR_* code; gfe_last_error()
 *     returns the message of the last failure on the calling thread. No exceptions and no
 *     process exit cross this boundary (Gridap turns a non-zero status into `error(...)`).
 *   - Ids follow Gridap: cell_dof_ids is a Table{Int32} with nd entries per cell, free dofs
 *     1..nfree, Dirichlet dofs negative (-1..-ndiri); negative ids are skipped by assembly
 *     exactly like Algebra/AlgebraInterfaces.jl:176-187.
 *   - Pointers may be host memory or device memory of the context's GPU; the library
 *     detects which (cudaPointerGetAttributes) and copies host data in/out on the context's
 *     stream. Outputs written to host memory are complete when the call returns.
 *   - Matrices live on the device inside a gfe_matrix and are exported on request as CSR
 *     (== CSC for the symmetric operators assembled here) with 0- or 1-based indices.
 *   - One context = one GPU, one CUDA stream, one calling thread (Gridap calls from one task).
 */
#ifndef GFE_H
#define GFE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------- */
enum {
  GFE_OK = 0,
  GFE_ERR_INVALID_ARGUMENT = 1,
  GFE_ERR_CUDA = 2,
  GFE_ERR_OUT_OF_MEMORY = 3,
  GFE_ERR_DEGENERATE_CELL = 4, /* det(J) <= 0 or not finite at a quadrature point */
  GFE_ERR_ROW_TOO_WIDE = 5,    /* a matrix row has more entries than the kernels support */
  GFE_ERR_TIMEOUT = 6,         /* a bounded device-side wait ran out */
  GFE_ERR_UNSUPPORTED = 7,     /* element / form / option combination not provided */
  GFE_ERR_NONFINITE = 8        /* NaN or Inf in coefficients, matrix or vectors */
};

typedef struct gfe_ctx gfe_ctx;
typedef struct gfe_matrix gfe_matrix;

/* Message of the last failing call on this thread ("" if none). */
const char* gfe_last_error(void);
/* Library version string. */
const char* gfe_version(void);

/* ---- context ----------------------------------------------------------------------------- */
int gfe_ctx_create(int device, gfe_ctx** ctx);
int gfe_ctx_destroy(gfe_ctx* ctx);
/* The context's cudaStream_t (as void*), for callers that time or order work around it. */
int gfe_ctx_stream(gfe_ctx* ctx, void** stream);
int gfe_ctx_synchronize(gfe_ctx* ctx);
/* Number of kernels this context has launched so far (for launch accounting). */
int gfe_ctx_kernel_launches(gfe_ctx* ctx, int64_t* count);
/* Kernel timing: when enabled, CUDA events on the context's stream bracket every launch of
 * the kernel classes below and their device times are summed. Enabling or disabling resets
 * the totals. gfe_ctx_kernel_time returns the total milliseconds and launch count. */
enum {
  GFE_KT_SPMV64 = 0,     /* FP64 SpMV + dot of the CG iteration */
  GFE_KT_SPMV32 = 1,     /* FP32 SpMV + dot of the inner CG iteration */
  GFE_KT_ASSEMBLE = 2,   /* row-gather numeric assembly */
  GFE_KT_RESIDUAL64 = 3, /* FP64 residual r = b - A x of iterative refinement */
  GFE_KT_ELEMENT = 4     /* element (cell-integral) kernels */
};
int gfe_ctx_set_timing(gfe_ctx* ctx, int enable);
int gfe_ctx_kernel_time(gfe_ctx* ctx, int kernel, double* total_ms, int64_t* launches);

/* ---- FE space set-up (host) -------------------------------------------------------------- */
/* CartesianDiscreteModel(domain, partition) arrays: node coordinates (nnodes*D, x fastest),
 * cell node ids (ncells * 2^D, 1-based, lexicographic local order) and the box entity of
 * every node (its face label). Any output may be NULL.
 * Replaces Geometry/CartesianGrids.jl:108-171 and CartesianDiscreteModels.jl:133-189. */
int gfe_cartesian_model(int dim, const int64_t* partition, const double* domain,
                        double* node_coords, int32_t* cell_node_ids, int32_t* node_entity);

/* Dof numbering of a nodal Lagrangian space whose nodes are the mesh nodes (Q1/P1, scalar
 * or ncomp components, node-major / component-interleaved). node_to_tag[nnodes] is the
 * get_face_tag_index result (0 = untagged), tag_masks[ntags*ncomp] the Dirichlet masks,
 * lnode_comp_to_ldof[nv*ncomp] the 1-based local dof of (local node, component).
 * Replaces FESpaces/CLagrangianFESpaces.jl:155-380. */
int gfe_clagrangian_dofs(int64_t nnodes, const int8_t* node_to_tag, int ncomp,
                         const uint8_t* tag_masks, int64_t ncells, int nv,
                         const int32_t* cell_node_ids, const int32_t* lnode_comp_to_ldof,
                         int32_t* node_comp_to_dof, int32_t* cell_dof_ids, int32_t* nfree,
                         int32_t* ndiri);

/* Conforming dof numbering of a Lagrangian space of order 2 (Q2: 9 nodes per QUAD, 27 per
 * HEX) on a Cartesian grid: topology edges and faces numbered first-touch over cells and
 * local faces, labels of every face from the domain box, dofs numbered dimension by dimension
 * (vertices, edges, faces, cell interiors) in face order with the components of a node
 * consecutive; Dirichlet dofs negative. entity_to_tag[3^dim] gives, per box entity, the
 * 1-based position of the first Dirichlet tag containing it (0 = none), tag_masks[ntags*ncomp]
 * the component masks. cell_dof_ids: ncells x (3^dim*ncomp), component-major over the nodes
 * in Gridap's local order (vertices, edges, faces, interior).
 * Replaces FESpaces/ConformingFESpaces.jl:367-636 with Geometry/GridTopologies.jl:1184-1250
 * and Geometry/CartesianDiscreteModels.jl:133-260. */
int gfe_cartesian_conforming_dofs(int dim, int order, const int64_t* partition, int ncomp,
                                  const int8_t* entity_to_tag, const uint8_t* tag_masks,
                                  int32_t* cell_dof_ids, int32_t* nfree, int32_t* ndiri);

/* ---- assembly: symbolic ------------------------------------------------------------------ */
/* Builds the sparsity pattern of the matrix that assembling cell matrices over
 * (cell_rows, cell_cols) produces: rows sorted, columns sorted and unique per row, entries
 * for every touched (row, col) pair of positive ids -- the pattern of Gridap's
 * SparseMatrixCSC/CSR after create_from_nz. Built on the device; *A receives a new matrix
 * with that pattern and zero values.
 * Replaces FESpaces/SparseMatrixAssemblers.jl:174-210 (symbolic_loop_matrix!) with
 * Algebra/SparseMatrixCSC.jl:214-283 (nz_counter / nz_allocation / create_from_nz). */
int gfe_symbolic_loop_matrix(gfe_ctx* ctx, int64_t ncells, int nd, const int32_t* cell_rows,
                             const int32_t* cell_cols, int64_t nrows, int64_t ncols,
                             gfe_matrix** A);
/* Releases the matrix (stream-ordered; no device synchronisation). Destroy every matrix of a
 * context before the context itself. */
int gfe_matrix_destroy(gfe_matrix* A);
int gfe_matrix_info(gfe_matrix* A, int64_t* nrows, int64_t* ncols, int64_t* nnz);
/* Copies the CSR arrays out (rowptr[nrows+1], colval[nnz], nzval[nnz]); index_base 0 or 1;
 * any output may be NULL. For the symmetric operators of this library CSR == CSC, so these
 * are also Gridap's SparseMatrixCSC colptr/rowval/nzval (index_base 1). */
int gfe_matrix_export_csr(gfe_matrix* A, int index_base, int64_t* rowptr, int64_t* colval,
                          double* nzval);
/* Zeroes the stored values, keeping the pattern (Gridap's fillstored!(A, 0) before
 * re-assembly, FESpaces/SparseMatrixAssemblers.jl:60-68). */
int gfe_matrix_fillstored_zero(gfe_matrix* A);

/* ---- assembly: numeric, caller-provided cell arrays --------------------------------------- */
/* Adds cell matrices (FP64, nd x nd column-major per cell, ncells of them, the layout of
 * Gridap's cell matrix arrays) into A's values in cell order -- rows outer by cell, i.e. the
 * exact accumulation order of InserterCSC -- skipping negative ids. A must come from
 * gfe_symbolic_loop_matrix over the same cell ids.
 * Replaces FESpaces/SparseMatrixAssemblers.jl:214-248 (numeric_loop_matrix!) and
 * Algebra/SparseMatrixCSC.jl:124-150 (InserterCSC.add_entry!). */
int gfe_numeric_loop_matrix(gfe_ctx* ctx, gfe_matrix* A, const double* cellmats);
/* b[i] += cellvecs[cell][li] for positive ids, in cell order; b has nrows entries and is
 * added to (zero it for a fresh assembly).
 * Replaces FESpaces/SparseMatrixAssemblers.jl:287-316 (numeric_loop_vector!). */
int gfe_numeric_loop_vector(gfe_ctx* ctx, int64_t ncells, int nd, const int32_t* cell_rows,
                            const double* cellvecs, int64_t nrows, double* b);

/* ---- assembly: fused integrate + assemble for recognised weak forms ----------------------- */
enum {
  GFE_REFFE_Q1 = 1, /* Lagrangian Q1 on QUAD/HEX, lexicographic nodes */
  GFE_REFFE_Q2 = 2  /* Lagrangian Q2 on QUAD/HEX (9/27 nodes: vertices, edges, faces, interior)
                       on (multi)linear cells given by node_coords + cell_node_ids (vertices) */
};
enum { GFE_GEOM_CARTESIAN = 0, GFE_GEOM_NODAL = 1 };
enum { GFE_FORM_DIFFUSION = 1 };                  /* a(u,v) = int kappa grad(v).grad(u) */
enum { GFE_COEF_ONE = 0, GFE_COEF_CONST = 1, GFE_COEF_CELL = 2 };
enum {
  GFE_SRC_NONE = 0,
  GFE_SRC_CONST = 1,  /* f = source[0] */
  GFE_SRC_NODAL = 2,  /* f = sum_a source[node_a] phi_a (an FE function on the mesh nodes) */
  GFE_SRC_QPOINT = 3, /* f(x_q) given per cell and quadrature point: source[cell*nq + q] */
  GFE_SRC_SINSUM = 4  /* f = sum_k a_k prod_d sin(pi m_kd x_d); source = [K, (a, m_1..m_D)*K] */
};
enum { GFE_PREC_FP64 = 0, GFE_PREC_FP32 = 1 };

typedef struct gfe_problem {
  int32_t dim;          /* 2 or 3 */
  int32_t reffe;        /* GFE_REFFE_* */
  int32_t ncomp;        /* 1 (scalar) */
  int32_t degree;       /* quadrature degree (Measure(trian, degree)) */
  int64_t ncells;
  int32_t nd;           /* dofs per cell */
  const int32_t* cell_dof_ids; /* ncells*nd, Gridap convention */
  int64_t nfree;
  /* geometry */
  int32_t geometry;     /* GFE_GEOM_* */
  int64_t partition[3]; /* Cartesian descriptor: cells per direction */
  double domain[6];     /* (x0, x1, y0, y1, z0, z1) */
  int64_t nnodes;
  const double* node_coords;   /* nnodes*dim (GFE_GEOM_NODAL) */
  const int32_t* cell_node_ids;/* ncells*2^dim, 1-based (GFE_GEOM_NODAL, GFE_SRC_NODAL) */
  /* weak form */
  int32_t form;         /* GFE_FORM_* */
  int32_t coef_kind;    /* GFE_COEF_* */
  const double* coef;   /* kappa (1 value or ncells values) */
  int32_t source_kind;  /* GFE_SRC_* */
  const double* source;
  int64_t source_len;   /* number of doubles at `source` */
  int32_t precision;    /* GFE_PREC_*: arithmetic of the cell integrals (scatter stays FP64);
                           FP32 on Q2 uses the tensor cores (TF32 operands, FP32 accumulate,
                           FP64 Jacobians) */
} gfe_problem;

/* Integrates the recognised bilinear and linear forms over every cell and assembles them
 * into A (pattern from gfe_symbolic_loop_matrix over problem->cell_dof_ids) and b (nfree
 * entries, overwritten). A or b may be NULL to skip one. Dirichlet values are zero, so the
 * lift of AttachDirichlet leaves b unchanged.
 * Replaces the cell-array evaluation that Gridap's numeric loops trigger
 * (CellData/CellQuadratures.jl:138-170, Fields/FieldsInterfaces.jl:708-720,
 * Fields/ApplyOptimizations.jl:293-310) together with numeric_loop_matrix_and_vector!
 * (FESpaces/SparseMatrixAssemblers.jl:365-405). */
int gfe_assemble_matrix_and_vector(gfe_ctx* ctx, const gfe_problem* problem, gfe_matrix* A,
                                   double* b);

/* ---- linear solve ------------------------------------------------------------------------ */
enum { GFE_SOLVER_CG = 0, GFE_SOLVER_IR_CG = 1, GFE_SOLVER_MIXED_CG = 2 };
enum { GFE_PC_NONE = 0, GFE_PC_JACOBI = 1 };

typedef struct gfe_solver_opts {
  int32_t method;       /* GFE_SOLVER_CG: FP64 PCG; GFE_SOLVER_IR_CG: FP32 inner PCG inside
                           FP64 iterative refinement (restarted per refinement step);
                           GFE_SOLVER_MIXED_CG: FP32 PCG with FP64 reliable updates (x and the
                           true residual in FP64, search direction kept) */
  int32_t precond;      /* GFE_PC_* */
  double rtol;          /* stop when ||b - A x||_2 <= rtol ||b||_2 (FP64 residual) */
  int32_t maxiter;      /* total inner iterations allowed */
  double inner_rtol;    /* IR_CG: relative reduction per refinement step; MIXED_CG: residual
                           reduction between reliable updates (default 0.1) */
  int32_t check_every;  /* iterations between host convergence checks (0 = default) */
} gfe_solver_opts;

typedef struct gfe_solve_report {
  int32_t iterations;       /* inner (Krylov) iterations */
  int32_t refinements;      /* FP64 refinement steps (IR-CG) or reliable updates (MIXED_CG) */
  int32_t converged;        /* 1 when the FP64 residual met rtol */
  int32_t status;           /* GFE_OK or the code that stopped the solver */
  double relres;            /* final ||b - A x|| / ||b|| in FP64, recomputed after the solve */
  int32_t operator_format;  /* SpMV format of the (inner) operator: 0 sliced ELL, 1 diagonal */
  int32_t ndiag;            /* diagonals of the diagonal format (0 otherwise) */
} gfe_solve_report;

/* Solves A x = b. Replaces the LinearSolver protocol's numerical_setup + solve!
 * (Algebra/LinearSolvers.jl:58-129,202-209) for a CG-family solver; Gridap ships no Krylov
 * solver, so this is the LinearSolver a user plugs in there. x need not be initialised. */
int gfe_solve(gfe_ctx* ctx, gfe_matrix* A, const gfe_solver_opts* opts, const double* b,
              double* x, gfe_solve_report* report);

/* y = A x in FP64 (Gridap's mul!(y, A, x) on the assembled matrix; used for residuals). */
int gfe_matrix_mul(gfe_ctx* ctx, gfe_matrix* A, const double* x, double* y);

/* ---- allocation-free solve ----------------------------------------------------------------- */
/* FP64 Jacobi-preconditioned CG (x0 = 0, stop on ||b - A x|| <= rtol ||b||) on a matrix the
 * caller holds in device memory as 0-based CSR (rowptr[n+1], colval[nnz], val[nnz]), with b
 * and x in device memory too. It allocates no device memory at all: for callers that cannot
 * call cudaMalloc -- applications whose device memory is owned by their own pool or arena
 * (e.g. a Julia CUDA.jl pool, or a code that allocates once at start-up and must not
 * allocate while it runs). Its work vectors live in a fixed static device array sized for
 * n <= 524,288 rows (about 16 MB held by every GPU that loads the library); larger n is
 * rejected with GFE_ERR_INVALID_ARGUMENT. The first call on a device looks up that array's
 * address (once per device); make it before any stream capture. All calls share the array:
 * calls that overlap on the GPU race. Work is ordered on `stream` (a cudaStream_t, NULL for
 * the default stream) and complete on return.
 * No counterpart in Gridap: it is an extra entry point of this library. */
int gfe_cg_solve_noalloc(const int32_t* rowptr, const int32_t* colval, const double* val,
                         int64_t n, int64_t nnz, const double* b, double* x, double rtol,
                         int32_t maxiter, void* stream, int32_t* iterations, double* relres);

#ifdef __cplusplus
}
#endif
#endif
