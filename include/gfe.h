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
  GFE_ERR_TIMEOUT = 6,         /* a bounded device-side wait ran out (the kernel waited for
                                  its copies in flight, bounded again, before it returned; if
                                  that wait also ran out, destroy the context) */
  GFE_ERR_UNSUPPORTED = 7,     /* element / form / option combination not provided */
  GFE_ERR_NONFINITE = 8,       /* NaN or Inf in coefficients, matrix or vectors */
  GFE_ERR_NOT_CONVERGED = 9    /* gfe_cg_solve_noalloc: maxiter reached above rtol */
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
  GFE_KT_ELEMENT = 4,    /* element (cell-integral) kernels */
  GFE_KT_PRECOND = 5,    /* learned block preconditioner (MLP on tensor cores + gather) */
  GFE_KT_VECTOR = 6      /* CG vector updates of one iteration (update + direction kernels) */
};
int gfe_ctx_set_timing(gfe_ctx* ctx, int enable);
int gfe_ctx_kernel_time(gfe_ctx* ctx, int kernel, double* total_ms, int64_t* launches);
/* Limit (ns, default 1e9) of the first bounded wait on the tensor-copy barrier of the lattice
 * SpMV. When it runs out the kernel records GFE_ERR_TIMEOUT, waits again (bounded, 1 s) for
 * its copies to land, skips its tile and the solve returns GFE_ERR_TIMEOUT; the context stays
 * usable. 0 makes the first wait give up at once: a switch for tests of that path, off by
 * default. No counterpart in Gridap. */
int gfe_ctx_set_wait_limit(gfe_ctx* ctx, uint64_t first_wait_ns);

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

/* simplexify(CartesianDiscreteModel((0,1)^3-like box, partition)) connectivity: tet 6c+t of
 * hexahedron c has the hexahedron's nodes at the t-th local tet of the oriented 3-cube
 * simplexification (1-based node ids, ntets*4).
 * Replaces Geometry/Grids.jl:487-558 with ReferenceFEs/ExtrusionPolytopes.jl:290-299. */
int gfe_simplex_model(const int64_t* partition, int32_t* tet_vertex_ids);
/* Conforming P2 dof numbering on that simplexified box: vertices first (vertex order), then
 * edges in first-touch order over (tet, local edge), the components of a node consecutive;
 * a vertex or edge is Dirichlet for the components in comp_mask[ncomp] when all its
 * vertices carry vertex_mask (the labeling face_labeling_from_vertex_filter builds).
 * cell_dof_ids: ntets x (10*ncomp), component-major over the 10 local nodes.
 * Replaces FESpaces/ConformingFESpaces.jl:367-636 with Geometry/GridTopologies.jl:1184-1250,
 * Geometry/UnstructuredDiscreteModels.jl:85-200 and Geometry/FaceLabelings.jl:590-611. */
int gfe_simplex_p2_dofs(const int64_t* partition, int32_t ncomp, const uint8_t* vertex_mask,
                        const uint8_t* comp_mask, int32_t* cell_dof_ids, int32_t* nfree,
                        int32_t* ndiri);

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
/* The same for rectangular cell blocks: nd_rows row ids and nd_cols column ids per cell (an
 * off-diagonal block of a multi-field system, e.g. velocity rows against pressure columns).
 * Replaces the per-block symbolic loops of MultiField/BlockSparseMatrixAssemblers.jl:
 * 197-230 (nz_counter / nz_allocation / create_from_nz over the block builders), each block
 * being FESpaces/SparseMatrixAssemblers.jl:174-210 on its (rows, cols) id pair. */
int gfe_symbolic_loop_matrix_rect(gfe_ctx* ctx, int64_t ncells, int nd_rows, int nd_cols,
                                  const int32_t* cell_rows, const int32_t* cell_cols,
                                  int64_t nrows, int64_t ncols, gfe_matrix** A);
/* The same with a local coupling mask: local_mask[li + lj*nd_rows] (nd_rows x nd_cols bytes,
 * host or device) zero drops every (cell_rows[c][li], cell_cols[c][lj]) touch, as for a
 * negative id. A multi-field cell matrix is an ArrayBlock whose untouched blocks (field pairs
 * the weak form does not couple) are `nothing` and add no entry to the pattern
 * (MultiField/MultiFieldFESpaces.jl:460-480, the touched flags of Arrays/ArrayBlocks.jl:23-45);
 * the mask is that block structure at local-dof resolution. */
int gfe_symbolic_loop_matrix_masked(gfe_ctx* ctx, int64_t ncells, int nd_rows, int nd_cols,
                                    const int32_t* cell_rows, const int32_t* cell_cols,
                                    const uint8_t* local_mask, int64_t nrows, int64_t ncols,
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
/* Adds cell matrices (FP64, nd x nd column-major per cell -- nd_rows x nd_cols for a matrix
 * from gfe_symbolic_loop_matrix_rect -- ncells of them, the layout of Gridap's cell matrix
 * arrays) into A's values in cell order -- rows outer by cell, i.e. the
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
  GFE_REFFE_Q2 = 2, /* Lagrangian Q2 on QUAD/HEX (9/27 nodes: vertices, edges, faces, interior)
                       on (multi)linear cells given by node_coords + cell_node_ids (vertices) */
  GFE_REFFE_P2_TET = 3 /* Lagrangian P2 on TET (10 nodes: vertices, then the midpoints of the
                          TET edges 12, 13, 23, 14, 24, 34), vector-valued (ncomp 3, local dofs
                          component-major); cells are the tets of simplexify(Cartesian box)
                          (GFE_GEOM_CARTESIAN: tet 6c+t of hexahedron c) or affine tets given
                          by node_coords + cell_node_ids (4 vertices, GFE_GEOM_NODAL) */
};
enum { GFE_GEOM_CARTESIAN = 0, GFE_GEOM_NODAL = 1 };
enum {
  GFE_FORM_DIFFUSION = 1,  /* a(u,v) = int kappa grad(v).grad(u),  l(v) = int f v */
  GFE_FORM_ELASTICITY = 2, /* a(u,v) = int eps(v) : (lambda tr(eps(u)) I + 2 mu eps(u)),
                              l(v) = int f . v; coef = (lambda, mu) once (CONST) or per cell
                              (CELL, 2 values per cell); source CONST with 3 values (f) */
  GFE_FORM_QUASILINEAR = 3 /* residual r(u; v) = int kappa alpha(u, grad u) grad u . grad v
                              - f v and its Jacobian at the state u (problem->state plus the
                              Dirichlet values): A receives the Jacobian, b the residual.
                              alpha is problem->law (GFE_LAW_*) with problem->law_params;
                              kappa = coef (ONE, CONST or CELL); f = source (NONE, CONST,
                              QPOINT). Scalar Q1/Q2, node coordinates required. */
};
enum {
  GFE_LAW_POLY = 0,  /* alpha = c0 + c1 u + c2 u^2 (law_params c0, c1, c2) */
  GFE_LAW_POWER = 1  /* alpha = (eps2 + |grad u|^2)^((p-2)/2) (law_params p, eps2): the
                        p-Laplacian flux |grad u|^(p-2) grad u for eps2 = 0 */
};
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
  int32_t ncomp;        /* 1 (scalar); 3 for GFE_FORM_ELASTICITY */
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
  const double* coef;   /* kappa (1 value or ncells values); (lambda, mu) for elasticity */
  int32_t source_kind;  /* GFE_SRC_* */
  const double* source;
  int64_t source_len;   /* number of doubles at `source` */
  int32_t precision;    /* GFE_PREC_*: arithmetic of the cell integrals (scatter stays FP64);
                           FP32 on Q2 uses the tensor cores (TF32 operands, FP32 accumulate,
                           FP64 Jacobians) */
  /* Dirichlet data of the trial space (TrialFESpace(V, u_D)): the value of Dirichlet dof -k
     at dirichlet_values[k-1], host or device; NULL (or ndirichlet = 0) for u_D = 0. With it,
     every cell (and facet) vector receives the lift  b_i -= sum_j A_ij u_D_j  over the cell's
     Dirichlet columns j before it is added (AttachDirichletMap, CellData/AttachDirichlet.jl:
     59-110, applied per triangulation in FESpaces/Assemblers.jl:525-542). */
  const double* dirichlet_values;
  int64_t ndirichlet;
  /* GFE_FORM_QUASILINEAR: the free values of the state u (nfree entries, host or device),
     the law and its parameters */
  const double* state;
  int32_t law;
  double law_params[4];
} gfe_problem;

/* The symbolic loop of problem->cell_dof_ids (rows and columns, nfree x nfree), with what the
 * assembler knows about the model: for Q1 hexahedra of a Cartesian grid (dim 3, partition)
 * whose ids are the interior-node numbering (checked on the device) the pattern, row
 * references and position table are written in closed form -- the same arrays, bit for bit,
 * that gfe_symbolic_loop_matrix computes, which it falls back to for any other ids.
 * Replaces FESpaces/SparseMatrixAssemblers.jl:174-210 with the assembler's spaces in hand
 * (SparseMatrixAssembler(U, V) holds the FE spaces and their model). */
int gfe_symbolic_loop_matrix_problem(gfe_ctx* ctx, const gfe_problem* problem, gfe_matrix** A);

/* Integrates the recognised bilinear and linear forms over every cell and assembles them
 * into A (pattern from gfe_symbolic_loop_matrix over problem->cell_dof_ids) and b (nfree
 * entries, overwritten). A or b may be NULL to skip one. With problem->dirichlet_values the
 * cell vectors carry the Dirichlet lift (b_i -= sum_j K_ij u_D_j); without, u_D = 0 and the
 * lift leaves b unchanged.
 * Replaces the cell-array evaluation that Gridap's numeric loops trigger
 * (CellData/CellQuadratures.jl:138-170, Fields/FieldsInterfaces.jl:708-720,
 * Fields/ApplyOptimizations.jl:293-310) together with numeric_loop_matrix_and_vector!
 * (FESpaces/SparseMatrixAssemblers.jl:365-405). */
int gfe_assemble_matrix_and_vector(gfe_ctx* ctx, const gfe_problem* problem, gfe_matrix* A,
                                   double* b);

/* ---- assembly: boundary terms (Neumann, Nitsche, Robin) ---------------------------------- */
/* Boundary integrals over facets of a Cartesian box, scalar Q1/Q2 (problem: dim, reffe,
 * partition, domain, cell_dof_ids, nd, nfree). The facets lie on the box `domain` with the
 * partition's spacing (also for a Cartesian model whose interior nodes are jittered, as
 * boundary nodes stay in place). Facet f belongs to cell facet_cells[f] (0-based) as its
 * local facet facet_lfaces[f] (0-based, Gridap's face order of the D-cube: z-, z+, y-, y+,
 * x-, x+ in 3-D; y-, y+, x-, x+ in 2-D); facets are added in the given order, each with its
 * owner cell's dof ids (Gridap's BoundaryTriangulation order is ascending facet id). The
 * facet rule is the tensor Gauss rule of `degree` on the facet, n the outward unit normal.
 * Replace the cell arrays of a BoundaryTriangulation measure
 * (Geometry/BoundaryTriangulations.jl:13-35,150-205, CellData/CellQuadratures.jl:138-170)
 * and their numeric loops (FESpaces/SparseMatrixAssemblers.jl:214-316). */
enum {
  GFE_BOP_VALUE = 0,       /* test function v */
  GFE_BOP_NORMAL_GRAD = 1  /* n . grad(v) */
};

/* b += int_Gamma g op(v) dGamma. g is constant (GFE_SRC_CONST, 1 value) or given at the
 * facet's Gauss points (GFE_SRC_QPOINT, nfacets * npoints values, facet by facet; facet
 * coordinates = the spanned axes in increasing order, the first fastest). test_op is a
 * GFE_BOP_*. b (nfree entries, host or device) is added to. */
int gfe_assemble_boundary_vector(gfe_ctx* ctx, const gfe_problem* problem, int64_t nfacets,
                                 const int32_t* facet_cells, const int32_t* facet_lfaces,
                                 int32_t degree, int32_t test_op, int32_t source_kind,
                                 const double* source, int64_t source_len, double* b);

/* A += int_Gamma c0 v u + c1 v (n.grad u) + c2 (n.grad v) u + c3 (n.grad v)(n.grad u) dGamma,
 * coefs = (c0, c1, c2, c3) constants (Nitsche: (gamma/h, -1, -1, 0); Robin: (alpha, 0, 0, 0)).
 * A is an assembled matrix whose pattern covers the owner cells' dof pairs (the volume
 * pattern does); its values are added to in facet order per entry. With
 * problem->dirichlet_values and b (nfree entries, host or device, may be NULL), b receives
 * the facets' Dirichlet lift b_i -= sum_j M_ij u_D_j. */
int gfe_assemble_boundary_matrix(gfe_ctx* ctx, const gfe_problem* problem, gfe_matrix* A,
                                 double* b, int64_t nfacets, const int32_t* facet_cells,
                                 const int32_t* facet_lfaces, int32_t degree,
                                 const double* coefs);

/* ---- free-dof reordering ------------------------------------------------------------------ */
/* iperm[old-1] = new (1-based) for the free dofs of cell_dof_ids (Gridap convention, host or
 * device), as compute_dof_permutation (FESpaces/FESpaceReindexing.jl:264-300) returns it:
 * GFE_REORDER_RCM, Reverse Cuthill-McKee with George-Liu pseudo-peripheral nodes; or
 * GFE_REORDER_SLOAN with weights w1, w2 (Gridap's defaults 1, 2). iperm is host memory.
 * Applying it: new cell ids = iperm[id-1] for id > 0 (reindex_free_dof_ids). */
enum { GFE_REORDER_RCM = 0, GFE_REORDER_SLOAN = 1 };
int gfe_dof_permutation(gfe_ctx* ctx, int64_t ncells, int32_t nd, const int32_t* cell_dof_ids,
                        int64_t nfree, int32_t algorithm, int32_t w1, int32_t w2,
                        int64_t* iperm);

/* ---- multi-field assembly (MultiFieldFESpace, block assemblers) --------------------------- */
/* Operators applied to a field's basis inside an integrand. */
enum {
  GFE_MOP_VALUE = 0, /* u (scalar) or u (vector: the basis e_c phi) */
  GFE_MOP_GRAD = 1,  /* grad u: a vector (scalar field) or a dim x dim tensor (vector field) */
  GFE_MOP_DIV = 2    /* div u of a vector field: a scalar */
};

/* One Lagrangian field on the common cells: ncomp components (1, or dim with the cell's
 * local dofs component-major: comp * nnodes + node), tabulated on the reference cell at the
 * problem's quadrature points. */
typedef struct gfe_mf_field {
  int32_t ncomp;
  int32_t nnodes;           /* local nodes per cell */
  const double* shapes;     /* nq x nnodes reference shape values */
  const double* grads;      /* nq x nnodes x dim reference gradients */
} gfe_mf_field;

/* One term of the integrand, summed over the quadrature points with weight w_q |J_q|:
 * bilinear (trial_field >= 0): coef * op_test(v) . op_trial(u), the dot product being the
 *   full contraction of two operands of the same shape (scalar x scalar, vector . vector,
 *   tensor : tensor), e.g. grad(v) : grad(u), -(div v) p, q (div u), v . grad(p);
 * linear (trial_field = -1): coef * op_test(v) . f(x_q) with f from qdata (ncells x nq x
 *   qdata_ncomp values, host or device, matching op_test's shape) or f = 1 when qdata is
 *   NULL.
 * cell_coef (ncells values, host or device, or NULL) scales the term cell by cell. */
typedef struct gfe_mf_term {
  int32_t test_field, trial_field;
  int32_t test_op, trial_op;
  double coef;
  const double* cell_coef;
  const double* qdata;
  int32_t qdata_ncomp;
} gfe_mf_term;

typedef struct gfe_mf_problem {
  int32_t dim;                  /* 2 or 3 */
  int64_t ncells;
  int64_t nnodes;
  const double* node_coords;    /* nnodes x dim */
  const int32_t* cell_node_ids; /* ncells x 2^dim, 1-based: the (multi)linear cell map */
  int32_t nq;                   /* quadrature points per cell */
  const double* qweights;       /* nq reference weights */
  const double* geo_grads;      /* nq x 2^dim x dim gradients of the cell map's Q1 shapes */
  int32_t nfields;
  const gfe_mf_field* fields;
  int32_t nterms;
  const gfe_mf_term* terms;
} gfe_mf_problem;

/* Integrates the terms on every cell and assembles the block (rows of row_fields against
 * columns of col_fields, each a list of field indices) into A and/or b:
 *  - A (may be NULL) comes from gfe_symbolic_loop_matrix(_rect) over the cell ids of the row
 *    fields (concatenated in row_fields order) and of the column fields; the cell matrix of
 *    the block is ndr x ndc with ndr = sum over row fields of ncomp * nnodes;
 *  - b (may be NULL; nrows entries -- A's rows when A is given -- added to) receives the
 *    linear terms of the row fields;
 *  - row_ids / col_ids are those concatenated cell ids (ncells x ndr, ncells x ndc), in the
 *    numbering A was built with; negative ids are Dirichlet dofs, -k reading
 *    dirichlet_values[k-1] (host or device, NULL: zero) for the lift b_i -= sum_j K_ij u_D_j.
 * One monolithic matrix (ConsecutiveMultiFieldStyle) is the block of all fields against all
 * fields; a block assembler calls this once per block.
 * Replaces the multi-field cell arrays (MultiField/MultiFieldCellFields.jl, BlockMap cell
 * matrices of MultiField/MultiFieldFESpaces.jl:460-488) and their assembly through
 * FESpaces/SparseMatrixAssemblers.jl:214-316 per block
 * (MultiField/BlockSparseMatrixAssemblers.jl:236-255). */
int gfe_multifield_assemble(gfe_ctx* ctx, const gfe_mf_problem* problem, int32_t nrow_fields,
                            const int32_t* row_fields, int32_t ncol_fields,
                            const int32_t* col_fields, const int32_t* row_ids,
                            const int32_t* col_ids, const double* dirichlet_values,
                            int64_t ndirichlet, gfe_matrix* A, int64_t nrows, double* b);

/* ---- linear solve ------------------------------------------------------------------------ */
enum {
  GFE_SOLVER_CG = 0,
  GFE_SOLVER_IR_CG = 1,
  GFE_SOLVER_MIXED_CG = 2,
  GFE_SOLVER_BICGSTAB = 3  /* FP64 BiCGStab, Jacobi (right) preconditioner: non-symmetric A */
};
enum {
  GFE_PC_NONE = 0,
  GFE_PC_JACOBI = 1,
  GFE_PC_MG = 2  /* gfe_solve_fcg without a learned pc: geometric multigrid V-cycle on the
                    lattice operator (uniform Cartesian Q1 in 3-D; FP32, damped Jacobi
                    smoothing, trilinear transfers, kappa averaged to coarse cells) */
};

typedef struct gfe_solver_opts {
  int32_t method;       /* GFE_SOLVER_CG: FP64 PCG; GFE_SOLVER_IR_CG: FP32 inner PCG inside
                           FP64 iterative refinement (restarted per refinement step);
                           GFE_SOLVER_MIXED_CG: FP32 PCG with FP64 reliable updates (x and the
                           true residual in FP64, search direction kept) */
  int32_t precond;      /* GFE_PC_* */
  double rtol;          /* stop when ||b - A x||_2 <= rtol ||b||_2 (FP64 residual) */
  int32_t maxiter;      /* total inner iterations allowed */
  double inner_rtol;    /* IR_CG: relative reduction per refinement step; MIXED_CG: residual
                           reduction between reliable updates (default 0.01); FCG: the same
                           (default 0.1, 1e-4 with GFE_PC_MG) */
  int32_t check_every;  /* iterations between host convergence checks (0 = default) */
  int32_t initial_guess;/* 0: start from x = 0; 1: start from the values in x (a restart from a
                           saved solution): the solver runs on A d = b - A x0 with its tolerance
                           scaled to ||b||, then x = x0 + d */
} gfe_solver_opts;

typedef struct gfe_solve_report {
  int32_t iterations;       /* inner (Krylov) iterations */
  int32_t refinements;      /* FP64 refinement steps (IR-CG) or reliable updates (MIXED_CG) */
  int32_t converged;        /* 1 when the FP64 residual met rtol */
  int32_t status;           /* GFE_OK or the code that stopped the solver */
  double relres;            /* final ||b - A x|| / ||b|| in FP64, recomputed after the solve */
  int32_t operator_format;  /* SpMV format of the (inner FP32) operator: 0 sliced ELL,
                               1 diagonal, 2 matrix-free (uniform Cartesian Q1 diffusion with
                               rows = interior nodes in node order: per-cell kappa times the
                               reference stiffness, applied cell-wise in FP32) */
  int32_t ndiag;            /* diagonals of the diagonal format, 27 for matrix-free, else 0 */
  int32_t fallback;         /* 1 when a learned preconditioner stagnated and Jacobi took over */
} gfe_solve_report;

/* Solves A x = b. Replaces the LinearSolver protocol's numerical_setup + solve!
 * (Algebra/LinearSolvers.jl:58-129,202-209) for a CG-family solver; Gridap ships no Krylov
 * solver, so this is the LinearSolver a user plugs in there. x need not be initialised. */
int gfe_solve(gfe_ctx* ctx, gfe_matrix* A, const gfe_solver_opts* opts, const double* b,
              double* x, gfe_solve_report* report);

/* y = A x in FP64 (Gridap's mul!(y, A, x) on the assembled matrix; used for residuals). */
int gfe_matrix_mul(gfe_ctx* ctx, gfe_matrix* A, const double* x, double* y);

/* ---- batched problems -------------------------------------------------------------------- */
/* Many independent scalar Q1 diffusion problems -div(kappa grad u) = f on unit cubes with
 * their own partitions (partitions[3*p..3*p+2], equal entries: cubic cells, n <= 1024), per-cell
 * kappa (concatenated in problem and Gridap cell order), homogeneous Dirichlet on the boundary,
 * assembled and solved together in ONE persistent kernel launch. Each problem runs a whole
 * Jacobi-PCG with the operator applied matrix-free in FP32 from the cell coefficients and
 * FP64 reliable updates (the FP64 true residual b - A x decides convergence:
 * ||b - A x|| <= rtol ||b|| in FP64). Thread-block clusters of 2-8 CTAs take the large
 * problems from a work counter, largest first, and solve each together; once those are
 * gone every CTA takes the smaller problems from a second counter and solves each alone.
 * Nothing waits on another group. The schedule (threads per CTA, CTAs per cluster, and the
 * size, relative to the largest problem, from which a problem goes to a cluster) is
 * autotuned on the first solve of a batch, which runs once with each of eight candidates.
 * Repeated calls give identical results.
 * No counterpart in Gridap (which solves one operator at a time). */
typedef struct gfe_batch gfe_batch;
int gfe_batch_create(gfe_ctx* ctx, int32_t nproblems, const int64_t* partitions,
                     const double* kappa, gfe_batch** batch);
int gfe_batch_destroy(gfe_batch* batch);
/* nrows = nfree = sum over problems of (n - 1)^3; ncells = sum of n^3. */
int gfe_batch_info(gfe_batch* batch, int64_t* nrows, int64_t* nfree, int64_t* ncells);
/* The schedule the autotuner chose (0, 0, 0 before the first solve): threads per CTA, CTAs
 * per cluster, and the cluster threshold (problems with at least that fraction of the largest
 * problem's rows go to clusters; 0: all of them). */
int gfe_batch_shape(gfe_batch* batch, int32_t* threads, int32_t* ctas_per_problem,
                    double* cluster_threshold);
/* Fixes the schedule to one of the candidates (256,1,0) (1024,1,0) (1024,2,0) (512,4,0)
 * (512,4,0.3) (1024,4,0.3) (1024,8,0) (1024,8,0.3) instead of autotuning; (0, 0, 0)
 * re-enables the autotuner. Schedules sum in different orders: a fixed one makes results
 * reproducible across batches. */
int gfe_batch_set_shape(gfe_batch* batch, int32_t threads, int32_t ctas_per_problem,
                        double cluster_threshold);
/* x (host, or device memory of the context's device) receives the problems' free-dof
 * solutions one after the other (sum of nfree entries); iterations[nproblems] (optional, host)
 * each problem's CG iterations; *nconverged how many reached rtol within maxiter (0 = 100000). */
int gfe_batch_assemble_solve(gfe_batch* batch, double source, double rtol, int32_t maxiter,
                             double* x, int32_t* iterations, int32_t* nconverged);

/* ---- learned block preconditioner + flexible CG -------------------------------------------- */
/* A preconditioner for 3-D Q1 problems on Cartesian grids: the cells are grouped in 2x2x2
 * blocks (27 nodes, neighbouring blocks share face nodes) and a small MLP (35 -> 64 -> 64 ->
 * 27, BF16 weights, FP32 accumulation on the tensor cores) maps each block's residual patch
 * (RMS-normalised) and its log-kappa pattern to an approximation of the block's local solve;
 * the block results are averaged at shared nodes. node_to_dof[nnodes] is the Q1 space's node
 * numbering (Gridap convention), kappa_cell[ncells] the cell coefficients.
 * No counterpart in Gridap: a LinearSolver preconditioner that a user plugs in. */
typedef struct gfe_learned_pc gfe_learned_pc;
int gfe_learned_pc_create(gfe_ctx* ctx, const int64_t* partition, const double* domain,
                          const int32_t* node_to_dof, int64_t nfree, const double* kappa_cell,
                          gfe_learned_pc** pc);
int gfe_learned_pc_destroy(gfe_learned_pc* pc);
/* Number of FP32 parameters: W1[48][64] | b1[64] | W2[64][64] | b2[64] | W3[64][32] | b3[32]. */
int gfe_learned_pc_num_params(void);
int gfe_learned_pc_set_weights(gfe_learned_pc* pc, const float* params);
int gfe_learned_pc_get_weights(gfe_learned_pc* pc, float* params);
/* z = M(r) for FP32 device vectors (for tests and custom solvers). */
int gfe_learned_pc_apply(gfe_learned_pc* pc, const float* r, float* z);
/* Training samples from an FP64 residual r (host or device) of A: for each listed block, the
 * network input (48 floats) and the target (32 floats): the block's local solve
 * A_b^{-1} r_b in FP64, in the network's normalised units. X and T are device arrays. */
int gfe_learned_pc_samples(gfe_learned_pc* pc, gfe_matrix* A, const double* r,
                           int64_t nsamples, const int64_t* block_ids, float* X, float* T);
/* Training samples from a residual / error pair of the method's own FP64 iterations: r = b - A x
 * and e = x* - x (x* the FP64 solution; both FP64, host or device, nfree entries): for each
 * listed block the network input (48 floats, as above) and the target e_b (32 floats) in the
 * network's units. The targets a smoother of the V-cycle learns. X and T are device arrays.
 * No counterpart in Gridap. */
int gfe_learned_pc_samples_error(gfe_learned_pc* pc, const double* r, const double* e,
                                 int64_t nsamples, const int64_t* block_ids, float* X, float* T);
/* Adam on the mean squared error over (X, T) (device, n rows), `epochs` passes of minibatches
 * of `batch` rows; initialises the weights when the pc has none. *loss = last epoch's mean. */
int gfe_learned_pc_train(gfe_learned_pc* pc, const float* X, const float* T, int64_t n,
                         int32_t epochs, int32_t batch, float lr, uint64_t seed, float* loss);
/* Flexible CG (FCG(1)) with FP32 vectors and FP64 reliable updates, preconditioned by
 *  - the geometric multigrid V-cycle on the lattice operator (opts->precond == GFE_PC_MG;
 *    GFE_ERR_UNSUPPORTED without the lattice form), whose fine-level smoother is the learned
 *    block preconditioner when pc != NULL (pre-smoothing x = M(b), post-smoothing
 *    x += M(b - A x); coarser levels damped Jacobi),
 *  - the learned block preconditioner alone (pc != NULL, another precond), or
 *  - Jacobi.
 * A learned preconditioner that stagnates (less than a 4x residual drop per 10 iterations,
 * twice in a row) hands over to Jacobi (report->fallback = 1). opts->inner_rtol is the
 * residual reduction between reliable updates; stops on the FP64 relative residual. */
int gfe_solve_fcg(gfe_ctx* ctx, gfe_matrix* A, gfe_learned_pc* pc, const gfe_solver_opts* opts,
                  const double* b, double* x, gfe_solve_report* report);

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
 * Stopping: the iteration stops on the recursively updated residual; the true residual
 * ||b - A x|| is then recomputed and CG restarts from x (at most 3 times, within maxiter)
 * while it is above rtol ||b||. *relres is that true relative residual. Returns GFE_OK when
 * it meets rtol, GFE_ERR_NOT_CONVERGED when maxiter ran out first (x holds the last iterate),
 * GFE_ERR_NONFINITE when b, the matrix or a reduction is NaN or Inf; pointers into another
 * GPU's memory are rejected with GFE_ERR_INVALID_ARGUMENT.
 * No counterpart in Gridap: it is an extra entry point of this library. */
int gfe_cg_solve_noalloc(const int32_t* rowptr, const int32_t* colval, const double* val,
                         int64_t n, int64_t nnz, const double* b, double* x, double rtol,
                         int32_t maxiter, void* stream, int32_t* iterations, double* relres);

#ifdef __cplusplus
}
#endif
#endif
