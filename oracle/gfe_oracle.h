/*
 * gfe_oracle.h -- TEST INFRASTRUCTURE ONLY (the oracle), not part of the product.
 *
 * A plain-C, CPU restatement of Gridap.jl v0.20.8's cell-wise finite-element assembly and
 * linear solve, for the element/geometry/weak-form combinations the GPU library covers.
 * Every function cites the Gridap source it follows (paths relative to the Gridap project).
 *
 * Only the test suite, the smoke check and the benchmark's CPU-baseline / reference legs may
 * load this library, and only as the checker or the timed CPU baseline; the product path
 * never calls it.
 *
 * Conventions (Gridap's):
 *   - node, cell and dof ids are 1-based; Dirichlet dofs are negative (-1, -2, ...);
 *   - cell arrays are column-major per cell (cellmat[c][i + j*nd], i = test/row, j = trial/col);
 *   - the assembled matrix is a SparseMatrixCSC{Float64,Int64}: 1-based colptr/rowval.
 */
#ifndef GFE_ORACLE_H
#define GFE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- polytopes ---------------------------------------------------------------------- */
/* Faces of the D-cube in Gridap's order (ReferenceFEs/ExtrusionPolytopes.jl:460-531).
 * Writes 3^D faces as (extrusion[D], anchor[D]) pairs; returns the number of faces. */
int orc_ncube_faces(int D, int32_t* ext, int32_t* anchor);

/* ---- Cartesian model (Geometry/CartesianGrids.jl:108-171, CartesianDiscreteModels.jl) -- */
void orc_cartesian_coords(int D, const int64_t* partition, const double* domain, double* coords);
void orc_cartesian_cell_nodes(int D, const int64_t* partition, int32_t* cell_nodes);
/* Box entity (1-based, n-cube face id) of every node: the labels Gridap's Cartesian face
 * labeling gives the vertices (Geometry/CartesianDiscreteModels.jl:133-189). */
void orc_cartesian_node_entity(int D, const int64_t* partition, int32_t* node_entity);
/* get_face_tag_index for d=0 (Geometry/FaceLabelings.jl:411-427): tags given as entity
 * lists tag_ptrs[ntags+1] (0-based offsets), tag_entities[]. UNSET = 0. */
void orc_node_tag_index(int64_t nnodes, const int32_t* node_entity, int ntags,
                        const int32_t* tag_ptrs, const int32_t* tag_entities, int8_t* node_to_tag);

/* ---- jittered Cartesian nodes (synthetic geometry for distorted-cell configurations) ---- */
/* coords += jitter on nodes that are not on the domain boundary (per node, D values). */
void orc_jitter_interior(int D, const int64_t* partition, const double* jitter, double* coords);

/* ---- CLagrangian dof numbering (FESpaces/CLagrangianFESpaces.jl:155-380) --------------- */
/* node_to_tag[nnodes] (0 = UNSET), tag_masks[ntags*ncomp]; lnode_comp_to_ldof[nv*ncomp]
 * (1-based local dof of (local node, comp)). Outputs node_comp_to_dof[nnodes*ncomp],
 * cell_dofs[ncells*nv*ncomp]. */
void orc_clagrangian_numbering(int64_t nnodes, const int8_t* node_to_tag, int ncomp,
                               const uint8_t* tag_masks, int64_t ncells, int nv,
                               const int32_t* cell_nodes, const int32_t* lnode_comp_to_ldof,
                               int32_t* node_comp_to_dof, int32_t* cell_dofs,
                               int32_t* nfree, int32_t* ndiri);

/* ---- conforming Q2 numbering on Cartesian grids (FESpaces/ConformingFESpaces.jl:367-636) --
 * Topology faces numbered first-touch (Geometry/GridTopologies.jl:1184-1250), face labels by
 * Gridap's Cartesian rule (Geometry/CartesianDiscreteModels.jl:133-260), dofs by dimension
 * then face id, own dofs "for node, for comp". entity_to_tag[3^D] (0 = untagged, else a
 * 1-based tag index), tag_masks[ntags*ncomp]. cell_dofs: ncells x (3^D * ncomp), local
 * order comp-major over the 3^D nodes (vertices, edges, faces, interior in n-cube order). */
int orc_conforming_q2(int D, const int64_t* partition, int ncomp, const int8_t* entity_to_tag,
                      const uint8_t* tag_masks, int32_t* cell_dofs, int32_t* nfree,
                      int32_t* ndiri);
/* Q2 Lagrange shape functions on the 3^D nodes in Gridap's order (n-cube faces: vertices,
 * edges, faces, interior; one node at each face centre). */
void orc_q2_shapes(int D, int npts, const double* pts, double* phi, double* dphi);
/* Diffusion cell arrays for Q2 on Q1 (trilinear) geometry: nodal geometry from the 2^D
 * cell vertices. Same steps as orc_q1_cell_arrays_diffusion. */
int orc_q2_cell_arrays_diffusion(int D, int64_t ncells, const int32_t* cell_vertices,
                                 const double* coords, const double* kappa_cell, int nq,
                                 const double* qx, const double* qw, int fkind,
                                 const double* fdata, double* cellmats, double* cellvecs);

/* ---- simplexified Cartesian boxes, P2 tets, elasticity ---------------------------------- */
/* Tet 6c+t of hex c: the hex's nodes at its t-th local tet (Geometry/Grids.jl:487-558,
 * ReferenceFEs/ExtrusionPolytopes.jl:290-299). tet_vertices[ntets*4], 1-based node ids. */
void orc_simplex_cells(const int64_t* partition, int32_t* tet_vertices);
/* Conforming P2 dofs on the simplexified box; vertex_mask[nverts] marks the vertices of the
 * Dirichlet vertex filter, comp_mask[ncomp] the constrained components. */
int orc_simplex_p2_numbering(const int64_t* partition, int ncomp, const uint8_t* vertex_mask,
                             const uint8_t* comp_mask, int32_t* cell_dofs, int32_t* nfree,
                             int32_t* ndiri);
void orc_p2tet_shapes(int npts, const double* pts, double* phi, double* dphi);
/* 14-point degree-5 Witherden-Vincent tet rule (Gridap's rule for degrees 4 and 5). */
double orc_wv_tet_degree5(double* pts, double* w);
int orc_p2tet_cell_arrays_elasticity(int64_t ncells, const int32_t* tet_vertices,
                                     const double* coords, const double* lame, int nq,
                                     const double* qx, const double* qw, const double* f,
                                     double* cellmats, double* cellvecs);

/* ---- quadrature (ReferenceFEs/Quadratures.jl:191-227, TensorProductQuadratures.jl:68-80) */
void orc_gauss_legendre01(int n, double* x, double* w);
/* Tensor-product Gauss-Legendre of a degree on [0,1]^D; returns npoints. */
int orc_tensor_quadrature(int D, int degree, double* coords, double* weights);

/* ---- Q1 (lexicographic-node multilinear) shape functions ------------------------------- */
void orc_q1_shapes(int D, int npts, const double* pts, double* phi, double* dphi);

/* ---- cell integrals ------------------------------------------------------------------- */
enum { ORC_F_NONE = 0, ORC_F_CONST = 1, ORC_F_NODAL = 2, ORC_F_QPOINT = 3 };
enum { ORC_GEOM_CARTESIAN = 0, ORC_GEOM_NODAL = 1 };
/* Physical coordinates of the quadrature points of every Q1 cell (ncells*nq*D). */
void orc_q1_cell_qpoints(int D, int64_t ncells, const int32_t* cell_nodes, const double* coords,
                         int nq, const double* qx, double* xq);
/* Diffusion stiffness  K_ij = sum_q (kappa grad v_i) . grad u_j |det Jt_q| w_q  and source
 * b_i = sum_q f(x_q) v_i |det Jt_q| w_q on Q1 cells (Fields/FieldsInterfaces.jl:708-720,
 * Fields/ApplyOptimizations.jl:293-310, TensorValues/Operations.jl:875-934).
 * geom = ORC_GEOM_CARTESIAN uses Jt = diag(h) (Geometry/CartesianGrids.jl:247-276);
 * ORC_GEOM_NODAL uses Jt_q = sum_a x_a (x) grad phi_a(xi_q) (Geometry/Grids.jl:237-241).
 * kappa_cell may be NULL (kappa = 1). cellmats/cellvecs may be NULL to skip. */
int orc_q1_cell_arrays_diffusion(int D, int64_t ncells, const int32_t* cell_nodes,
                                 const double* coords, int geom, const double* h,
                                 const double* kappa_cell, int nq, const double* qx,
                                 const double* qw, int fkind, const double* fdata,
                                 double* cellmats, double* cellvecs);

/* ---- assembly (FESpaces/SparseMatrixAssemblers.jl:174-316, Algebra/SparseMatrixCSC.jl) - */
typedef struct {
  int64_t nrows, ncols, nnz;
  int64_t* colptr; /* ncols+1, 1-based */
  int64_t* rowval; /* nnz, 1-based      */
  double* nzval;   /* nnz               */
} orc_csc;
/* symbolic loop (CounterCSC) + nz_allocation + numeric loop (InserterCSC) + create_from_nz.
 * cellmats may be NULL (pattern only, values 0). Returns 0 on success. */
int orc_assemble_matrix_csc(int64_t ncells, int nd, const int32_t* cell_rows,
                            const int32_t* cell_cols, const double* cellmats, int64_t nrows,
                            int64_t ncols, orc_csc* out);
/* The same for rectangular cells: ndr row ids, ndc column ids, ndr x ndc column-major cell
 * matrices (one block of a multi-field system). */
int orc_assemble_matrix_csc_rect(int64_t ncells, int ndr, int ndc, const int32_t* cell_rows,
                                 const int32_t* cell_cols, const double* cellmats,
                                 int64_t nrows, int64_t ncols, orc_csc* out);
void orc_csc_free(orc_csc* a);
/* Greedy first-fit colouring of the cells by shared free dofs; returns the colour count. */
int orc_color_cells(int64_t ncells, int nd, const int32_t* cell_dofs, int64_t nfree,
                    int32_t* color);
/* Colour-parallel assembly (OpenMP): cells of one colour in parallel, colours in order. */
int orc_assemble_csc_colored(int64_t ncells, int nd, const int32_t* cell_dofs,
                             const double* cellmats, const double* cellvecs, int64_t n,
                             int ncolors, const int64_t* color_ptr, const int64_t* color_cells,
                             int nthreads, orc_csc* out, double* b);
/* Threads of the per-cell loops (default 1: serial). */
void orc_set_cell_threads(int n);
/* Dense vector assembly (SparseMatrixAssemblers.jl:287-316). b must be zeroed by caller. */
void orc_assemble_vector(int64_t ncells, int nd, const int32_t* cell_rows,
                         const double* cellvecs, double* b);

/* ---- solver --------------------------------------------------------------------------- */
/* Jacobi-preconditioned CG (precond=1) or plain CG (precond=0) on a symmetric CSC matrix,
 * x0 = 0, stopping on ||r||_2 <= rtol ||b||_2. nthreads > 1 uses OpenMP row-parallel loops
 * (symmetric matrix: column j of the CSC is row j). Returns the iteration count (<0 on
 * error); *relres gets the final recursive relative residual. */
int orc_pcg(const orc_csc* A, const double* b, double* x, double rtol, int maxit, int precond,
            int nthreads, double* relres);
/* y = A x for a CSC matrix (serial, column-oriented as SparseArrays' mul!). */
void orc_csc_mul(const orc_csc* A, const double* x, double* y);

/* ---- free-dof reordering (gfe_oracle_reorder.c) --------------------------------------- */
/* compute_adjacency (Arrays/Tables.jl:1053-1107): 1-based ptrs (nfree+1) and data, malloc'd
 * (release with orc_free). */
int orc_compute_adjacency(int64_t ncells, int nd, const int32_t* cell_dofs, int64_t nfree,
                          int64_t** ptrs, int32_t** data);
void orc_free(void* p);
/* Reverse Cuthill-McKee / Sloan permutations (FESpaceReindexing.jl): iperm[old-1] = new. */
int orc_rcm_perm(int64_t nfree, const int64_t* ptrs, const int32_t* adj, int64_t* iperm);
int orc_sloan_perm(int64_t nfree, const int64_t* ptrs, const int32_t* adj, int64_t w1,
                   int64_t w2, int64_t* iperm);

#ifdef __cplusplus
}
#endif
#endif
