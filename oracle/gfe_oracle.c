/*
 * gfe_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle), not part of the product.
 *
 * CPU restatement of Gridap.jl v0.20.8's assembly and solve path. The functions follow the
 * Gridap sources cited beside each one, step by step, including the order in which values
 * are accumulated, so that the CUDA library can be checked against it entry by entry. The
 * restatement is pinned by the known-answer values in Gridap's own test suite (see
 * tests/golden/).
 */
#include "gfe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static double det_t(int D, const double* a);

/* Threads of the per-cell loops (cell matrices and vectors). 1 (the default) runs them
 * serially, as Gridap's lazy cell arrays are evaluated; more threads split the cells, which
 * changes no arithmetic. */
static int g_cell_threads = 1;
void orc_set_cell_threads(int n) { g_cell_threads = n > 0 ? n : 1; }
static void inv_t(int D, const double* a, double* r);

/* ====================================================================================== */
/* polytopes                                                                               */
/* ====================================================================================== */

/* Gridap enumerates the faces of an extrusion polytope recursively and then applies a
 * sequence of stable sorts: by anchor[1..D], then extrusion[1..D], then face dimension
 * (ReferenceFEs/ExtrusionPolytopes.jl:460-481). The last sort is the primary key, so the
 * final order is: dimension, then extrusion read with its last component most significant,
 * then anchor read the same way. Every (extrusion, anchor) pair is distinct, so that key
 * fixes the order regardless of the recursion's initial order. */
static int ncube_key(int D, const int32_t* ext, const int32_t* anc) {
  int dim = 0, e = 0, a = 0;
  for (int d = 0; d < D; ++d) {
    dim += ext[d] != 0;
    e |= (ext[d] != 0) << d;
    a |= (anc[d] != 0) << d;
  }
  return (dim << 16) | (e << 8) | a;
}

int orc_ncube_faces(int D, int32_t* ext, int32_t* anchor) {
  int n = 0;
  int32_t e[3], a[3];
  int keys[27];
  int32_t tmp_e[27 * 3], tmp_a[27 * 3];
  for (int em = 0; em < (1 << D); ++em)
    for (int am = 0; am < (1 << D); ++am) {
      if (am & em) continue; /* anchor is 0 along extruded directions */
      for (int d = 0; d < D; ++d) {
        e[d] = (em >> d) & 1;
        a[d] = (am >> d) & 1;
      }
      memcpy(tmp_e + n * D, e, sizeof(int32_t) * D);
      memcpy(tmp_a + n * D, a, sizeof(int32_t) * D);
      keys[n] = ncube_key(D, e, a);
      ++n;
    }
  /* selection by key */
  int used[27] = {0};
  for (int k = 0; k < n; ++k) {
    int best = -1;
    for (int i = 0; i < n; ++i)
      if (!used[i] && (best < 0 || keys[i] < keys[best])) best = i;
    used[best] = 1;
    memcpy(ext + k * D, tmp_e + best * D, sizeof(int32_t) * D);
    memcpy(anchor + k * D, tmp_a + best * D, sizeof(int32_t) * D);
  }
  return n;
}

/* ====================================================================================== */
/* Cartesian model                                                                         */
/* ====================================================================================== */

/* Node coordinates: x0[d] + (I[d]-1)*dx[d], dx = (hi-lo)/n, nodes in column-major
 * LinearIndices order (Geometry/CartesianGrids.jl:58-62,115-123). */
void orc_cartesian_coords(int D, const int64_t* part, const double* domain, double* coords) {
  int64_t np[3] = {1, 1, 1};
  double x0[3], dx[3];
  for (int d = 0; d < D; ++d) {
    np[d] = part[d] + 1;
    x0[d] = domain[2 * d];
    dx[d] = (domain[2 * d + 1] - domain[2 * d]) / (double)part[d];
  }
  int64_t node = 0;
  for (int64_t k = 0; k < np[2]; ++k)
    for (int64_t j = 0; j < np[1]; ++j)
      for (int64_t i = 0; i < np[0]; ++i, ++node) {
        int64_t I[3] = {i, j, k};
        for (int d = 0; d < D; ++d) coords[node * D + d] = x0[d] + (double)I[d] * dx[d];
      }
}

/* Cell nodes: cell (i,j,k) gets nodes[(i,j,k) + lnode] for lnode in CartesianIndices of
 * 2^D, first index fastest (Geometry/CartesianGrids.jl:152-161). Ids 1-based. */
void orc_cartesian_cell_nodes(int D, const int64_t* part, int32_t* cell_nodes) {
  int64_t n[3] = {1, 1, 1}, np[3] = {1, 1, 1};
  for (int d = 0; d < D; ++d) {
    n[d] = part[d];
    np[d] = part[d] + 1;
  }
  int nv = 1 << D;
  int64_t cell = 0;
  for (int64_t k = 0; k < n[2]; ++k)
    for (int64_t j = 0; j < n[1]; ++j)
      for (int64_t i = 0; i < n[0]; ++i, ++cell)
        for (int a = 0; a < nv; ++a) {
          int64_t I[3] = {i + (a & 1), j + ((a >> 1) & 1), k + ((a >> 2) & 1)};
          int64_t id = I[0] + np[0] * (I[1] + np[1] * I[2]);
          cell_nodes[cell * nv + a] = (int32_t)(id + 1);
        }
}

/* A vertex of the Cartesian mesh lies in the interior of exactly one face of the domain
 * box: extruded along directions where it is strictly inside, anchored at 1 where it sits
 * on the upper side. Its label is that face's 1-based id in the box polytope
 * (Geometry/CartesianDiscreteModels.jl:133-189 assigns these entities). */
void orc_cartesian_node_entity(int D, const int64_t* part, int32_t* node_entity) {
  int32_t ext[27 * 3], anc[27 * 3];
  int nf = orc_ncube_faces(D, ext, anc);
  int64_t np[3] = {1, 1, 1};
  for (int d = 0; d < D; ++d) np[d] = part[d] + 1;
  int64_t node = 0;
  for (int64_t k = 0; k < np[2]; ++k)
    for (int64_t j = 0; j < np[1]; ++j)
      for (int64_t i = 0; i < np[0]; ++i, ++node) {
        int64_t I[3] = {i, j, k};
        int32_t e[3] = {0, 0, 0}, a[3] = {0, 0, 0};
        for (int d = 0; d < D; ++d) {
          if (I[d] == 0) {
            e[d] = 0; a[d] = 0;
          } else if (I[d] == part[d]) {
            e[d] = 0; a[d] = 1;
          } else {
            e[d] = 1; a[d] = 0;
          }
        }
        int found = 0;
        for (int f = 0; f < nf; ++f) {
          int ok = 1;
          for (int d = 0; d < D; ++d)
            if (ext[f * D + d] != e[d] || anc[f * D + d] != a[d]) ok = 0;
          if (ok) { found = f + 1; break; }
        }
        node_entity[node] = found;
      }
}

/* get_face_tag_index: the first tag (in the given order) whose entity set contains the
 * face's entity (Geometry/FaceLabelings.jl:411-427). */
void orc_node_tag_index(int64_t nnodes, const int32_t* node_entity, int ntags,
                        const int32_t* tag_ptrs, const int32_t* tag_entities,
                        int8_t* node_to_tag) {
  for (int64_t n = 0; n < nnodes; ++n) {
    node_to_tag[n] = 0;
    for (int t = 0; t < ntags; ++t) {
      int hit = 0;
      for (int32_t p = tag_ptrs[t]; p < tag_ptrs[t + 1]; ++p)
        if (tag_entities[p] == node_entity[n]) { hit = 1; break; }
      if (hit) { node_to_tag[n] = (int8_t)(t + 1); break; }
    }
  }
}

void orc_jitter_interior(int D, const int64_t* part, const double* jitter, double* coords) {
  int64_t np[3] = {1, 1, 1};
  for (int d = 0; d < D; ++d) np[d] = part[d] + 1;
  int64_t node = 0;
  for (int64_t k = 0; k < np[2]; ++k)
    for (int64_t j = 0; j < np[1]; ++j)
      for (int64_t i = 0; i < np[0]; ++i, ++node) {
        int64_t I[3] = {i, j, k};
        int interior = 1;
        for (int d = 0; d < D; ++d)
          if (I[d] == 0 || I[d] == part[d]) interior = 0;
        if (interior)
          for (int d = 0; d < D; ++d) coords[node * D + d] += jitter[node * D + d];
      }
}

/* ====================================================================================== */
/* CLagrangian numbering                                                                   */
/* ====================================================================================== */

/* _generate_node_to_dof_glue_component_major (FESpaces/CLagrangianFESpaces.jl:155-275):
 * walk nodes in order; for each node walk components; a masked (node,comp) of a tagged
 * node becomes the next Dirichlet dof (negative), every other one the next free dof.
 * _fill_cell_dofs_clagrangian! (:356-380) then gathers cell dofs through the local
 * (node,comp) -> local dof table. */
void orc_clagrangian_numbering(int64_t nnodes, const int8_t* node_to_tag, int ncomp,
                               const uint8_t* tag_masks, int64_t ncells, int nv,
                               const int32_t* cell_nodes, const int32_t* lnode_comp_to_ldof,
                               int32_t* node_comp_to_dof, int32_t* cell_dofs,
                               int32_t* nfree, int32_t* ndiri) {
  int32_t nf = 0, nd = 0;
  for (int64_t n = 0; n < nnodes; ++n) {
    int tag = node_to_tag[n];
    for (int c = 0; c < ncomp; ++c) {
      int diri = tag != 0 && tag_masks[(tag - 1) * ncomp + c];
      if (diri)
        node_comp_to_dof[n * ncomp + c] = -(++nd);
      else
        node_comp_to_dof[n * ncomp + c] = ++nf;
    }
  }
  *nfree = nf;
  *ndiri = nd;
  int ndof_cell = nv * ncomp;
  for (int64_t cell = 0; cell < ncells; ++cell)
    for (int a = 0; a < nv; ++a) {
      int64_t node = cell_nodes[cell * nv + a] - 1;
      for (int c = 0; c < ncomp; ++c) {
        int ldof = lnode_comp_to_ldof[a * ncomp + c];
        cell_dofs[cell * ndof_cell + ldof - 1] = node_comp_to_dof[node * ncomp + c];
      }
    }
}

/* ====================================================================================== */
/* conforming Q2 numbering on Cartesian grids                                              */
/* ====================================================================================== */

/* local vertices of each n-cube face (lexicographic in the face's own coordinates) */
static int face_lvertices(int D, const int32_t* ext, const int32_t* anc, int32_t* lv) {
  int nv = 0;
  int span[3], ns = 0;
  for (int d = 0; d < D; ++d)
    if (ext[d]) span[ns++] = d;
  for (int m = 0; m < (1 << ns); ++m) {
    int v = 0;
    for (int d = 0; d < D; ++d) {
      int bit = anc[d];
      for (int t = 0; t < ns; ++t)
        if (span[t] == d) bit = (m >> t) & 1;
      v |= bit << d;
    }
    lv[nv++] = v;
  }
  return nv;
}

static int cmp_i32(const void* a, const void* b) {
  int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

int orc_conforming_q2(int D, const int64_t* part, int ncomp, const int8_t* entity_to_tag,
                      const uint8_t* tag_masks, int32_t* cell_dofs, int32_t* nfree,
                      int32_t* ndiri) {
  int32_t ext[27 * 3], anc[27 * 3];
  const int nlf = orc_ncube_faces(D, ext, anc); /* 3^D local faces incl. the cell */
  int32_t lf_dim[27], lf_nv[27], lf_v[27][8];
  for (int f = 0; f < nlf; ++f) {
    lf_dim[f] = 0;
    for (int d = 0; d < D; ++d) lf_dim[f] += ext[f * D + d];
    lf_nv[f] = face_lvertices(D, ext + f * D, anc + f * D, lf_v[f]);
  }
  int64_t n[3] = {1, 1, 1}, np[3] = {1, 1, 1};
  for (int d = 0; d < D; ++d) {
    n[d] = part[d];
    np[d] = part[d] + 1;
  }
  const int64_t ncells = n[0] * n[1] * n[2];
  const int64_t nverts = np[0] * np[1] * np[2];
  const int nvc = 1 << D;
  int32_t* cv = (int32_t*)malloc(sizeof(int32_t) * ncells * nvc);
  orc_cartesian_cell_nodes(D, part, cv);
  /* vertex -> cells */
  int64_t* vptr = (int64_t*)calloc(nverts + 1, sizeof(int64_t));
  for (int64_t c = 0; c < ncells; ++c)
    for (int a = 0; a < nvc; ++a) vptr[cv[c * nvc + a]] += 1;
  for (int64_t v = 0; v < nverts; ++v) vptr[v + 1] += vptr[v];
  int64_t* vfill = (int64_t*)calloc(nverts, sizeof(int64_t));
  int32_t* vcells = (int32_t*)malloc(sizeof(int32_t) * vptr[nverts]);
  for (int64_t c = 0; c < ncells; ++c)
    for (int a = 0; a < nvc; ++a) {
      int64_t v = cv[c * nvc + a] - 1;
      vcells[vptr[v] + vfill[v]++] = (int32_t)c; /* ascending cell order */
    }
  /* cell -> face ids per local face (vertices = node ids; cell interiors = cell ids); faces
   * of each dimension numbered first-touch over (cell, local face) */
  int32_t* cf = (int32_t*)malloc(sizeof(int32_t) * ncells * nlf);
  for (int64_t i = 0; i < ncells * nlf; ++i) cf[i] = 0;
  int32_t nface_d[4] = {0, 0, 0, 0};
  for (int dd = 1; dd < D; ++dd) {
    int32_t next = 0;
    for (int64_t c = 0; c < ncells; ++c)
      for (int f = 0; f < nlf; ++f) {
        if (lf_dim[f] != dd || cf[c * nlf + f] != 0) continue;
        int32_t fv[8];
        for (int k = 0; k < lf_nv[f]; ++k) fv[k] = cv[c * nvc + lf_v[f][k]];
        qsort(fv, lf_nv[f], sizeof(int32_t), cmp_i32);
        ++next;
        /* cells around all vertices of the face: intersect vertex -> cells lists */
        int64_t v0 = fv[0] - 1;
        for (int64_t p = vptr[v0]; p < vptr[v0 + 1]; ++p) {
          int32_t c2 = vcells[p];
          int ok = 1;
          for (int k = 1; k < lf_nv[f] && ok; ++k) {
            int64_t vk = fv[k] - 1, hit = 0;
            for (int64_t q = vptr[vk]; q < vptr[vk + 1]; ++q)
              if (vcells[q] == c2) hit = 1;
            ok = (int)hit;
          }
          if (!ok) continue;
          /* local face of c2 with the same vertex set */
          for (int f2 = 0; f2 < nlf; ++f2) {
            if (lf_dim[f2] != dd) continue;
            int32_t gv[8];
            for (int k = 0; k < lf_nv[f2]; ++k) gv[k] = cv[c2 * nvc + lf_v[f2][k]];
            qsort(gv, lf_nv[f2], sizeof(int32_t), cmp_i32);
            if (memcmp(gv, fv, sizeof(int32_t) * lf_nv[f]) == 0) cf[(int64_t)c2 * nlf + f2] = next;
          }
        }
      }
    nface_d[dd] = next;
  }
  nface_d[0] = (int32_t)nverts;
  nface_d[D] = (int32_t)ncells;
  for (int64_t c = 0; c < ncells; ++c)
    for (int f = 0; f < nlf; ++f) {
      if (lf_dim[f] == 0) cf[c * nlf + f] = cv[c * nvc + lf_v[f][0]];
      if (lf_dim[f] == D) cf[c * nlf + f] = (int32_t)(c + 1);
    }
  /* labels: a d-face with one cell around takes that cell's local face id; one with fewer
   * than 2^(D-d) cells is "boundary" and takes the first non-interior, non-boundary label of
   * a higher-dimensional face containing it (CartesianDiscreteModels.jl:195-260) */
  int32_t* lab[4];
  int32_t* ncell_around[4];
  for (int dd = 0; dd <= D; ++dd) {
    lab[dd] = (int32_t*)malloc(sizeof(int32_t) * (nface_d[dd] + 1));
    ncell_around[dd] = (int32_t*)calloc(nface_d[dd] + 1, sizeof(int32_t));
  }
  const int32_t interior = nlf, boundary = -1;
  for (int64_t c = 0; c < ncells; ++c)
    for (int f = 0; f < nlf; ++f) ncell_around[lf_dim[f]][cf[c * nlf + f]] += 1;
  for (int dd = 0; dd <= D; ++dd)
    for (int32_t i = 1; i <= nface_d[dd]; ++i) {
      int32_t k = ncell_around[dd][i];
      lab[dd][i] = interior;
      if (dd < D && k != (1 << (D - dd)) && k != 1) lab[dd][i] = boundary;
    }
  for (int64_t c = 0; c < ncells; ++c)
    for (int f = 0; f < nlf; ++f) {
      int dd = lf_dim[f];
      int32_t i = cf[c * nlf + f];
      if (dd < D && ncell_around[dd][i] == 1) lab[dd][i] = f + 1;
    }
  /* fix boundary labels from higher-dimensional faces, ascending dimension j > d; the
   * d-face -> j-faces relation is taken from the cells' local faces */
  for (int dd = 0; dd <= D - 2; ++dd)
    for (int jj = dd + 1; jj <= D - 1; ++jj)
      for (int64_t c = 0; c < ncells; ++c)
        for (int f = 0; f < nlf; ++f) {
          if (lf_dim[f] != dd) continue;
          int32_t i = cf[c * nlf + f];
          if (lab[dd][i] != boundary) continue;
          /* j-faces of this cell that contain local face f, in local order */
          for (int g = 0; g < nlf; ++g) {
            if (lf_dim[g] != jj) continue;
            int contains = 1;
            for (int k = 0; k < lf_nv[f]; ++k) {
              int in = 0;
              for (int m = 0; m < lf_nv[g]; ++m) in |= lf_v[g][m] == lf_v[f][k];
              contains &= in;
            }
            if (!contains) continue;
            int32_t gl = lab[jj][cf[c * nlf + g]];
            if (gl != interior && gl != boundary) {
              lab[dd][i] = gl;
              break;
            }
          }
        }
  /* dofs: dimension by dimension, face id order, one node per face, comps inside */
  int32_t* fdof[4];
  int32_t nf = 0, nd = 0;
  for (int dd = 0; dd <= D; ++dd) {
    fdof[dd] = (int32_t*)malloc(sizeof(int32_t) * (nface_d[dd] + 1) * ncomp);
    for (int32_t i = 1; i <= nface_d[dd]; ++i) {
      int32_t ent = lab[dd][i];
      int tag = (ent >= 1 && ent <= nlf) ? entity_to_tag[ent - 1] : 0;
      for (int k = 0; k < ncomp; ++k) {
        int diri = tag > 0 && tag_masks[(tag - 1) * ncomp + k];
        fdof[dd][i * ncomp + k] = diri ? -(++nd) : ++nf;
      }
    }
  }
  const int ndc = nlf * ncomp;
  for (int64_t c = 0; c < ncells; ++c)
    for (int f = 0; f < nlf; ++f)
      for (int k = 0; k < ncomp; ++k)
        cell_dofs[c * ndc + k * nlf + f] = fdof[lf_dim[f]][cf[c * nlf + f] * ncomp + k];
  *nfree = nf;
  *ndiri = nd;
  for (int dd = 0; dd <= D; ++dd) {
    free(lab[dd]);
    free(ncell_around[dd]);
    free(fdof[dd]);
  }
  free(cv); free(vptr); free(vfill); free(vcells); free(cf);
  return 0;
}

/* Q2 node of local face f: lattice index 2*anchor along fixed directions, 1 along spanned */
void orc_q2_shapes(int D, int npts, const double* pts, double* phi, double* dphi) {
  int32_t ext[27 * 3], anc[27 * 3];
  const int nn = orc_ncube_faces(D, ext, anc);
  for (int p = 0; p < npts; ++p)
    for (int a = 0; a < nn; ++a) {
      double L[3], dL[3];
      for (int d = 0; d < D; ++d) {
        const int idx = ext[a * D + d] ? 1 : 2 * anc[a * D + d];
        const double t = pts[p * D + d];
        if (idx == 0) {
          L[d] = 2.0 * (t - 0.5) * (t - 1.0);
          dL[d] = 4.0 * t - 3.0;
        } else if (idx == 1) {
          L[d] = 4.0 * t * (1.0 - t);
          dL[d] = 4.0 - 8.0 * t;
        } else {
          L[d] = 2.0 * t * (t - 0.5);
          dL[d] = 4.0 * t - 1.0;
        }
      }
      double v = 1.0;
      for (int d = 0; d < D; ++d) v *= L[d];
      phi[p * nn + a] = v;
      for (int k = 0; k < D; ++k) {
        double g = 1.0;
        for (int d = 0; d < D; ++d) g *= (d == k) ? dL[d] : L[d];
        dphi[(p * nn + a) * D + k] = g;
      }
    }
}

int orc_q2_cell_arrays_diffusion(int D, int64_t ncells, const int32_t* cell_vertices,
                                 const double* coords, const double* kappa_cell, int nq,
                                 const double* qx, const double* qw, int fkind,
                                 const double* fdata, double* cellmats, double* cellvecs) {
  const int nv = 1 << D, nn = D == 2 ? 9 : 27;
  double* phi1 = (double*)malloc(sizeof(double) * nq * nv);
  double* dphi1 = (double*)malloc(sizeof(double) * nq * nv * D);
  double* phi = (double*)malloc(sizeof(double) * nq * nn);
  double* dphi = (double*)malloc(sizeof(double) * nq * nn * D);
  orc_q1_shapes(D, nq, qx, phi1, dphi1);
  orc_q2_shapes(D, nq, qx, phi, dphi);
  int bad = 0;
  /* cells are independent: threads (orc_set_cell_threads) split the cell range, and every
   * cell's arithmetic is the serial one, so the arrays are identical for any thread count */
#pragma omp parallel for schedule(dynamic, 256) num_threads(g_cell_threads) if (g_cell_threads > 1)
  for (int64_t c = 0; c < ncells; ++c) {
    double g[27 * 3];
    const int32_t* vs = cell_vertices + c * nv;
    double* K = cellmats ? cellmats + c * nn * nn : NULL;
    double* bv = cellvecs ? cellvecs + c * nn : NULL;
    if (K) memset(K, 0, sizeof(double) * nn * nn);
    if (bv) memset(bv, 0, sizeof(double) * nn);
    const double kap = kappa_cell ? kappa_cell[c] : 1.0;
    for (int q = 0; q < nq; ++q) {
      double Jt[9] = {0}, iJt[9];
      for (int a = 0; a < nv; ++a) {
        const double* xa = coords + (int64_t)(vs[a] - 1) * D;
        for (int k = 0; k < D; ++k)
          for (int l = 0; l < D; ++l) Jt[k * D + l] += dphi1[(q * nv + a) * D + k] * xa[l];
      }
      const double dJ = det_t(D, Jt);
      if (!(dJ > 0.0) && !(dJ < 0.0)) {
#pragma omp atomic write
        bad = 1;
        break;
      }
      inv_t(D, Jt, iJt);
      const double dV = fabs(dJ) * qw[q];
      for (int a = 0; a < nn; ++a)
        for (int k = 0; k < D; ++k) {
          double s = 0.0;
          for (int l = 0; l < D; ++l) s += iJt[k * D + l] * dphi[(q * nn + a) * D + l];
          g[a * D + k] = s;
        }
      if (K)
        for (int j = 0; j < nn; ++j)
          for (int i = 0; i < nn; ++i) {
            double s = 0.0;
            if (kappa_cell)
              for (int k = 0; k < D; ++k) s += (kap * g[i * D + k]) * g[j * D + k];
            else
              for (int k = 0; k < D; ++k) s += g[i * D + k] * g[j * D + k];
            K[i + j * nn] += s * dV;
          }
      if (bv && fkind != ORC_F_NONE) {
        double fq = fkind == ORC_F_CONST ? fdata[0] : fdata[c * nq + q];
        for (int i = 0; i < nn; ++i) bv[i] += (fq * phi[q * nn + i]) * dV;
      }
    }
  }
  free(phi1); free(dphi1); free(phi); free(dphi);
  return bad ? -1 : 0;
}

/* ====================================================================================== */
/* quadrature                                                                              */
/* ====================================================================================== */

/* Gauss-Legendre nodes/weights on [-1,1] by Newton iteration on P_n (the Golub-Welsch
 * rule gives the same unique nodes), mapped to [0,1] as x=(x+1)/2, w=w/2
 * (ReferenceFEs/TensorProductQuadratures.jl:68-80). Nodes ascending. */
void orc_gauss_legendre01(int n, double* x, double* w) {
  /* evaluated in long double, then rounded: the weights come out within ~0.5 ulp */
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int i = 0; i < n; ++i) {
    long double z = cosl(pi * (i + 0.75L) / (n + 0.5L));
    long double p0 = 1.0L, p1 = z, dp = 1.0L;
    for (int it = 0; it < 100; ++it) {
      p0 = 1.0L;
      p1 = z;
      for (int k = 2; k <= n; ++k) {
        long double p2 = ((2.0L * k - 1.0L) * z * p1 - (k - 1.0L) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = (n == 1) ? 1.0L : n * (z * p1 - p0) / (z * z - 1.0L);
      long double dz = p1 / dp;
      z -= dz;
      if (fabsl(dz) < 1e-30L) break;
    }
    p0 = 1.0L;
    p1 = z;
    for (int k = 2; k <= n; ++k) {
      long double p2 = ((2.0L * k - 1.0L) * z * p1 - (k - 1.0L) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = (n == 1) ? 1.0L : n * (z * p1 - p0) / (z * z - 1.0L);
    /* z decreases with i: store ascending */
    x[n - 1 - i] = (double)((z + 1.0L) / 2.0L);
    w[n - 1 - i] = (double)((2.0L / ((1.0L - z * z) * dp * dp)) / 2.0L);
  }
}

/* npoints per direction = div(degree,2)+1 (Quadratures.jl:191); tensor product over
 * CartesianIndices, first index fastest, w = prod of 1D weights (Quadratures.jl:193-227). */
int orc_tensor_quadrature(int D, int degree, double* coords, double* weights) {
  int n = degree / 2 + 1;
  double x1[64], w1[64];
  orc_gauss_legendre01(n, x1, w1);
  int np = 1;
  for (int d = 0; d < D; ++d) np *= n;
  for (int k = 0; k < np; ++k) {
    int r = k;
    double w = 1.0;
    for (int d = 0; d < D; ++d) {
      int i = r % n;
      r /= n;
      coords[k * D + d] = x1[i];
      w *= w1[i];
    }
    weights[k] = w;
  }
  return np;
}

/* ====================================================================================== */
/* Q1 shape functions                                                                      */
/* ====================================================================================== */

/* Multilinear Lagrange basis on the lexicographically ordered vertices of [0,1]^D (the
 * node order of Gridap's first-order LagrangianRefFE on QUAD/HEX,
 * ReferenceFEs/CLagrangianRefFEs.jl:246-275). phi[p*nv+a], dphi[(p*nv+a)*D+k]. */
void orc_q1_shapes(int D, int npts, const double* pts, double* phi, double* dphi) {
  int nv = 1 << D;
  for (int p = 0; p < npts; ++p)
    for (int a = 0; a < nv; ++a) {
      double f[3], g[3];
      for (int d = 0; d < D; ++d) {
        int b = (a >> d) & 1;
        double xi = pts[p * D + d];
        f[d] = b ? xi : 1.0 - xi;
        g[d] = b ? 1.0 : -1.0;
      }
      double v = 1.0;
      for (int d = 0; d < D; ++d) v *= f[d];
      phi[p * nv + a] = v;
      for (int k = 0; k < D; ++k) {
        double dv = 1.0;
        for (int d = 0; d < D; ++d) dv *= (d == k) ? g[d] : f[d];
        dphi[(p * nv + a) * D + k] = dv;
      }
    }
}

/* ====================================================================================== */
/* tensor algebra of TensorValues/Operations.jl:875-934,989                                */
/* ====================================================================================== */

/* A[k][l] stored as A[k*D+l]. */
static double det_t(int D, const double* a) {
  if (D == 1) return a[0];
  if (D == 2) return a[0] * a[3] - a[1] * a[2];
  double a11 = a[0], a12 = a[1], a13 = a[2], a21 = a[3], a22 = a[4], a23 = a[5], a31 = a[6],
         a32 = a[7], a33 = a[8];
  return a11 * a22 * a33 + a12 * a23 * a31 + a13 * a21 * a32 -
         (a11 * a23 * a32 + a12 * a21 * a33 + a13 * a22 * a31);
}

static void inv_t(int D, const double* a, double* r) {
  if (D == 1) {
    r[0] = 1.0 / a[0];
    return;
  }
  if (D == 2) {
    double c = 1.0 / det_t(2, a);
    r[0] = a[3] * c;
    r[1] = -a[1] * c;
    r[2] = -a[2] * c;
    r[3] = a[0] * c;
    return;
  }
  double a11 = a[0], a12 = a[1], a13 = a[2], a21 = a[3], a22 = a[4], a23 = a[5], a31 = a[6],
         a32 = a[7], a33 = a[8];
  double c = 1.0 / det_t(3, a);
  r[0] = (a22 * a33 - a23 * a32) * c;
  r[3] = -(a21 * a33 - a23 * a31) * c;
  r[6] = (a21 * a32 - a22 * a31) * c;
  r[1] = -(a12 * a33 - a13 * a32) * c;
  r[4] = (a11 * a33 - a13 * a31) * c;
  r[7] = -(a11 * a32 - a12 * a31) * c;
  r[2] = (a12 * a23 - a13 * a22) * c;
  r[5] = -(a11 * a23 - a13 * a21) * c;
  r[8] = (a11 * a22 - a12 * a21) * c;
}

/* ====================================================================================== */
/* cell integrals                                                                          */
/* ====================================================================================== */

void orc_q1_cell_qpoints(int D, int64_t ncells, const int32_t* cell_nodes, const double* coords,
                         int nq, const double* qx, double* xq) {
  int nv = 1 << D;
  double* phi = (double*)malloc(sizeof(double) * nq * nv);
  double* dphi = (double*)malloc(sizeof(double) * nq * nv * D);
  orc_q1_shapes(D, nq, qx, phi, dphi);
  for (int64_t c = 0; c < ncells; ++c)
    for (int q = 0; q < nq; ++q)
      for (int l = 0; l < D; ++l) {
        double s = 0.0;
        for (int a = 0; a < nv; ++a)
          s += phi[q * nv + a] * coords[(int64_t)(cell_nodes[c * nv + a] - 1) * D + l];
        xq[(c * nq + q) * D + l] = s;
      }
  free(phi);
  free(dphi);
}

int orc_q1_cell_arrays_diffusion(int D, int64_t ncells, const int32_t* cell_nodes,
                                 const double* coords, int geom, const double* h,
                                 const double* kappa_cell, int nq, const double* qx,
                                 const double* qw, int fkind, const double* fdata,
                                 double* cellmats, double* cellvecs) {
  int nv = 1 << D;
  double* phi = (double*)malloc(sizeof(double) * nq * nv);
  double* dphi = (double*)malloc(sizeof(double) * nq * nv * D);
  orc_q1_shapes(D, nq, qx, phi, dphi);
  int bad = 0;
  /* cells are independent (see orc_q2_cell_arrays_diffusion) */
#pragma omp parallel for schedule(dynamic, 1024) num_threads(g_cell_threads) if (g_cell_threads > 1)
  for (int64_t c = 0; c < ncells; ++c) {
    double g[8 * 3];
    const int32_t* nodes = cell_nodes + c * nv;
    double* K = cellmats ? cellmats + c * nv * nv : NULL;
    double* bv = cellvecs ? cellvecs + c * nv : NULL;
    if (K) memset(K, 0, sizeof(double) * nv * nv);
    if (bv) memset(bv, 0, sizeof(double) * nv);
    double kap = kappa_cell ? kappa_cell[c] : 1.0;
    for (int q = 0; q < nq; ++q) {
      /* Jt at the quadrature point */
      double Jt[9] = {0}, iJt[9];
      if (geom == ORC_GEOM_CARTESIAN) {
        for (int k = 0; k < D; ++k) Jt[k * D + k] = h[k];
      } else {
        for (int a = 0; a < nv; ++a) {
          const double* xa = coords + (int64_t)(nodes[a] - 1) * D;
          for (int k = 0; k < D; ++k)
            for (int l = 0; l < D; ++l) Jt[k * D + l] += dphi[(q * nv + a) * D + k] * xa[l];
        }
      }
      double dJ = det_t(D, Jt);
      if (!(dJ > 0.0) && !(dJ < 0.0)) {
#pragma omp atomic write
        bad = 1; /* degenerate cell */
        break;
      }
      inv_t(D, Jt, iJt);
      double dV = fabs(dJ) * qw[q];
      /* physical gradients: invJt . grad phi_hat */
      for (int a = 0; a < nv; ++a)
        for (int k = 0; k < D; ++k) {
          double s = 0.0;
          for (int l = 0; l < D; ++l) s += iJt[k * D + l] * dphi[(q * nv + a) * D + l];
          g[a * D + k] = s;
        }
      if (K) {
        for (int j = 0; j < nv; ++j)
          for (int i = 0; i < nv; ++i) {
            double s = 0.0;
            if (kappa_cell)
              for (int k = 0; k < D; ++k) s += (kap * g[i * D + k]) * g[j * D + k];
            else
              for (int k = 0; k < D; ++k) s += g[i * D + k] * g[j * D + k];
            K[i + j * nv] += s * dV;
          }
      }
      if (bv && fkind != ORC_F_NONE) {
        double fq;
        if (fkind == ORC_F_CONST) {
          fq = fdata[0];
        } else if (fkind == ORC_F_NODAL) {
          fq = 0.0;
          for (int a = 0; a < nv; ++a) fq += fdata[nodes[a] - 1] * phi[q * nv + a];
        } else {
          fq = fdata[c * nq + q];
        }
        for (int i = 0; i < nv; ++i) bv[i] += (fq * phi[q * nv + i]) * dV;
      }
    }
  }
  free(phi);
  free(dphi);
  return bad ? -1 : 0;
}

/* ====================================================================================== */
/* assembly                                                                                */
/* ====================================================================================== */

/* lower bound of x in v[lo..hi] (inclusive), returns hi+1 if all smaller
 * (Base.searchsortedfirst as used by Algebra/SparseMatrixCSC.jl:128). */
static int64_t sorted_first(const int64_t* v, int64_t x, int64_t lo, int64_t hi) {
  int64_t a = lo, b = hi + 1;
  while (a < b) {
    int64_t m = a + (b - a) / 2;
    if (v[m] < x) a = m + 1; else b = m;
  }
  return a;
}

int orc_assemble_matrix_csc(int64_t ncells, int nd, const int32_t* cell_rows,
                            const int32_t* cell_cols, const double* cellmats, int64_t nrows,
                            int64_t ncols, orc_csc* out) {
  return orc_assemble_matrix_csc_rect(ncells, nd, nd, cell_rows, cell_cols, cellmats, nrows,
                                      ncols, out);
}

/* Rectangular cell blocks (ndr rows x ndc cols per cell, column-major cell matrices): the
 * assembly of one block of a multi-field system (MultiField/BlockSparseMatrixAssemblers.jl:
 * 197-230 runs the loops below on every block's (rows, cols) pair). */
int orc_assemble_matrix_csc_rect(int64_t ncells, int ndr, int ndc, const int32_t* cell_rows,
                                 const int32_t* cell_cols, const double* cellmats,
                                 int64_t nrows, int64_t ncols, orc_csc* out) {
  /* symbolic loop: CounterCSC.colnnzmax[j] += 1 for every positive (i,j) touched
   * (FESpaces/SparseMatrixAssemblers.jl:174-210, Algebra/SparseMatrixCSC.jl:72-89) */
  int64_t* colnnz = (int64_t*)calloc(ncols + 1, sizeof(int64_t));
  int64_t* colptr = (int64_t*)malloc(sizeof(int64_t) * (ncols + 1));
  if (!colnnz || !colptr) return -1;
  for (int64_t c = 0; c < ncells; ++c) {
    const int32_t* rs = cell_rows + c * ndr;
    const int32_t* cs = cell_cols + c * ndc;
    for (int lj = 0; lj < ndc; ++lj) {
      if (cs[lj] <= 0) continue;
      for (int li = 0; li < ndr; ++li)
        if (rs[li] > 0) colnnz[cs[lj] - 1] += 1;
    }
  }
  /* nz_allocation (SparseMatrixCSC.jl:250-262): colptr from counts, colnnz reset */
  colptr[0] = 1;
  for (int64_t j = 0; j < ncols; ++j) colptr[j + 1] = colptr[j] + colnnz[j];
  int64_t ndata = colptr[ncols] - 1;
  int64_t* rowval = (int64_t*)malloc(sizeof(int64_t) * (ndata > 0 ? ndata : 1));
  double* nzval = (double*)calloc(ndata > 0 ? ndata : 1, sizeof(double));
  if (!rowval || !nzval) return -1;
  memset(colnnz, 0, sizeof(int64_t) * (ncols + 1));
  /* numeric loop: InserterCSC.add_entry! in cell order, cols outer, rows inner
   * (SparseMatrixAssemblers.jl:214-248, AlgebraInterfaces.jl:176-187,
   * SparseMatrixCSC.jl:124-150); arrays here are 0-based views of 1-based data. */
  for (int64_t c = 0; c < ncells; ++c) {
    const int32_t* rs = cell_rows + c * ndr;
    const int32_t* cs = cell_cols + c * ndc;
    const double* vs = cellmats ? cellmats + c * ndr * ndc : NULL;
    for (int lj = 0; lj < ndc; ++lj) {
      int64_t j = cs[lj];
      if (j <= 0) continue;
      for (int li = 0; li < ndr; ++li) {
        int64_t i = rs[li];
        if (i <= 0) continue;
        double v = vs ? vs[li + lj * ndr] : 0.0;
        int64_t pini = colptr[j - 1] - 1;
        int64_t pend = pini + colnnz[j - 1] - 1;
        int64_t p = sorted_first(rowval, i, pini, pend);
        if (p > pend) {
          colnnz[j - 1] += 1;
          rowval[p] = i;
          nzval[p] = v;
        } else if (rowval[p] != i) {
          for (int64_t k = pend; k >= p; --k) {
            rowval[k + 1] = rowval[k];
            nzval[k + 1] = nzval[k];
          }
          colnnz[j - 1] += 1;
          rowval[p] = i;
          nzval[p] = v;
        } else {
          nzval[p] += v;
        }
      }
    }
  }
  /* create_from_nz (SparseMatrixCSC.jl:264-283): compact columns in place */
  int64_t k = 0;
  for (int64_t j = 0; j < ncols; ++j) {
    int64_t pini = colptr[j] - 1;
    for (int64_t p = pini; p < pini + colnnz[j]; ++p, ++k) {
      nzval[k] = nzval[p];
      rowval[k] = rowval[p];
    }
  }
  colptr[0] = 1;
  for (int64_t j = 0; j < ncols; ++j) colptr[j + 1] = colptr[j] + colnnz[j];
  free(colnnz);
  out->nrows = nrows;
  out->ncols = ncols;
  out->nnz = colptr[ncols] - 1;
  out->colptr = colptr;
  out->rowval = rowval;
  out->nzval = nzval;
  return 0;
}

/* Greedy first-fit cell colouring: cell c (in cell order) takes the smallest colour that no
 * earlier cell sharing a free dof with it holds (at most 64 colours). Cells of one colour
 * share no free dof, so their additions touch disjoint rows and columns. Returns the number
 * of colours, or -1 when 64 do not suffice. */
int orc_color_cells(int64_t ncells, int nd, const int32_t* cell_dofs, int64_t nfree,
                    int32_t* color) {
  uint64_t* used = (uint64_t*)calloc(nfree + 1, sizeof(uint64_t));
  if (!used) return -1;
  int ncol = 0;
  for (int64_t c = 0; c < ncells; ++c) {
    uint64_t forbid = 0;
    for (int a = 0; a < nd; ++a) {
      const int32_t d = cell_dofs[c * nd + a];
      if (d > 0) forbid |= used[d];
    }
    if (forbid == ~(uint64_t)0) {
      free(used);
      return -1;
    }
    int k = 0;
    while (forbid >> k & 1u) ++k;
    color[c] = k;
    if (k + 1 > ncol) ncol = k + 1;
    for (int a = 0; a < nd; ++a) {
      const int32_t d = cell_dofs[c * nd + a];
      if (d > 0) used[d] |= (uint64_t)1 << k;
    }
  }
  free(used);
  return ncol;
}

/* The assembly of orc_assemble_matrix_csc_rect (square, rows and columns from the same ids)
 * run colour by colour, the cells of one colour split over `nthreads` threads: the symbolic
 * count, the InserterCSC insertions and the vector additions of cells of one colour touch
 * disjoint columns, so no two threads write the same column. The pattern equals the serial
 * one; a value is the same sum taken in colour order, then cell order, instead of cell
 * order (equal up to rounding). The OpenMP counterpart of a multi-threaded Gridap assembly.
 * cellvecs / b may be NULL. */
int orc_assemble_csc_colored(int64_t ncells, int nd, const int32_t* cell_dofs,
                             const double* cellmats, const double* cellvecs, int64_t n,
                             int ncolors, const int64_t* color_ptr, const int64_t* color_cells,
                             int nthreads, orc_csc* out, double* b) {
  const int nt = nthreads > 0 ? nthreads : 1;
  if (ncolors < 0 || color_ptr[ncolors] != ncells) return -1;
  int64_t* colnnz = (int64_t*)calloc(n + 1, sizeof(int64_t));
  int64_t* colptr = (int64_t*)malloc(sizeof(int64_t) * (n + 1));
  if (!colnnz || !colptr) return -1;
  for (int k = 0; k < ncolors; ++k) {
#pragma omp parallel for schedule(dynamic, 512) num_threads(nt) if (nt > 1)
    for (int64_t t = color_ptr[k]; t < color_ptr[k + 1]; ++t) {
      const int32_t* rs = cell_dofs + color_cells[t] * nd;
      int cnt = 0;
      for (int li = 0; li < nd; ++li) cnt += rs[li] > 0;
      for (int lj = 0; lj < nd; ++lj)
        if (rs[lj] > 0) colnnz[rs[lj] - 1] += cnt;
    }
  }
  colptr[0] = 1;
  for (int64_t j = 0; j < n; ++j) colptr[j + 1] = colptr[j] + colnnz[j];
  const int64_t ndata = colptr[n] - 1;
  int64_t* rowval = (int64_t*)malloc(sizeof(int64_t) * (ndata > 0 ? ndata : 1));
  double* nzval = (double*)calloc(ndata > 0 ? ndata : 1, sizeof(double));
  if (!rowval || !nzval) return -1;
  memset(colnnz, 0, sizeof(int64_t) * (n + 1));
  if (b) memset(b, 0, sizeof(double) * n);
  for (int k = 0; k < ncolors; ++k) {
#pragma omp parallel for schedule(dynamic, 512) num_threads(nt) if (nt > 1)
    for (int64_t t = color_ptr[k]; t < color_ptr[k + 1]; ++t) {
      const int64_t c = color_cells[t];
      const int32_t* rs = cell_dofs + c * nd;
      const double* vs = cellmats ? cellmats + c * nd * nd : NULL;
      for (int lj = 0; lj < nd; ++lj) {
        const int64_t j = rs[lj];
        if (j <= 0) continue;
        for (int li = 0; li < nd; ++li) {
          const int64_t i = rs[li];
          if (i <= 0) continue;
          const double v = vs ? vs[li + lj * nd] : 0.0;
          const int64_t pini = colptr[j - 1] - 1;
          const int64_t pend = pini + colnnz[j - 1] - 1;
          const int64_t p = sorted_first(rowval, i, pini, pend);
          if (p > pend) {
            colnnz[j - 1] += 1;
            rowval[p] = i;
            nzval[p] = v;
          } else if (rowval[p] != i) {
            for (int64_t q = pend; q >= p; --q) {
              rowval[q + 1] = rowval[q];
              nzval[q + 1] = nzval[q];
            }
            colnnz[j - 1] += 1;
            rowval[p] = i;
            nzval[p] = v;
          } else {
            nzval[p] += v;
          }
        }
      }
      if (b && cellvecs)
        for (int li = 0; li < nd; ++li)
          if (rs[li] > 0) b[rs[li] - 1] += cellvecs[c * nd + li];
    }
  }
  int64_t w = 0;
  for (int64_t j = 0; j < n; ++j) {
    const int64_t pini = colptr[j] - 1;
    for (int64_t p = pini; p < pini + colnnz[j]; ++p, ++w) {
      nzval[w] = nzval[p];
      rowval[w] = rowval[p];
    }
  }
  colptr[0] = 1;
  for (int64_t j = 0; j < n; ++j) colptr[j + 1] = colptr[j] + colnnz[j];
  free(colnnz);
  out->nrows = n;
  out->ncols = n;
  out->nnz = colptr[n] - 1;
  out->colptr = colptr;
  out->rowval = rowval;
  out->nzval = nzval;
  return 0;
}

void orc_csc_free(orc_csc* a) {
  free(a->colptr);
  free(a->rowval);
  free(a->nzval);
  a->colptr = NULL;
  a->rowval = NULL;
  a->nzval = NULL;
}

/* Dense vector: b[i] += v for positive ids, cell order (SparseMatrixAssemblers.jl:287-316,
 * AlgebraInterfaces.jl:200-207). */
void orc_assemble_vector(int64_t ncells, int nd, const int32_t* cell_rows,
                         const double* cellvecs, double* b) {
  for (int64_t c = 0; c < ncells; ++c)
    for (int li = 0; li < nd; ++li) {
      int32_t i = cell_rows[c * nd + li];
      if (i > 0) b[i - 1] += cellvecs[c * nd + li];
    }
}

/* ====================================================================================== */
/* solver                                                                                  */
/* ====================================================================================== */

void orc_csc_mul(const orc_csc* A, const double* x, double* y) {
  memset(y, 0, sizeof(double) * A->nrows);
  for (int64_t j = 0; j < A->ncols; ++j) {
    double xj = x[j];
    for (int64_t p = A->colptr[j] - 1; p < A->colptr[j + 1] - 1; ++p)
      y[A->rowval[p] - 1] += A->nzval[p] * xj;
  }
}

/* symmetric matrix: row r = column r of the CSC */
static void sym_mul(const orc_csc* A, const double* x, double* y, int nt) {
  int64_t n = A->ncols;
  (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
  for (int64_t r = 0; r < n; ++r) {
    double s = 0.0;
    for (int64_t p = A->colptr[r] - 1; p < A->colptr[r + 1] - 1; ++p)
      s += A->nzval[p] * x[A->rowval[p] - 1];
    y[r] = s;
  }
}

static double dotp(int64_t n, const double* a, const double* b, int nt) {
  double s = 0.0;
  (void)nt;
#pragma omp parallel for schedule(static) reduction(+ : s) num_threads(nt) if (nt > 1)
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* Preconditioned conjugate gradients (Hestenes-Stiefel) with x0 = 0. This is the
 * LinearSolver a Gridap user plugs in through solve!(x, ns, b)
 * (Algebra/LinearSolvers.jl:58-129, 202-209): Gridap itself ships no Krylov method. */
int orc_pcg(const orc_csc* A, const double* b, double* x, double rtol, int maxit, int precond,
            int nthreads, double* relres) {
  int64_t n = A->nrows;
  int nt = nthreads > 0 ? nthreads : 1;
  double* r = (double*)malloc(sizeof(double) * n);
  double* z = (double*)malloc(sizeof(double) * n);
  double* p = (double*)malloc(sizeof(double) * n);
  double* q = (double*)malloc(sizeof(double) * n);
  double* dinv = (double*)malloc(sizeof(double) * n);
  if (!r || !z || !p || !q || !dinv) return -1;
  for (int64_t i = 0; i < n; ++i) {
    dinv[i] = 1.0;
    if (precond)
      for (int64_t k = A->colptr[i] - 1; k < A->colptr[i + 1] - 1; ++k)
        if (A->rowval[k] - 1 == i) dinv[i] = 1.0 / A->nzval[k];
  }
  for (int64_t i = 0; i < n; ++i) {
    x[i] = 0.0;
    r[i] = b[i];
    z[i] = dinv[i] * r[i];
    p[i] = z[i];
  }
  double bnorm = sqrt(dotp(n, b, b, nt));
  double rz = dotp(n, r, z, nt);
  double rn = bnorm;
  int it = 0;
  if (bnorm == 0.0) {
    *relres = 0.0;
    goto done;
  }
  while (it < maxit) {
    sym_mul(A, p, q, nt);
    double pq = dotp(n, p, q, nt);
    double alpha = rz / pq;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int64_t i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
    }
    ++it;
    rn = sqrt(dotp(n, r, r, nt));
    if (rn <= rtol * bnorm) break;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int64_t i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
    double rz1 = dotp(n, r, z, nt);
    double beta = rz1 / rz;
    rz = rz1;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
  }
  *relres = rn / bnorm;
done:
  free(r); free(z); free(p); free(q); free(dinv);
  return it;
}

/* ====================================================================================== */
/* simplexified Cartesian meshes, P2 tetrahedra, Witherden-Vincent quadrature, elasticity */
/* ====================================================================================== */

/* Local tets of a HEX (1-based local vertices, x fastest), the oriented simplexification of
 * the 3-cube (ReferenceFEs/ExtrusionPolytopes.jl:290-299). */
static const int ORC_HEX_TETS[6][4] = {{1, 2, 3, 7}, {1, 2, 5, 7}, {2, 3, 4, 7},
                                       {2, 4, 7, 8}, {2, 5, 6, 7}, {2, 6, 7, 8}};
/* TET edges as vertex pairs, in the order of Gridap's extrusion-polytope face generation
 * (ReferenceFEs/ExtrusionPolytopes.jl:460-531 applied to the (TET, TET, TET) extrusion). */
static const int ORC_TET_EDGES[6][2] = {{1, 2}, {1, 3}, {2, 3}, {1, 4}, {2, 4}, {3, 4}};

/* simplexify_connectivity (Geometry/Grids.jl:518-558): tet 6c+t of hex c has the hex's
 * nodes at ORC_HEX_TETS[t]. */
void orc_simplex_cells(const int64_t* part, int32_t* tet_vertices) {
  const int64_t nc = part[0] * part[1] * part[2];
  int32_t* hex = (int32_t*)malloc(sizeof(int32_t) * nc * 8);
  orc_cartesian_cell_nodes(3, part, hex);
  for (int64_t c = 0; c < nc; ++c)
    for (int t = 0; t < 6; ++t)
      for (int a = 0; a < 4; ++a)
        tet_vertices[(c * 6 + t) * 4 + a] = hex[c * 8 + ORC_HEX_TETS[t][a] - 1];
  free(hex);
}

/* Conforming P2 numbering on the simplexified box: tet edges numbered first-touch over
 * (tet, local edge) with the cells-around-vertices search of
 * Geometry/GridTopologies.jl:1184-1250; a face is Dirichlet when every one of its vertices
 * is (the labeling of Geometry/FaceLabelings.jl:590-611, face_labeling_from_vertex_filter);
 * dofs numbered vertices first, then edges, in face id order with the components of a face
 * consecutive (FESpaces/ConformingFESpaces.jl:543-636). cell_dofs: ntets x (10*ncomp),
 * comp-major over the 10 nodes (4 vertices, 6 edge midpoints in TET edge order). */
int orc_simplex_p2_numbering(const int64_t* part, int ncomp, const uint8_t* vertex_mask,
                             const uint8_t* comp_mask, int32_t* cell_dofs, int32_t* nfree,
                             int32_t* ndiri) {
  const int64_t ncells = part[0] * part[1] * part[2] * 6;
  const int64_t nverts = (part[0] + 1) * (part[1] + 1) * (part[2] + 1);
  int32_t* tv = (int32_t*)malloc(sizeof(int32_t) * ncells * 4);
  orc_simplex_cells(part, tv);
  int64_t* vptr = (int64_t*)calloc(nverts + 1, sizeof(int64_t));
  for (int64_t c = 0; c < ncells; ++c)
    for (int a = 0; a < 4; ++a) vptr[tv[c * 4 + a]] += 1;
  for (int64_t v = 0; v < nverts; ++v) vptr[v + 1] += vptr[v];
  int64_t* vfill = (int64_t*)calloc(nverts, sizeof(int64_t));
  int32_t* vcells = (int32_t*)malloc(sizeof(int32_t) * vptr[nverts]);
  for (int64_t c = 0; c < ncells; ++c)
    for (int a = 0; a < 4; ++a) {
      int64_t v = tv[c * 4 + a] - 1;
      vcells[vptr[v] + vfill[v]++] = (int32_t)c;
    }
  int32_t* ce = (int32_t*)calloc(ncells * 6, sizeof(int32_t));
  int32_t nedges = 0;
  for (int64_t c = 0; c < ncells; ++c)
    for (int e = 0; e < 6; ++e) {
      if (ce[c * 6 + e]) continue;
      const int32_t va = tv[c * 4 + ORC_TET_EDGES[e][0] - 1];
      const int32_t vb = tv[c * 4 + ORC_TET_EDGES[e][1] - 1];
      ++nedges;
      for (int64_t p = vptr[va - 1]; p < vptr[va]; ++p) {
        const int32_t c2 = vcells[p];
        int hit = 0;
        for (int a = 0; a < 4; ++a) hit |= tv[(int64_t)c2 * 4 + a] == vb;
        if (!hit) continue;
        for (int e2 = 0; e2 < 6; ++e2) {
          const int32_t wa = tv[(int64_t)c2 * 4 + ORC_TET_EDGES[e2][0] - 1];
          const int32_t wb = tv[(int64_t)c2 * 4 + ORC_TET_EDGES[e2][1] - 1];
          if ((wa == va && wb == vb) || (wa == vb && wb == va)) ce[(int64_t)c2 * 6 + e2] = nedges;
        }
      }
    }
  /* edge endpoints */
  int32_t* ev = (int32_t*)malloc(sizeof(int32_t) * 2 * (nedges + 1));
  for (int64_t c = 0; c < ncells; ++c)
    for (int e = 0; e < 6; ++e) {
      ev[2 * ce[c * 6 + e]] = tv[c * 4 + ORC_TET_EDGES[e][0] - 1];
      ev[2 * ce[c * 6 + e] + 1] = tv[c * 4 + ORC_TET_EDGES[e][1] - 1];
    }
  int32_t* vdof = (int32_t*)malloc(sizeof(int32_t) * (nverts + 1) * ncomp);
  int32_t* edof = (int32_t*)malloc(sizeof(int32_t) * (nedges + 1) * ncomp);
  int32_t nf = 0, nd = 0;
  for (int64_t v = 1; v <= nverts; ++v)
    for (int k = 0; k < ncomp; ++k) {
      const int diri = vertex_mask[v - 1] && comp_mask[k];
      vdof[v * ncomp + k] = diri ? -(++nd) : ++nf;
    }
  for (int32_t e = 1; e <= nedges; ++e)
    for (int k = 0; k < ncomp; ++k) {
      const int tagged = vertex_mask[ev[2 * e] - 1] && vertex_mask[ev[2 * e + 1] - 1];
      const int diri = tagged && comp_mask[k];
      edof[e * ncomp + k] = diri ? -(++nd) : ++nf;
    }
  const int ndc = 10 * ncomp;
  for (int64_t c = 0; c < ncells; ++c)
    for (int k = 0; k < ncomp; ++k) {
      for (int a = 0; a < 4; ++a) cell_dofs[c * ndc + k * 10 + a] = vdof[tv[c * 4 + a] * ncomp + k];
      for (int e = 0; e < 6; ++e)
        cell_dofs[c * ndc + k * 10 + 4 + e] = edof[ce[c * 6 + e] * ncomp + k];
    }
  *nfree = nf;
  *ndiri = nd;
  free(tv); free(vptr); free(vfill); free(vcells); free(ce); free(ev); free(vdof); free(edof);
  return 0;
}

/* P2 Lagrange basis on the unit tet at Gridap's nodes: vertices (0,0,0), (1,0,0), (0,1,0),
 * (0,0,1), then the midpoints of the TET edges (ReferenceFEs/CLagrangianRefFEs.jl:493-547).
 * With barycentrics l0 = 1-x-y-z, l1 = x, l2 = y, l3 = z the nodal basis is l_a (2 l_a - 1)
 * at vertex a and 4 l_a l_b at edge (a, b). phi[npts*10], dphi[npts*10*3]. */
void orc_p2tet_shapes(int npts, const double* pts, double* phi, double* dphi) {
  static const double G[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int q = 0; q < npts; ++q) {
    const double x = pts[q * 3], y = pts[q * 3 + 1], z = pts[q * 3 + 2];
    const double l[4] = {1.0 - x - y - z, x, y, z};
    for (int a = 0; a < 4; ++a) {
      if (phi) phi[q * 10 + a] = l[a] * (2.0 * l[a] - 1.0);
      if (dphi)
        for (int d = 0; d < 3; ++d) dphi[(q * 10 + a) * 3 + d] = (4.0 * l[a] - 1.0) * G[a][d];
    }
    for (int e = 0; e < 6; ++e) {
      const int a = ORC_TET_EDGES[e][0] - 1, b = ORC_TET_EDGES[e][1] - 1;
      if (phi) phi[q * 10 + 4 + e] = 4.0 * l[a] * l[b];
      if (dphi)
        for (int d = 0; d < 3; ++d)
          dphi[(q * 10 + 4 + e) * 3 + d] = 4.0 * (G[a][d] * l[b] + l[a] * G[b][d]);
    }
  }
}

/* The 14-point degree-5 symmetric rule of Witherden & Vincent (2015) on the unit tet, which
 * Gridap uses for degrees 4 and 5 (ReferenceFEs/WitherdenVincentQuadratures.jl:367-520,
 * Quadratures.jl:157-182): two S31 orbits (barycentrics (a,a,a,1-3a) and permutations) and
 * one S22 orbit ((b,b,1/2-b,1/2-b) and permutations). The orbit parameters and weights are
 * the solution of the degree-5 moment equations, found here by Gauss-Newton in extended
 * precision from a start near the published values; points are listed in Gridap's orbit
 * expansion order and the weights sum to 1/6. pts[14*3], w[14]. Returns the residual. */
static void wv_points(const long double* u, long double P[14][3], long double W[14],
                      long double dP[14][3][6], long double dW[14][6]) {
  int r = 0;
  memset(dP, 0, sizeof(long double) * 14 * 3 * 6);
  memset(dW, 0, sizeof(long double) * 14 * 6);
  for (int o = 0; o < 2; ++o) {
    const long double a = u[o], c = 1.0L - 3.0L * a;
    /* [-1,1] pattern (s,s,t), (s,t,s), (t,s,s), (s,s,s): s <-> a, t <-> c */
    const int pat[4][3] = {{0, 0, 1}, {0, 1, 0}, {1, 0, 0}, {0, 0, 0}};
    for (int k = 0; k < 4; ++k, ++r) {
      for (int d = 0; d < 3; ++d) {
        P[r][d] = pat[k][d] ? c : a;
        dP[r][d][o] = pat[k][d] ? -3.0L : 1.0L;
      }
      W[r] = u[3 + o];
      dW[r][3 + o] = 1.0L;
    }
  }
  {
    const long double b = u[2], e = 0.5L - b;
    /* (s,t,t), (t,s,t), (s,s,t), (s,t,s), (t,s,s), (t,t,s): s <-> b, t <-> 1/2-b */
    const int pat[6][3] = {{0, 1, 1}, {1, 0, 1}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0}, {1, 1, 0}};
    for (int k = 0; k < 6; ++k, ++r) {
      for (int d = 0; d < 3; ++d) {
        P[r][d] = pat[k][d] ? e : b;
        dP[r][d][2] = pat[k][d] ? -1.0L : 1.0L;
      }
      W[r] = u[5];
      dW[r][5] = 1.0L;
    }
  }
}

static long double lpow(long double x, int n) {
  long double r = 1.0L;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

static long double lfact(int n) {
  long double r = 1.0L;
  for (int i = 2; i <= n; ++i) r *= i;
  return r;
}

double orc_wv_tet_degree5(double* pts, double* w) {
  long double u[6] = {0.31L, 0.09L, 0.045L, 0.0188L, 0.0122L, 0.0071L};
  long double P[14][3], W[14], dP[14][3][6], dW[14][6];
  long double res = 0.0L;
  for (int it = 0; it < 60; ++it) {
    wv_points(u, P, W, dP, dW);
    long double JtJ[6][6] = {{0}}, Jtr[6] = {0};
    res = 0.0L;
    for (int p = 0; p <= 5; ++p)
      for (int q = 0; p + q <= 5; ++q)
        for (int s = 0; p + q + s <= 5; ++s) {
          const long double exact = lfact(p) * lfact(q) * lfact(s) / lfact(p + q + s + 3);
          long double f = -exact, g[6] = {0};
          for (int k = 0; k < 14; ++k) {
            const long double m = lpow(P[k][0], p) * lpow(P[k][1], q) * lpow(P[k][2], s);
            f += W[k] * m;
            const long double dm[3] = {
                p ? p * lpow(P[k][0], p - 1) * lpow(P[k][1], q) * lpow(P[k][2], s) : 0.0L,
                q ? q * lpow(P[k][0], p) * lpow(P[k][1], q - 1) * lpow(P[k][2], s) : 0.0L,
                s ? s * lpow(P[k][0], p) * lpow(P[k][1], q) * lpow(P[k][2], s - 1) : 0.0L};
            for (int j = 0; j < 6; ++j)
              g[j] += dW[k][j] * m +
                      W[k] * (dm[0] * dP[k][0][j] + dm[1] * dP[k][1][j] + dm[2] * dP[k][2][j]);
          }
          res += f * f;
          for (int i = 0; i < 6; ++i) {
            Jtr[i] += g[i] * f;
            for (int j = 0; j < 6; ++j) JtJ[i][j] += g[i] * g[j];
          }
        }
    /* solve JtJ d = -Jtr (Gaussian elimination with partial pivoting) */
    long double M[6][7];
    for (int i = 0; i < 6; ++i) {
      for (int j = 0; j < 6; ++j) M[i][j] = JtJ[i][j];
      M[i][6] = -Jtr[i];
    }
    for (int c = 0; c < 6; ++c) {
      int piv = c;
      for (int i = c + 1; i < 6; ++i)
        if (fabsl(M[i][c]) > fabsl(M[piv][c])) piv = i;
      for (int j = 0; j < 7; ++j) {
        long double t = M[c][j];
        M[c][j] = M[piv][j];
        M[piv][j] = t;
      }
      for (int i = c + 1; i < 6; ++i) {
        const long double f = M[i][c] / M[c][c];
        for (int j = c; j < 7; ++j) M[i][j] -= f * M[c][j];
      }
    }
    long double d[6];
    for (int i = 5; i >= 0; --i) {
      long double s = M[i][6];
      for (int j = i + 1; j < 6; ++j) s -= M[i][j] * d[j];
      d[i] = s / M[i][i];
    }
    long double dn = 0.0L;
    for (int i = 0; i < 6; ++i) {
      u[i] += d[i];
      dn += fabsl(d[i]);
    }
    if (dn < 1e-30L) break;
  }
  wv_points(u, P, W, dP, dW);
  for (int k = 0; k < 14; ++k) {
    for (int d = 0; d < 3; ++d) pts[k * 3 + d] = (double)P[k][d];
    w[k] = (double)W[k];
  }
  return (double)sqrtl(res);
}

/* Isotropic linear elasticity on P2 tets with affine (P1) geometry, following Gridap's
 * per-quadrature-point steps: Jt = sum_a grad phi1_a (x) x_a over the 4 vertices
 * (Geometry/Grids.jl:237-241), grad phi = inv(Jt) . grad phi_hat (Fields/FieldsInterfaces.jl
 * :98-106), eps(u) = symmetric part of grad u for u = phi e_comp (Fields/DiffOperators.jl:48),
 * sigma = lambda tr(eps) I + 2 mu eps, a = eps(v) : sigma(u), K_ij += a |det Jt| w_q
 * (Fields/FieldsInterfaces.jl:708-720); b_i += (f . v_i) |det Jt| w_q. Local dofs are
 * comp-major: dof k*10 + n is node n, component k. lame[2*ncells] = (lambda, mu) per cell;
 * f[3] constant body force. cellmats[ncells*900] column-major, cellvecs[ncells*30]. */
int orc_p2tet_cell_arrays_elasticity(int64_t ncells, const int32_t* tet_vertices,
                                     const double* coords, const double* lame, int nq,
                                     const double* qx, const double* qw, const double* f,
                                     double* cellmats, double* cellvecs) {
  double* phi = (double*)malloc(sizeof(double) * nq * 10);
  double* dphi = (double*)malloc(sizeof(double) * nq * 10 * 3);
  orc_p2tet_shapes(nq, qx, phi, dphi);
  static const double G1[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  int bad = 0;
  /* cells are independent (see orc_q2_cell_arrays_diffusion) */
#pragma omp parallel for schedule(dynamic, 64) num_threads(g_cell_threads) if (g_cell_threads > 1)
  for (int64_t c = 0; c < ncells; ++c) {
    double Jt[9] = {0}, iJt[9];
    for (int a = 0; a < 4; ++a) {
      const double* xa = coords + (int64_t)(tet_vertices[c * 4 + a] - 1) * 3;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) Jt[k * 3 + l] += G1[a][k] * xa[l];
    }
    const double dJ = det_t(3, Jt);
    if (!(dJ > 0.0) && !(dJ < 0.0)) {
#pragma omp atomic write
      bad = 1;
      continue;
    }
    inv_t(3, Jt, iJt);
    const double lam = lame[2 * c], mu = lame[2 * c + 1];
    double* K = cellmats ? cellmats + c * 900 : NULL;
    double* bv = cellvecs ? cellvecs + c * 30 : NULL;
    if (K) memset(K, 0, sizeof(double) * 900);
    if (bv) memset(bv, 0, sizeof(double) * 30);
    for (int q = 0; q < nq; ++q) {
      const double dV = fabs(dJ) * qw[q];
      double g[10][3];
      for (int n = 0; n < 10; ++n)
        for (int k = 0; k < 3; ++k) {
          double s = 0.0;
          for (int l = 0; l < 3; ++l) s += iJt[k * 3 + l] * dphi[(q * 10 + n) * 3 + l];
          g[n][k] = s;
        }
      if (K) {
        for (int j = 0; j < 30; ++j) {
          const int cj = j / 10, nj = j % 10;
          /* grad u: (grad u)_{ab} = d_a phi delta_{cj b}; eps = sym; sigma */
          double eu[3][3], su[3][3];
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
              eu[a][b] = 0.5 * ((b == cj ? g[nj][a] : 0.0) + (a == cj ? g[nj][b] : 0.0));
          const double tr = eu[0][0] + eu[1][1] + eu[2][2];
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) su[a][b] = (a == b ? lam * tr : 0.0) + 2.0 * mu * eu[a][b];
          for (int i = 0; i < 30; ++i) {
            const int ci = i / 10, ni = i % 10;
            double s = 0.0;
            for (int a = 0; a < 3; ++a)
              for (int b = 0; b < 3; ++b) {
                const double ev =
                    0.5 * ((b == ci ? g[ni][a] : 0.0) + (a == ci ? g[ni][b] : 0.0));
                s += ev * su[a][b];
              }
            K[i + j * 30] += s * dV;
          }
        }
      }
      if (bv && f)
        for (int i = 0; i < 30; ++i) bv[i] += (f[i / 10] * phi[q * 10 + i % 10]) * dV;
    }
  }
  free(phi);
  free(dphi);
  return bad ? -1 : 0;
}
