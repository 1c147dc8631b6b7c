// gfe_boundary.cu -- boundary-integral terms on the facets of a Cartesian box, Q1 and Q2:
// load vectors  int_Gamma g v  and  int_Gamma g (n.grad v)  (Neumann data, the Nitsche right
// hand side) and facet matrices
//   int_Gamma c0 v u + c1 v (n.grad u) + c2 (n.grad v) u + c3 (n.grad v)(n.grad u)
// (the Nitsche and Robin terms) added into an assembled CSR matrix.
//
// Gridap integrates over a BoundaryTriangulation: every selected boundary facet carries the
// cell array of its owner cell evaluated at the facet's quadrature points
// (Geometry/BoundaryTriangulations.jl:13-35,150-205), and the assembly adds those arrays with
// the owner cell's dof ids in facet order (FESpaces/SparseMatrixAssemblers.jl:214-316).
// On a Cartesian box every facet with the same local facet index has the same shape-function
// values, normal and Jacobian, so host tables per local facet (2D of them) hold everything:
// phi_i and n.grad(phi_i) at the facet's tensor Gauss points mapped into the cell (the
// facet's spanned axes in increasing order carry the facet coordinates, its normal axis is
// fixed at 0 or 1), and |J_F|, the product of the cell sizes along the spanned axes. Vectors:
// one thread per facet forms sum_q g_q op(phi_i)(q) w_q |J_F| and the volume assembly's
// row gather adds them into b in facet order. Matrices: one thread per matrix row walks the
// row's facet references in facet order and adds the facet matrix rows at their CSR
// positions (binary search in the row's sorted column list); Dirichlet columns give the lift
// b_i -= M_ij u_D_j when the problem carries Dirichlet values.
#include <cmath>
#include <vector>

#include "gfe_internal.h"

namespace gfe {
namespace {

// local facet lf of the D-cube in Gridap's face order: normal axis and side
__host__ __device__ inline void facet_axis(int D, int lf, int* axis, int* side) {
  // faces of dimension D-1 come ordered by the fixed (normal) axis from the last to the
  // first, lower side before upper: 3-D (z-, z+, y-, y+, x-, x+), 2-D (y-, y+, x-, x+)
  *axis = D - 1 - lf / 2;
  *side = lf & 1;
}

__device__ inline bool facet_ok(int32_t c, int32_t lf, int64_t ncells, int nfacet_types) {
  return c >= 0 && c < ncells && lf >= 0 && lf < nfacet_types;
}

// facet vectors (nd per facet) and their rows (the owner cell's dof ids)
__global__ void k_facet_vectors(int64_t nf, int nd, int nqf, const int32_t* __restrict__ fcell,
                                const int32_t* __restrict__ flface,
                                const int32_t* __restrict__ cell_ids,
                                const double* __restrict__ tab,  // [2D][nqf][nd] op(phi)*w
                                const double* __restrict__ jac,  // [2D] facet |J_F|
                                int src_kind, const double* __restrict__ src, int64_t ncells,
                                int nfacet_types, double* __restrict__ fvec,
                                int32_t* __restrict__ frows, DevError* err) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int32_t c = fcell[f];
  const int32_t lf = flface[f];
  if (!facet_ok(c, lf, ncells, nfacet_types)) {
    if (atomicCAS(&err->code, 0, GFE_ERR_INVALID_ARGUMENT) == 0) err->index = f;
    for (int i = 0; i < nd; ++i) {  // an inert facet: no rows, no values
      fvec[f * nd + i] = 0.0;
      frows[f * nd + i] = 0;
    }
    return;
  }
  const double* t = tab + (int64_t)lf * nqf * nd;
  for (int i = 0; i < nd; ++i) {
    double s = 0.0;
    for (int q = 0; q < nqf; ++q) {
      const double g = src_kind == GFE_SRC_CONST ? src[0] : src[f * nqf + q];
      s += g * t[q * nd + i];
    }
    fvec[f * nd + i] = s * jac[lf];
    frows[f * nd + i] = cell_ids[(int64_t)c * nd + i];
  }
}

// rows of the facets only (matrix terms)
__global__ void k_facet_rows(int64_t nf, int nd, const int32_t* __restrict__ fcell,
                             const int32_t* __restrict__ flface,
                             const int32_t* __restrict__ cell_ids, int64_t ncells,
                             int nfacet_types, int32_t* __restrict__ frows, DevError* err) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int32_t c = fcell[f];
  const bool ok = facet_ok(c, flface[f], ncells, nfacet_types);
  if (!ok && atomicCAS(&err->code, 0, GFE_ERR_INVALID_ARGUMENT) == 0) err->index = f;
  for (int i = 0; i < nd; ++i) frows[f * nd + i] = ok ? cell_ids[(int64_t)c * nd + i] : 0;
}

// A_rj += M[lf][li][lj] over the row's facet references (ascending facet, so each entry
// receives its facet terms in facet order); Dirichlet columns: b_r -= M u_D per facet.
__global__ void k_facet_matrix_rows(int64_t nrows, int nd, const int64_t* __restrict__ ref_ptr,
                                    const int32_t* __restrict__ refs,
                                    const int32_t* __restrict__ fcell,
                                    const int32_t* __restrict__ flface,
                                    const int32_t* __restrict__ cell_ids,
                                    const double* __restrict__ mtab,  // [2D][nd][nd]
                                    const int32_t* __restrict__ rowptr,
                                    const int32_t* __restrict__ colval, double* __restrict__ val,
                                    const double* __restrict__ uD, int64_t ndiri,
                                    double* __restrict__ b, DevError* err) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int32_t lo = rowptr[r], hi = rowptr[r + 1];
  for (int64_t q = ref_ptr[r]; q < ref_ptr[r + 1]; ++q) {
    const int32_t e = refs[q];
    const int32_t f = e / nd;
    const int li = e - f * nd;
    const int32_t c = fcell[f];
    const double* M = mtab + ((int64_t)flface[f] * nd + li) * nd;
    double lift = 0.0;
    for (int lj = 0; lj < nd; ++lj) {
      const int32_t col = cell_ids[(int64_t)c * nd + lj];
      if (col > 0) {
        int32_t a = lo, z = hi;  // first position with colval >= col-1
        while (a < z) {
          const int32_t m = (a + z) >> 1;
          if (colval[m] < col - 1) a = m + 1; else z = m;
        }
        if (a >= hi || colval[a] != col - 1) {  // column outside the pattern
          if (atomicCAS(&err->code, 0, GFE_ERR_INVALID_ARGUMENT) == 0) err->index = r;
          continue;
        }
        val[a] += M[lj];
      } else if (col < 0 && uD) {
        const int64_t k = -(int64_t)col - 1;
        if (k >= ndiri) {
          if (atomicCAS(&err->code, 0, GFE_ERR_INVALID_ARGUMENT) == 0) err->index = r;
          continue;
        }
        lift -= M[lj] * uD[k];
      }
    }
    if (uD && b) b[r] += lift;
  }
}

__global__ void k_check_finite_b(const double* __restrict__ v, int64_t n, DevError* err) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (!isfinite(v[i]) && atomicCAS(&err->code, 0, GFE_ERR_NONFINITE) == 0) err->index = i;
}

}  // namespace

// Per local facet: shape values phi[lf][q][i], outward normal derivatives dn[lf][q][i]
// (sign * dphi/dx_axis with dx = h_axis dxi), the facet rule's weights w[q] and |J_F|[lf].
struct FacetTables {
  int D = 0, nq = 0, nd = 0;
  std::vector<double> phi, dn, w, jac;
};

static int facet_tables(const gfe_problem* p, int degree, FacetTables& t) {
  const int D = p->dim;
  const bool q2 = p->reffe == GFE_REFFE_Q2;
  std::vector<double> fx;
  GFE_TRY(tensor_quadrature(D - 1, degree, fx, t.w));  // Gauss rule of the facet polytope
  const int nq = (int)t.w.size();
  const int nn = q2 ? (D == 2 ? 9 : 27) : (1 << D);
  double h[3];
  for (int d = 0; d < D; ++d) {
    h[d] = (p->domain[2 * d + 1] - p->domain[2 * d]) / (double)p->partition[d];
    if (!(h[d] > 0.0))
      return set_error(GFE_ERR_INVALID_ARGUMENT, "boundary terms: empty box along axis %d", d);
  }
  t.D = D;
  t.nq = nq;
  t.nd = nn;
  t.phi.assign((size_t)2 * D * nq * nn, 0.0);
  t.dn.assign((size_t)2 * D * nq * nn, 0.0);
  t.jac.assign(2 * D, 1.0);
  for (int lf = 0; lf < 2 * D; ++lf) {
    int axis, side;
    facet_axis(D, lf, &axis, &side);
    for (int d = 0; d < D; ++d)
      if (d != axis) t.jac[lf] *= h[d];
    std::vector<double> pts((size_t)nq * D);
    for (int q = 0; q < nq; ++q) {
      int k = 0;
      for (int d = 0; d < D; ++d)
        pts[(size_t)q * D + d] = d == axis ? (double)side : fx[(size_t)q * (D - 1) + k++];
    }
    std::vector<double> phi, dphi;
    if (q2) {
      q2_shapes(D, nq, pts.data(), phi, dphi);
    } else {  // Q1: prod_d (x_d or 1 - x_d), vertex a has coordinate bit d = (a >> d) & 1
      phi.assign((size_t)nq * nn, 1.0);
      dphi.assign((size_t)nq * nn * D, 1.0);
      for (int q = 0; q < nq; ++q)
        for (int a = 0; a < nn; ++a)
          for (int d = 0; d < D; ++d) {
            const double x = pts[(size_t)q * D + d];
            const bool hi = (a >> d) & 1;
            phi[(size_t)q * nn + a] *= hi ? x : 1.0 - x;
            for (int k = 0; k < D; ++k)
              dphi[((size_t)q * nn + a) * D + k] *= k == d ? (hi ? 1.0 : -1.0) : (hi ? x : 1.0 - x);
          }
    }
    const double sgn = side ? 1.0 : -1.0;
    for (int q = 0; q < nq; ++q)
      for (int i = 0; i < nn; ++i) {
        const size_t o = ((size_t)lf * nq + q) * nn + i;
        t.phi[o] = phi[(size_t)q * nn + i];
        t.dn[o] = sgn * dphi[((size_t)q * nn + i) * D + axis] / h[axis];
      }
  }
  return GFE_OK;
}

static int check_boundary_problem(const gfe_problem* p, const char* who) {
  if (!p->cell_dof_ids)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: bad arguments", who);
  // the facets are the box's: axis-aligned with the partition's spacing in both geometries
  // (node jitter of a Cartesian model moves interior nodes only)
  if ((p->dim != 2 && p->dim != 3) || p->ncomp != 1 ||
      (p->reffe != GFE_REFFE_Q1 && p->reffe != GFE_REFFE_Q2))
    return set_error(GFE_ERR_UNSUPPORTED, "%s: scalar Q1/Q2 on Cartesian boxes", who);
  const int nn = p->reffe == GFE_REFFE_Q2 ? (p->dim == 2 ? 9 : 27) : (1 << p->dim);
  if (p->nd != nn) return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: nd mismatch", who);
  return GFE_OK;
}

}  // namespace gfe

using namespace gfe;

namespace {

// facet list, cell ids and (optionally) the source on the device
struct FacetViews {
  const int32_t *cells = nullptr, *lfaces = nullptr, *ids = nullptr;
};

int facet_views(gfe_ctx* ctx, const gfe_problem* p, int64_t nfacets, const int32_t* fc,
                const int32_t* fl, FacetViews& v) {
  const void *vc, *vl, *vi;
  GFE_TRY(device_view(ctx, fc, sizeof(int32_t) * nfacets, SCR_TMP2, &vc));
  GFE_TRY(device_view(ctx, fl, sizeof(int32_t) * nfacets, SCR_TMP3, &vl));
  GFE_TRY(device_view(ctx, p->cell_dof_ids, sizeof(int32_t) * (size_t)p->ncells * p->nd,
                      SCR_CELLIDS, &vi));
  v.cells = (const int32_t*)vc;
  v.lfaces = (const int32_t*)vl;
  v.ids = (const int32_t*)vi;
  return GFE_OK;
}

}  // namespace

extern "C" int gfe_assemble_boundary_vector(gfe_ctx* ctx, const gfe_problem* p, int64_t nfacets,
                                            const int32_t* facet_cells,
                                            const int32_t* facet_lfaces, int32_t degree,
                                            int32_t test_op, int32_t source_kind,
                                            const double* source, int64_t source_len,
                                            double* b) {
  NvtxRange nvtx_range("gfe_assemble_boundary_vector");
  clear_error();
  const char* who = "gfe_assemble_boundary_vector";
  if (!ctx || !p || !b || nfacets < 0 || (nfacets > 0 && (!facet_cells || !facet_lfaces)) ||
      !source)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: bad arguments", who);
  GFE_TRY(check_boundary_problem(p, who));
  if (source_kind != GFE_SRC_CONST && source_kind != GFE_SRC_QPOINT)
    return set_error(GFE_ERR_UNSUPPORTED, "%s: constant or quadrature-point g", who);
  if (test_op != GFE_BOP_VALUE && test_op != GFE_BOP_NORMAL_GRAD)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: test_op %d", who, test_op);
  DeviceGuard g(ctx->device);
  FacetTables t;
  GFE_TRY(facet_tables(p, degree, t));
  const int nd = t.nd, nqf = t.nq, D = t.D;
  if (source_kind == GFE_SRC_CONST ? source_len < 1 : source_len != nfacets * nqf)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: source needs 1 or nfacets*%d values", who,
                     nqf);
  // op(phi_i) * w_q per local facet
  std::vector<double> tab((size_t)2 * D * nqf * nd);
  const std::vector<double>& op = test_op == GFE_BOP_VALUE ? t.phi : t.dn;
  for (int lf = 0; lf < 2 * D; ++lf)
    for (int q = 0; q < nqf; ++q)
      for (int i = 0; i < nd; ++i) {
        const size_t o = ((size_t)lf * nqf + q) * nd + i;
        tab[o] = op[o] * t.w[q];
      }
  const size_t nb = sizeof(double) * (size_t)(p->nfree > 0 ? p->nfree : 1);
  const bool bdev = is_device_ptr(b);
  double* db = b;
  if (!bdev) {
    GFE_TRY(ctx->scratch[SCR_VEC_B].reserve(nb));
    db = ctx->scratch[SCR_VEC_B].as<double>();
    GFE_CUDA_TRY(cudaMemcpyAsync(db, b, sizeof(double) * p->nfree, cudaMemcpyHostToDevice,
                                 ctx->stream));
  }
  if (nfacets > 0) {
    FacetViews fv;
    GFE_TRY(facet_views(ctx, p, nfacets, facet_cells, facet_lfaces, fv));
    const void* vs;
    const int64_t ns = source_kind == GFE_SRC_CONST ? 1 : source_len;
    GFE_TRY(device_view(ctx, source, sizeof(double) * ns, SCR_SRC, &vs));
    k_check_finite_b<<<grid_for(ns, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
        (const double*)vs, ns, ctx->d_err);
    DevBuf work(ctx);
    GFE_TRY(work.reserve(sizeof(double) * (tab.size() + t.jac.size() + (size_t)nfacets * nd) +
                         sizeof(int32_t) * (size_t)nfacets * nd + 256));
    double* dtab = work.as<double>();
    double* djac = dtab + tab.size();
    double* fvec = djac + t.jac.size();
    int32_t* frows = reinterpret_cast<int32_t*>(fvec + (size_t)nfacets * nd);
    GFE_CUDA_TRY(cudaMemcpyAsync(dtab, tab.data(), sizeof(double) * tab.size(),
                                 cudaMemcpyHostToDevice, ctx->stream));
    GFE_CUDA_TRY(cudaMemcpyAsync(djac, t.jac.data(), sizeof(double) * t.jac.size(),
                                 cudaMemcpyHostToDevice, ctx->stream));
    k_facet_vectors<<<grid_for(nfacets, 128), 128, 0, ctx->stream>>>(
        nfacets, nd, nqf, fv.cells, fv.lfaces, fv.ids, dtab, djac, source_kind,
        (const double*)vs, p->ncells, 2 * D, fvec, frows, ctx->d_err);
    ctx->launches += 2;
    GFE_CUDA_TRY(cudaGetLastError());
    GFE_TRY(check_device_error(ctx, "gfe_assemble_boundary_vector (facets)"));
    GFE_TRY(assemble_cellvecs(ctx, nfacets, nd, frows, fvec, p->nfree, db));
    // the host tables must outlive the copies
    GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  }
  if (!bdev) GFE_TRY(copy_out(ctx, b, db, sizeof(double) * p->nfree));
  return check_device_error(ctx, who);
}

extern "C" int gfe_assemble_boundary_matrix(gfe_ctx* ctx, const gfe_problem* p, gfe_matrix* A,
                                            double* b, int64_t nfacets,
                                            const int32_t* facet_cells,
                                            const int32_t* facet_lfaces, int32_t degree,
                                            const double* coefs) {
  NvtxRange nvtx_range("gfe_assemble_boundary_matrix");
  clear_error();
  const char* who = "gfe_assemble_boundary_matrix";
  if (!ctx || !p || !A || !coefs || A->ctx != ctx || nfacets < 0 ||
      (nfacets > 0 && (!facet_cells || !facet_lfaces)))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: bad arguments", who);
  GFE_TRY(check_boundary_problem(p, who));
  if (A->nrows != p->nfree || A->nd != p->nd ||
      A->cols_per_cell() != p->nd)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: matrix does not match the problem", who);
  for (int k = 0; k < 4; ++k)
    if (!std::isfinite(coefs[k]))
      return set_error(GFE_ERR_NONFINITE, "%s: coefficient %d is not finite", who, k);
  const bool lift = p->dirichlet_values && p->ndirichlet > 0 && b;
  DeviceGuard g(ctx->device);
  GFE_TRY(ensure_values(ctx, A));
  A->zf_values = false;  // facet terms add into the values
  FacetTables t;
  GFE_TRY(facet_tables(p, degree, t));
  const int nd = t.nd, nq = t.nq, D = t.D;
  // facet matrices: M[lf][i][j] = sum_q (c0 phi_i phi_j + c1 phi_i dn_j + c2 dn_i phi_j
  //                                      + c3 dn_i dn_j) w_q |J_F|   (i test, j trial)
  std::vector<double> mtab((size_t)2 * D * nd * nd, 0.0);
  for (int lf = 0; lf < 2 * D; ++lf)
    for (int q = 0; q < nq; ++q) {
      const double* ph = t.phi.data() + ((size_t)lf * nq + q) * nd;
      const double* dn = t.dn.data() + ((size_t)lf * nq + q) * nd;
      for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j) {
          const double integrand = coefs[0] * ph[i] * ph[j] + coefs[1] * ph[i] * dn[j] +
                                   coefs[2] * dn[i] * ph[j] + coefs[3] * dn[i] * dn[j];
          mtab[((size_t)lf * nd + i) * nd + j] += integrand * t.w[q] * t.jac[lf];
        }
    }
  // the values change: drop the solver's derived copies
  A->mf_state = 0;
  A->plan_valid = false;
  A->dia_checked = false;
  if (nfacets == 0) return GFE_OK;
  FacetViews fv;
  GFE_TRY(facet_views(ctx, p, nfacets, facet_cells, facet_lfaces, fv));
  double* db = nullptr;
  const double* duD = nullptr;
  const bool bdev = b && is_device_ptr(b);
  if (lift) {
    const void* vu;
    GFE_TRY(device_view(ctx, p->dirichlet_values, sizeof(double) * p->ndirichlet, SCR_SRC,
                        &vu));
    duD = (const double*)vu;
    db = b;
    if (!bdev) {
      GFE_TRY(ctx->scratch[SCR_VEC_B].reserve(sizeof(double) * (p->nfree > 0 ? p->nfree : 1)));
      db = ctx->scratch[SCR_VEC_B].as<double>();
      GFE_CUDA_TRY(cudaMemcpyAsync(db, b, sizeof(double) * p->nfree, cudaMemcpyHostToDevice,
                                   ctx->stream));
    }
  }
  DevBuf work(ctx);
  GFE_TRY(work.reserve(sizeof(double) * mtab.size() + sizeof(int32_t) * (size_t)nfacets * nd +
                       256));
  double* dm = work.as<double>();
  int32_t* frows = reinterpret_cast<int32_t*>(dm + mtab.size());
  GFE_CUDA_TRY(cudaMemcpyAsync(dm, mtab.data(), sizeof(double) * mtab.size(),
                               cudaMemcpyHostToDevice, ctx->stream));
  k_facet_rows<<<grid_for(nfacets, 128), 128, 0, ctx->stream>>>(
      nfacets, nd, fv.cells, fv.lfaces, fv.ids, p->ncells, 2 * D, frows, ctx->d_err);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  GFE_TRY(check_device_error(ctx, "gfe_assemble_boundary_matrix (facets)"));
  // row -> (facet, local row) references in facet order
  gfe_matrix T;
  T.ctx = ctx;
  T.cell_rows.owner = T.ref_ptr.owner = T.refs.owner = ctx;
  T.nrows = A->nrows;
  T.ncols = A->ncols;
  T.nd = nd;
  T.ncells = nfacets;
  const size_t idsz = sizeof(int32_t) * (size_t)nfacets * nd;
  GFE_TRY(T.cell_rows.reserve(idsz));
  GFE_CUDA_TRY(cudaMemcpyAsync(T.cell_rows.ptr, frows, idsz, cudaMemcpyDeviceToDevice,
                               ctx->stream));
  GFE_TRY(build_refs(ctx, &T));
  k_facet_matrix_rows<<<grid_for(A->nrows, 128), 128, 0, ctx->stream>>>(
      A->nrows, nd, T.ref_ptr.as<int64_t>(), T.refs.as<int32_t>(), fv.cells, fv.lfaces, fv.ids,
      dm, A->rowptr.as<int32_t>(), A->colval.as<int32_t>(), A->val.as<double>(), duD,
      lift ? p->ndirichlet : 0, db, ctx->d_err);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  // the host table must outlive its copy
  GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (lift && !bdev) GFE_TRY(copy_out(ctx, b, db, sizeof(double) * p->nfree));
  return check_device_error(ctx, who);
}
