// gfe_multifield.cu -- cell integrals of multi-field weak forms and their assembly.
//
// A MultiFieldFESpace (MultiField/MultiFieldFESpaces.jl) couples several Lagrangian fields
// on the same cells; its cell matrices are blocks (test field i, trial field j), each the
// quadrature sum of contractions of basis operators (value, gradient, divergence), e.g.
// Stokes' grad(v) : grad(u) - (div v) p + q (div u). Here one pass over the cells:
//
//   1. k_mf_geometry:  per (cell, quadrature point) the weight w_q |det J| and J^-T of the
//                      (multi)linear cell map;
//   2. k_mf_cellmats:  per cell (one block of threads) the physical gradients of every field
//                      at every point in shared memory, then each entry of the block's cell
//                      matrix (column-major, ndr x ndc) as a sum over points of the terms;
//   3. k_mf_cellvecs:  per cell the linear terms, minus K_cell u_D over the cell's Dirichlet
//                      columns (the lift of AttachDirichletMap, CellData/AttachDirichlet.jl:
//                      59-110), in the cell;
//   4. the row-gather numeric loops of the single-field path on those stored cell arrays:
//      each matrix and vector entry receives its cells' contributions in ascending cell
//      order, as Gridap's assembly of the ArrayBlock cell arrays does.
#include "gfe_internal.h"

namespace gfe {
namespace {

constexpr int kMfBlock = 128;
constexpr int kMaxFields = 8;
constexpr int kMaxTerms = 32;

struct MfField {
  int ncomp, nnodes, nd;  // nd = ncomp * nnodes
  const double* shapes;   // nq x nnodes
  const double* grads;    // nq x nnodes x dim
};

struct MfTerm {
  int test_field, trial_field, test_op, trial_op;
  double coef;
  const double* cell_coef;
  const double* qdata;
  int qdata_ncomp;
};

struct MfArgs {
  int dim, nq;
  int64_t ncells;
  int nfields, nterms;
  MfField f[kMaxFields];
  MfTerm t[kMaxTerms];
  // the block: row fields then column fields, local dof -> (field, comp, node)
  int nrf, ncf;
  int rf[kMaxFields], cf[kMaxFields];
  int ndr, ndc;
  // per-cell shared layout: geometry (nq * (1 + dim^2)), then the physical gradients of the
  // fields in use (pg_off[f] doubles in, nq * nnodes * dim each; -1 when unused)
  int pg_off[kMaxFields];
  int smem_doubles;
};

__device__ __forceinline__ void local_dof(const MfArgs& a, const int* fl, int nf, int l,
                                          int* field, int* comp, int* node) {
  int k = 0;
  while (k + 1 < nf && l >= a.f[fl[k]].nd) {
    l -= a.f[fl[k]].nd;
    ++k;
  }
  const MfField& F = a.f[fl[k]];
  *field = fl[k];
  *comp = l / F.nnodes;
  *node = l - *comp * F.nnodes;
}

// w_q |J| and J^-T per (cell, point): geo[(cell*nq + q) * (1 + D*D)] = w|J|, then J^-T row
// major. J[d][e] = dx_d / dxi_e = sum_a X_a[d] dN_a/dxi_e.
__global__ void k_mf_geometry(int dim, int64_t ncells, int nq, int64_t nnodes,
                              const double* __restrict__ coords,
                              const int32_t* __restrict__ cell_nodes,
                              const double* __restrict__ qw, const double* __restrict__ gg,
                              double* __restrict__ geo, DevError* err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncells * nq) return;
  const int64_t cell = i / nq;
  const int q = (int)(i - cell * nq);
  const int nv = 1 << dim;
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int a = 0; a < nv; ++a) {
    const int64_t node = (int64_t)cell_nodes[cell * nv + a] - 1;
    if (node < 0 || node >= nnodes) {
      if (atomicCAS(&err->code, 0, GFE_ERR_INVALID_ARGUMENT) == 0) err->index = cell;
      return;
    }
    for (int d = 0; d < dim; ++d) {
      const double x = coords[node * dim + d];
      for (int e = 0; e < dim; ++e) J[d][e] += x * gg[((int64_t)q * nv + a) * dim + e];
    }
  }
  double det, inv[3][3];
  if (dim == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    inv[0][0] = J[1][1] / det;
    inv[0][1] = -J[0][1] / det;
    inv[1][0] = -J[1][0] / det;
    inv[1][1] = J[0][0] / det;
  } else {
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    inv[0][0] = c00 / det;
    inv[1][0] = c01 / det;
    inv[2][0] = c02 / det;
    inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  }
  if (!(det != 0.0) || !isfinite(det)) {
    if (atomicCAS(&err->code, 0, GFE_ERR_NONFINITE) == 0) err->index = cell;
  }
  double* g = geo + i * (1 + dim * dim);
  g[0] = qw[q] * fabs(det);
  // J^-T: (J^-T)[d][e] = inv[e][d]; grad_x phi = J^-T grad_xi phi
  for (int d = 0; d < dim; ++d)
    for (int e = 0; e < dim; ++e) g[1 + d * dim + e] = inv[e][d];
}

// op_test(v) . op_trial(u) for one pair of basis functions at one point: (field is vector,
// component, value phi, physical gradient P) of each side; shapes were checked by the host.
__device__ __forceinline__ double contract(int dim, int top, bool tvec, int tc, double tphi,
                                           const double* tP, int uop, bool uvec, int uc,
                                           double uphi, const double* uP) {
  if (top == GFE_MOP_VALUE && uop == GFE_MOP_VALUE)
    return (tvec && tc != uc) ? 0.0 : tphi * uphi;
  if (top == GFE_MOP_GRAD && uop == GFE_MOP_GRAD) {
    if (tvec && tc != uc) return 0.0;
    double s = 0.0;
    for (int d = 0; d < dim; ++d) s += tP[d] * uP[d];
    return s;
  }
  if (top == GFE_MOP_DIV && uop == GFE_MOP_DIV) return tP[tc] * uP[uc];
  if (top == GFE_MOP_DIV && uop == GFE_MOP_VALUE) return tP[tc] * uphi;
  if (top == GFE_MOP_VALUE && uop == GFE_MOP_DIV) return tphi * uP[uc];
  if (top == GFE_MOP_VALUE && uop == GFE_MOP_GRAD) return tphi * uP[tc];  // v . grad p
  if (top == GFE_MOP_GRAD && uop == GFE_MOP_VALUE) return tP[uc] * uphi;  // grad q . u
  (void)uvec;
  return 0.0;
}

// op_test(v) . f for a linear term, f the term's data at the point (or 1).
__device__ __forceinline__ double test_dot_data(int dim, int top, bool tvec, int tc, double tphi,
                                                const double* tP, const double* f) {
  if (top == GFE_MOP_VALUE) return tphi * f[tvec ? tc : 0];
  if (top == GFE_MOP_DIV) return tP[tc] * f[0];
  double s = 0.0;  // GRAD
  const double* g = tvec ? f + tc * dim : f;
  for (int d = 0; d < dim; ++d) s += tP[d] * g[d];
  return s;
}

// The cell's point geometry and the physical gradients of the fields in use, in shared memory.
__device__ void mf_load_cell(const MfArgs& a, const double* __restrict__ geo, int64_t cell,
                             double* sm) {
  const int D = a.dim, G = 1 + D * D;
  for (int i = threadIdx.x; i < a.nq * G; i += blockDim.x) sm[i] = geo[cell * a.nq * G + i];
  __syncthreads();
  for (int f = 0; f < a.nfields; ++f) {
    if (a.pg_off[f] < 0) continue;
    const MfField& F = a.f[f];
    double* P = sm + a.pg_off[f];
    for (int i = threadIdx.x; i < a.nq * F.nnodes; i += blockDim.x) {
      const int q = i / F.nnodes;
      const double* jt = sm + q * G + 1;
      const double* gr = F.grads + (int64_t)i * D;
      for (int d = 0; d < D; ++d) {
        double s = 0.0;
        for (int e = 0; e < D; ++e) s += jt[d * D + e] * gr[e];
        P[i * D + d] = s;
      }
    }
  }
  __syncthreads();
}

// Cell matrices of the block, column-major ndr x ndc per cell; one block of threads per cell.
__global__ void __launch_bounds__(kMfBlock)
    k_mf_cellmats(const __grid_constant__ MfArgs a, const double* __restrict__ geo,
                  double* __restrict__ mats) {
  extern __shared__ double sm[];
  const int D = a.dim, G = 1 + D * D;
  const int n = a.ndr * a.ndc;
  for (int64_t cell = blockIdx.x; cell < a.ncells; cell += gridDim.x) {
    __syncthreads();
    mf_load_cell(a, geo, cell, sm);
    double* out = mats + cell * (int64_t)n;
    for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
      const int li = idx % a.ndr, lj = idx / a.ndr;
      int tf, tc, tn, uf, uc, un;
      local_dof(a, a.rf, a.nrf, li, &tf, &tc, &tn);
      local_dof(a, a.cf, a.ncf, lj, &uf, &uc, &un);
      unsigned terms = 0u;
      for (int k = 0; k < a.nterms; ++k)
        if (a.t[k].test_field == tf && a.t[k].trial_field == uf) terms |= 1u << k;
      double acc = 0.0;
      const MfField& TF = a.f[tf];
      const MfField& UF = a.f[uf];
      const bool tvec = TF.ncomp > 1, uvec = UF.ncomp > 1;
      // value.value and grad:grad of two vector fields couple equal components only: an
      // entry whose terms are all of that kind with tc != uc is an exact zero, skip its loop
      if (tvec && uvec && tc != uc) {
        unsigned live = 0u;
        for (unsigned m = terms; m; m &= m - 1) {
          const MfTerm& T = a.t[__ffs(m) - 1];
          const bool per_comp = T.test_op == T.trial_op &&
                                (T.test_op == GFE_MOP_VALUE || T.test_op == GFE_MOP_GRAD);
          if (!per_comp) live |= m & (~m + 1u);
        }
        terms = live;
      }
      if (terms) {
        for (int q = 0; q < a.nq; ++q) {
          const double tphi = TF.shapes[q * TF.nnodes + tn];
          const double uphi = UF.shapes[q * UF.nnodes + un];
          const double* tP = sm + a.pg_off[tf] + (q * TF.nnodes + tn) * D;
          const double* uP = sm + a.pg_off[uf] + (q * UF.nnodes + un) * D;
          double s = 0.0;
          for (unsigned m = terms; m; m &= m - 1) {
            const MfTerm& T = a.t[__ffs(m) - 1];
            const double c = T.cell_coef ? T.coef * T.cell_coef[cell] : T.coef;
            s += c * contract(D, T.test_op, tvec, tc, tphi, tP, T.trial_op, uvec, uc, uphi, uP);
          }
          acc += sm[q * G] * s;
        }
      }
      out[idx] = acc;
    }
  }
}

// Cell vectors of the block's rows: the linear terms, then minus K_cell u_D over the cell's
// Dirichlet columns (ids -k read uD[k-1]).
__global__ void __launch_bounds__(kMfBlock)
    k_mf_cellvecs(const __grid_constant__ MfArgs a, const double* __restrict__ geo,
                  const double* __restrict__ mats, const int32_t* __restrict__ col_ids,
                  const double* __restrict__ uD, int64_t ndiri, double* __restrict__ vecs,
                  DevError* err) {
  extern __shared__ double sm[];
  const int D = a.dim, G = 1 + D * D;
  const double one[9] = {1, 1, 1, 1, 1, 1, 1, 1, 1};
  for (int64_t cell = blockIdx.x; cell < a.ncells; cell += gridDim.x) {
    __syncthreads();
    mf_load_cell(a, geo, cell, sm);
    for (int li = threadIdx.x; li < a.ndr; li += blockDim.x) {
      int tf, tc, tn;
      local_dof(a, a.rf, a.nrf, li, &tf, &tc, &tn);
      const MfField& TF = a.f[tf];
      const bool tvec = TF.ncomp > 1;
      double v = 0.0;
      unsigned terms = 0u;
      for (int k = 0; k < a.nterms; ++k)
        if (a.t[k].trial_field < 0 && a.t[k].test_field == tf) terms |= 1u << k;
      if (terms) {
        for (int q = 0; q < a.nq; ++q) {
          const double tphi = TF.shapes[q * TF.nnodes + tn];
          const double* tP = sm + a.pg_off[tf] + (q * TF.nnodes + tn) * D;
          double s = 0.0;
          for (unsigned m = terms; m; m &= m - 1) {
            const MfTerm& T = a.t[__ffs(m) - 1];
            const double c = T.cell_coef ? T.coef * T.cell_coef[cell] : T.coef;
            const double* f =
                T.qdata ? T.qdata + ((cell * a.nq) + q) * (int64_t)T.qdata_ncomp : one;
            s += c * test_dot_data(D, T.test_op, tvec, tc, tphi, tP, f);
          }
          v += sm[q * G] * s;
        }
      }
      if (mats && uD) {
        const double* K = mats + cell * (int64_t)a.ndr * a.ndc;
        double w = 0.0;
        for (int lj = 0; lj < a.ndc; ++lj) {
          const int32_t id = col_ids[cell * a.ndc + lj];
          if (id >= 0) continue;
          const int64_t k = -(int64_t)id - 1;
          if (k >= ndiri) {
            if (atomicCAS(&err->code, 0, GFE_ERR_INVALID_ARGUMENT) == 0) err->index = cell;
            continue;
          }
          w += K[li + (int64_t)lj * a.ndr] * uD[k];
        }
        v -= w;
      }
      vecs[cell * a.ndr + li] = v;
    }
  }
}

// Host-side shape check of one bilinear or linear term.
bool term_ok(int dim, const gfe_mf_field* F, const gfe_mf_term& t, int nfields) {
  auto shape = [&](int f, int op) -> int {  // 0 scalar, 1 vector, 2 tensor, -1 invalid
    const bool vec = F[f].ncomp > 1;
    if (op == GFE_MOP_VALUE) return vec ? 1 : 0;
    if (op == GFE_MOP_GRAD) return vec ? 2 : 1;
    if (op == GFE_MOP_DIV) return vec ? 0 : -1;
    return -1;
  };
  if (t.test_field < 0 || t.test_field >= nfields) return false;
  const int ts = shape(t.test_field, t.test_op);
  if (ts < 0) return false;
  if (t.trial_field < 0) {
    if (!t.qdata) return ts == 0;
    const int need = ts == 0 ? 1 : (ts == 1 ? dim : dim * dim);
    return t.qdata_ncomp == need;
  }
  if (t.trial_field >= nfields) return false;
  return shape(t.trial_field, t.trial_op) == ts;
}

}  // namespace
}  // namespace gfe

using namespace gfe;

extern "C" int gfe_multifield_assemble(gfe_ctx* ctx, const gfe_mf_problem* p,
                                       int32_t nrow_fields, const int32_t* row_fields,
                                       int32_t ncol_fields, const int32_t* col_fields,
                                       const int32_t* row_ids, const int32_t* col_ids,
                                       const double* dirichlet_values, int64_t ndirichlet,
                                       gfe_matrix* A, int64_t nrows, double* b) {
  gfe::NvtxRange nvtx_range("gfe_multifield_assemble");
  clear_error();
  const char* who = "gfe_multifield_assemble";
  if (!ctx || !p || (p->dim != 2 && p->dim != 3) || p->ncells < 0 || p->nq < 1 ||
      p->nfields < 1 || p->nfields > kMaxFields || p->nterms < 0 || p->nterms > kMaxTerms ||
      !p->fields || (p->nterms > 0 && !p->terms) || nrow_fields < 1 ||
      nrow_fields > kMaxFields || !row_fields || (A && (ncol_fields < 1 || !col_fields)) ||
      ncol_fields > kMaxFields || (!A && !b) || (A && A->ctx != ctx) || nrows < 0)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: bad arguments", who);
  if (p->ncells > 0 && (!p->node_coords || !p->cell_node_ids || !p->qweights || !p->geo_grads ||
                        !row_ids || (ncol_fields > 0 && !col_ids)))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: missing arrays", who);
  const int D = p->dim;
  MfArgs a{};
  a.dim = D;
  a.nq = p->nq;
  a.ncells = p->ncells;
  a.nfields = p->nfields;
  a.nterms = p->nterms;
  for (int f = 0; f < p->nfields; ++f) {
    const gfe_mf_field& F = p->fields[f];
    if (F.nnodes < 1 || (F.ncomp != 1 && F.ncomp != D) || !F.shapes || !F.grads)
      return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: field %d malformed", who, f);
  }
  for (int k = 0; k < p->nterms; ++k)
    if (!term_ok(D, p->fields, p->terms[k], p->nfields))
      return set_error(GFE_ERR_UNSUPPORTED,
                       "%s: term %d pairs operands of different shapes (or a field index is "
                       "out of range)", who, k);
  a.nrf = nrow_fields;
  a.ncf = ncol_fields;
  a.ndr = 0;
  a.ndc = 0;
  for (int i = 0; i < kMaxFields; ++i) a.pg_off[i] = -1;
  for (int i = 0; i < nrow_fields; ++i) {
    if (row_fields[i] < 0 || row_fields[i] >= p->nfields)
      return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: row field out of range", who);
    a.rf[i] = row_fields[i];
    a.ndr += p->fields[row_fields[i]].ncomp * p->fields[row_fields[i]].nnodes;
  }
  for (int i = 0; i < ncol_fields; ++i) {
    if (col_fields[i] < 0 || col_fields[i] >= p->nfields)
      return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: column field out of range", who);
    a.cf[i] = col_fields[i];
    a.ndc += p->fields[col_fields[i]].ncomp * p->fields[col_fields[i]].nnodes;
  }
  if (A && (A->nd != a.ndr || A->cols_per_cell() != a.ndc || A->ncells != p->ncells))
    return set_error(GFE_ERR_INVALID_ARGUMENT,
                     "%s: the matrix pattern was built for other cell ids", who);
  if (A) nrows = A->nrows;
  DeviceGuard g(ctx->device);
  // device copies of the inputs (the tables are small; host arrays are staged)
  std::vector<DevBuf*> bufs;
  struct Owned {
    std::vector<DevBuf*>& v;
    ~Owned() {
      for (DevBuf* b : v) delete b;
    }
  } owned{bufs};
  auto dev = [&](const void* h, size_t n, const void** out) -> int {
    if (!h || n == 0 || is_device_ptr(h)) {
      *out = h;
      return GFE_OK;
    }
    DevBuf* d = new DevBuf(ctx);
    bufs.push_back(d);
    GFE_TRY(d->reserve(n));
    GFE_CUDA_TRY(cudaMemcpyAsync(d->ptr, h, n, cudaMemcpyHostToDevice, ctx->stream));
    *out = d->ptr;
    return GFE_OK;
  };
  const int nv = 1 << D;
  const int64_t nc = p->ncells;
  const void *coords, *cnodes, *qw, *gg, *rids = nullptr, *cids = nullptr, *uD = nullptr;
  GFE_TRY(dev(p->node_coords, sizeof(double) * (size_t)p->nnodes * D, &coords));
  GFE_TRY(dev(p->cell_node_ids, sizeof(int32_t) * (size_t)nc * nv, &cnodes));
  GFE_TRY(dev(p->qweights, sizeof(double) * p->nq, &qw));
  GFE_TRY(dev(p->geo_grads, sizeof(double) * (size_t)p->nq * nv * D, &gg));
  GFE_TRY(dev(row_ids, sizeof(int32_t) * (size_t)nc * a.ndr, &rids));
  if (a.ndc > 0) GFE_TRY(dev(col_ids, sizeof(int32_t) * (size_t)nc * a.ndc, &cids));
  if (dirichlet_values && ndirichlet > 0)
    GFE_TRY(dev(dirichlet_values, sizeof(double) * (size_t)ndirichlet, &uD));
  for (int f = 0; f < p->nfields; ++f) {
    const gfe_mf_field& F = p->fields[f];
    const void *sh, *gr;
    GFE_TRY(dev(F.shapes, sizeof(double) * (size_t)p->nq * F.nnodes, &sh));
    GFE_TRY(dev(F.grads, sizeof(double) * (size_t)p->nq * F.nnodes * D, &gr));
    a.f[f] = MfField{F.ncomp, F.nnodes, F.ncomp * F.nnodes, (const double*)sh,
                     (const double*)gr};
  }
  for (int k = 0; k < p->nterms; ++k) {
    const gfe_mf_term& T = p->terms[k];
    const void *cc = nullptr, *qd = nullptr;
    GFE_TRY(dev(T.cell_coef, sizeof(double) * (size_t)nc, &cc));
    if (T.trial_field < 0 && T.qdata)
      GFE_TRY(dev(T.qdata, sizeof(double) * (size_t)nc * p->nq * T.qdata_ncomp, &qd));
    a.t[k] = MfTerm{T.test_field, T.trial_field, T.test_op, T.trial_op, T.coef,
                    (const double*)cc, (const double*)qd, T.qdata_ncomp};
  }
  // shared layout: the point geometry, then the physical gradients of the block's fields
  int off = p->nq * (1 + D * D);
  auto use = [&](int f) {
    if (a.pg_off[f] >= 0) return;
    a.pg_off[f] = off;
    off += p->nq * p->fields[f].nnodes * D;
  };
  for (int i = 0; i < a.nrf; ++i) use(a.rf[i]);
  for (int i = 0; i < a.ncf; ++i) use(a.cf[i]);
  a.smem_doubles = off;
  const size_t smem = sizeof(double) * (size_t)off;
  if (smem > 200 * 1024)
    return set_error(GFE_ERR_UNSUPPORTED, "%s: %zu bytes of point data per cell", who, smem);
  if (smem > 48 * 1024) {
    GFE_CUDA_TRY(cudaFuncSetAttribute(k_mf_cellmats, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    GFE_CUDA_TRY(cudaFuncSetAttribute(k_mf_cellvecs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  }
  if (nc == 0) return GFE_OK;
  // 1. geometry
  DevBuf geo(ctx);
  GFE_TRY(geo.reserve(sizeof(double) * (size_t)nc * p->nq * (1 + D * D)));
  timer_begin(ctx, GFE_KT_ELEMENT);
  k_mf_geometry<<<grid_for(nc * p->nq, 128), 128, 0, ctx->stream>>>(
      D, nc, p->nq, p->nnodes, (const double*)coords, (const int32_t*)cnodes,
      (const double*)qw,
      (const double*)gg, geo.as<double>(), ctx->d_err);
  timer_end(ctx);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  GFE_TRY(check_device_error(ctx, who));
  const unsigned gcells = grid_for(nc, 1, (int64_t)ctx->num_sms * 16);
  // 2. cell matrices (also for the lift of the vector)
  DevBuf mats(ctx);
  const bool need_mats = A || (b && uD && a.ndc > 0);
  if (need_mats) {
    GFE_TRY(mats.reserve(sizeof(double) * (size_t)nc * a.ndr * a.ndc));
    timer_begin(ctx, GFE_KT_ELEMENT);
    k_mf_cellmats<<<gcells, kMfBlock, smem, ctx->stream>>>(a, geo.as<double>(),
                                                            mats.as<double>());
    timer_end(ctx);
    ctx->launches++;
    GFE_CUDA_TRY(cudaGetLastError());
  }
  if (A) {
    GFE_TRY(assemble_cellmats(ctx, A, mats.as<double>()));
    A->mf_state = 0;
    A->plan_valid = false;
    A->dia_checked = false;
  }
  // 3. cell vectors, lifted, and their row-gather assembly
  if (b) {
    DevBuf vecs(ctx);
    GFE_TRY(vecs.reserve(sizeof(double) * (size_t)nc * a.ndr));
    timer_begin(ctx, GFE_KT_ELEMENT);
    k_mf_cellvecs<<<gcells, kMfBlock, smem, ctx->stream>>>(
        a, geo.as<double>(), need_mats ? mats.as<double>() : nullptr, (const int32_t*)cids,
        (const double*)uD, ndirichlet, vecs.as<double>(), ctx->d_err);
    timer_end(ctx);
    ctx->launches++;
    GFE_CUDA_TRY(cudaGetLastError());
    GFE_TRY(check_device_error(ctx, who));
    const bool bdev = is_device_ptr(b);
    double* db = b;
    DevBuf hb(ctx);
    if (!bdev) {
      GFE_TRY(hb.reserve(sizeof(double) * (size_t)(nrows > 0 ? nrows : 1)));
      db = hb.as<double>();
      GFE_CUDA_TRY(cudaMemcpyAsync(db, b, sizeof(double) * nrows, cudaMemcpyHostToDevice,
                                   ctx->stream));
    }
    GFE_TRY(assemble_cellvecs(ctx, nc, a.ndr, (const int32_t*)rids, vecs.as<double>(), nrows,
                              db));
    if (!bdev) GFE_TRY(copy_out(ctx, b, db, sizeof(double) * nrows));
  }
  return check_device_error(ctx, who);
}
