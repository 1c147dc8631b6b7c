// gfe_nonlinear.cu -- residual and Jacobian of quasilinear diffusion at a state u, for the
// Newton loops of a nonlinear FEOperator (FESpaces/FEOperatorsFromWeakForm.jl:117-190 with
// Algebra/NLSolvers.jl:1-87): every Newton step re-assembles the Jacobian into the fixed
// pattern (fillstored + numeric loop) and the residual into b.
//
//   r_i(u)    = sum_q dV_q [ k alpha_q grad u_q . g_i - f_q phi_i ]
//   J_ij(u)   = sum_q dV_q k [ alpha_q g_j . g_i + beta_q phi_j (grad u_q . g_i)
//                                + gamma_q (grad u_q . g_j)(grad u_q . g_i) ]
// with g_i the physical gradient of shape function i, alpha the law, beta = d alpha / d u,
// gamma = 2 d alpha / d |grad u|^2 (so that d(alpha grad u)/d(grad u) = alpha I +
// gamma grad u grad u^T), k the per-cell or constant coefficient.
//   poly law  alpha = c0 + c1 u + c2 u^2: beta = c1 + 2 c2 u, gamma = 0;
//   power law alpha = (e + |grad u|^2)^((p-2)/2): beta = 0,
//             gamma = (p-2) (e + |grad u|^2)^((p-4)/2)  (Gridap's p-Laplacian dflux).
//
// One block per cell (grid-stride): the cell's geometry, state values, per-point physical
// gradients and law values are staged in shared memory, then the threads take the NN^2
// Jacobian entries and the NN residual entries. Cell arrays are stored entry-major
// (entry * ncells + cell) and the row gather adds them in cell order.
#include <cmath>
#include <vector>

#include "gfe_internal.h"
#include "gfe_rows.cuh"

namespace gfe {
namespace {

template <int D, int NN>
__global__ void k_quasilinear_cells(int64_t ncells, const int32_t* __restrict__ cell_vertices,
                                    const double* __restrict__ coords,
                                    const int32_t* __restrict__ cell_ids,
                                    const double* __restrict__ state, int64_t nfree,
                                    const double* __restrict__ uD, int64_t ndiri,
                                    const double* __restrict__ tabs, int nq, int coef_kind,
                                    const double* __restrict__ coef, int src_kind,
                                    const double* __restrict__ src, int law, double c0,
                                    double c1, double c2, double* __restrict__ K,
                                    double* __restrict__ bvec, DevError* err) {
  constexpr int NV = 1 << D;
  extern __shared__ double sm[];
  // tables: w[nq] | phi[nq*NN] | dref[nq*NN*D] | dphi1[nq*NV*D]
  const int ntab = nq + nq * NN + nq * NN * D + nq * NV * D;
  const double* w = sm;
  const double* phi = w + nq;
  const double* dref = phi + nq * NN;
  const double* dphi1 = dref + nq * NN * D;
  double* xv = sm + ntab;           // NV*D
  double* uc = xv + NV * D;         // NN
  double* iJ = uc + NN;             // nq*D*D
  double* dv = iJ + nq * D * D;     // nq
  double* g = dv + nq;              // nq*NN*D physical gradients
  double* a = g + nq * NN * D;      // nq*NN: grad u . g_i
  double* cq = a + nq * NN;         // nq*3: k alpha dV, k beta dV, k gamma dV
  double* gu = cq + nq * 3;         // nq*D: grad u at q
  double* fq = gu + nq * D;         // nq: f dV
  for (int i = threadIdx.x; i < ntab; i += blockDim.x) sm[i] = tabs[i];
  __syncthreads();
  for (int64_t cell = blockIdx.x; cell < ncells; cell += gridDim.x) {
    if (threadIdx.x < NV * D) {
      const int v = threadIdx.x / D, d = threadIdx.x % D;
      xv[threadIdx.x] = coords[((int64_t)cell_vertices[cell * NV + v] - 1) * D + d];
    }
    if (threadIdx.x < NN) {
      const int32_t id = cell_ids[cell * NN + threadIdx.x];
      double u = 0.0;
      if (id > 0 && id <= nfree) {
        u = state[id - 1];
      } else if (id < 0 && -(int64_t)id <= ndiri) {
        u = uD[-(int64_t)id - 1];
      } else if (id != 0 && !(id < 0 && ndiri == 0)) {
        raise_err(err, GFE_ERR_INVALID_ARGUMENT, cell);
      }
      uc[threadIdx.x] = u;
    }
    const double kap = coef_kind == GFE_COEF_CELL ? coef[cell]
                       : coef_kind == GFE_COEF_CONST ? coef[0] : 1.0;
    __syncthreads();
    // geometry per point: Jt[k][l] = d x_l / d xi_k, its inverse and |det| w
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
      double Jt[9] = {0};
      for (int v = 0; v < NV; ++v)
        for (int k = 0; k < D; ++k)
          for (int l = 0; l < D; ++l)
            Jt[k * D + l] += dphi1[(q * NV + v) * D + k] * xv[v * D + l];
      double det, inv[9];
      if (D == 2) {
        det = Jt[0] * Jt[3] - Jt[1] * Jt[2];
        inv[0] = Jt[3] / det;
        inv[1] = -Jt[1] / det;
        inv[2] = -Jt[2] / det;
        inv[3] = Jt[0] / det;
      } else {
        const double c00 = Jt[4] * Jt[8] - Jt[5] * Jt[7];
        const double c01 = Jt[5] * Jt[6] - Jt[3] * Jt[8];
        const double c02 = Jt[3] * Jt[7] - Jt[4] * Jt[6];
        det = Jt[0] * c00 + Jt[1] * c01 + Jt[2] * c02;
        inv[0] = c00 / det;
        inv[1] = (Jt[2] * Jt[7] - Jt[1] * Jt[8]) / det;
        inv[2] = (Jt[1] * Jt[5] - Jt[2] * Jt[4]) / det;
        inv[3] = c01 / det;
        inv[4] = (Jt[0] * Jt[8] - Jt[2] * Jt[6]) / det;
        inv[5] = (Jt[2] * Jt[3] - Jt[0] * Jt[5]) / det;
        inv[6] = c02 / det;
        inv[7] = (Jt[1] * Jt[6] - Jt[0] * Jt[7]) / det;
        inv[8] = (Jt[0] * Jt[4] - Jt[1] * Jt[3]) / det;
      }
      if (!(det != 0.0) || !isfinite(det)) raise_err(err, GFE_ERR_DEGENERATE_CELL, cell);
      for (int k = 0; k < D * D; ++k) iJ[q * D * D + k] = inv[k];
      dv[q] = w[q] * fabs(det);
    }
    __syncthreads();
    // physical gradients g[q][i] = inv(Jt) dref[q][i]
    for (int t = threadIdx.x; t < nq * NN; t += blockDim.x) {
      const int q = t / NN;
      for (int k = 0; k < D; ++k) {
        double s = 0.0;
        for (int l = 0; l < D; ++l) s += iJ[q * D * D + k * D + l] * dref[t * D + l];
        g[t * D + k] = s;
      }
    }
    __syncthreads();
    // state and law per point
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
      double u = 0.0, gq[3] = {0.0, 0.0, 0.0};
      for (int i = 0; i < NN; ++i) {
        u += phi[q * NN + i] * uc[i];
        for (int k = 0; k < D; ++k) gq[k] += g[(q * NN + i) * D + k] * uc[i];
      }
      double n2 = 0.0;
      for (int k = 0; k < D; ++k) {
        gu[q * D + k] = gq[k];
        n2 += gq[k] * gq[k];
      }
      double al, be, ga;
      if (law == GFE_LAW_POLY) {
        al = c0 + c1 * u + c2 * u * u;
        be = c1 + 2.0 * c2 * u;
        ga = 0.0;
      } else {
        const double s = c1 + n2;  // eps2 + |grad u|^2
        al = pow(s, 0.5 * (c0 - 2.0));
        be = 0.0;
        ga = (c0 - 2.0) * pow(s, 0.5 * (c0 - 4.0));
      }
      const double kd = kap * dv[q];
      cq[q * 3 + 0] = kd * al;
      cq[q * 3 + 1] = kd * be;
      cq[q * 3 + 2] = kd * ga;
      double f = 0.0;
      if (src_kind == GFE_SRC_CONST) f = src[0];
      else if (src_kind == GFE_SRC_QPOINT) f = src[cell * nq + q];
      fq[q] = f * dv[q];
      if (!isfinite(cq[q * 3]) || !isfinite(cq[q * 3 + 1]) || !isfinite(cq[q * 3 + 2]))
        raise_err(err, GFE_ERR_NONFINITE, cell);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nq * NN; t += blockDim.x) {
      const int q = t / NN;
      double s = 0.0;
      for (int k = 0; k < D; ++k) s += gu[q * D + k] * g[t * D + k];
      a[t] = s;
    }
    __syncthreads();
    if (K)
      for (int e = threadIdx.x; e < NN * NN; e += blockDim.x) {
        const int i = e % NN, j = e / NN;  // i test row, j trial column
        double s = 0.0;
        for (int q = 0; q < nq; ++q) {
          double gg = 0.0;
          for (int k = 0; k < D; ++k) gg += g[(q * NN + i) * D + k] * g[(q * NN + j) * D + k];
          s += cq[q * 3] * gg + cq[q * 3 + 1] * a[q * NN + i] * phi[q * NN + j] +
               cq[q * 3 + 2] * a[q * NN + i] * a[q * NN + j];
        }
        K[(int64_t)e * ncells + cell] = s;
      }
    if (bvec)
      for (int i = threadIdx.x; i < NN; i += blockDim.x) {
        double s = 0.0;
        for (int q = 0; q < nq; ++q) s += cq[q * 3] * a[q * NN + i] - fq[q] * phi[q * NN + i];
        bvec[(int64_t)i * ncells + cell] = s;
      }
    __syncthreads();
  }
}

template <int D, int NN>
int launch_quasilinear(gfe_ctx* ctx, int64_t ncells, const int32_t* vn, const double* vc,
                       const int32_t* ids, const double* st, int64_t nfree, const double* uD,
                       int64_t ndiri, const double* tabs, int ntab, int nq, int coef_kind,
                       const double* coef, int src_kind, const double* src,
                       const gfe_problem* p, double* K, double* bv) {
  constexpr int NV = 1 << D;
  const size_t sm = sizeof(double) * ((size_t)ntab + NV * D + NN + (size_t)nq * D * D + nq +
                                      (size_t)nq * NN * D + (size_t)nq * NN + nq * 3 +
                                      (size_t)nq * D + nq);
  if (sm > 227 * 1024)
    return set_error(GFE_ERR_UNSUPPORTED, "quasilinear: quadrature too large (%d points)", nq);
  auto kern = k_quasilinear_cells<D, NN>;
  GFE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  const unsigned grid = (unsigned)std::min<int64_t>(ncells, (int64_t)ctx->num_sms * 8);
  timer_begin(ctx, GFE_KT_ELEMENT);
  kern<<<grid, 128, sm, ctx->stream>>>(ncells, vn, vc, ids, st, nfree, uD, ndiri, tabs, nq,
                                       coef_kind, coef, src_kind, src, p->law,
                                       p->law_params[0], p->law_params[1], p->law_params[2], K,
                                       bv, ctx->d_err);
  timer_end(ctx);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

}  // namespace

int assemble_quasilinear(gfe_ctx* ctx, const gfe_problem* p, gfe_matrix* A, double* d_b) {
  const int D = p->dim;
  if ((D != 2 && D != 3) || p->ncomp != 1 ||
      (p->reffe != GFE_REFFE_Q1 && p->reffe != GFE_REFFE_Q2))
    return set_error(GFE_ERR_UNSUPPORTED, "quasilinear: scalar Q1/Q2 in 2-D or 3-D");
  if (p->law != GFE_LAW_POLY && p->law != GFE_LAW_POWER)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "quasilinear: unknown law %d", p->law);
  for (int k = 0; k < 4; ++k)
    if (!std::isfinite(p->law_params[k]))
      return set_error(GFE_ERR_NONFINITE, "quasilinear: law parameter %d is not finite", k);
  if (!p->node_coords || !p->cell_node_ids || (p->nfree > 0 && !p->state))
    return set_error(GFE_ERR_INVALID_ARGUMENT,
                     "quasilinear: node coordinates, cell vertices and the state are needed");
  if (p->source_kind != GFE_SRC_NONE && p->source_kind != GFE_SRC_CONST &&
      p->source_kind != GFE_SRC_QPOINT)
    return set_error(GFE_ERR_UNSUPPORTED, "quasilinear: constant or quadrature-point f");
  const int nv = 1 << D;
  const bool q2 = p->reffe == GFE_REFFE_Q2;
  const int nn = q2 ? (D == 2 ? 9 : 27) : nv;
  if (p->nd != nn) return set_error(GFE_ERR_INVALID_ARGUMENT, "quasilinear: nd mismatch");
  if (A && (A->ncells != p->ncells || A->nd != p->nd))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "quasilinear: matrix built for other cells");
  std::vector<double> qx, qw;
  GFE_TRY(tensor_quadrature(D, p->degree, qx, qw));
  const int nq = (int)qw.size();
  const int64_t ncells = p->ncells;
  if (p->source_kind == GFE_SRC_QPOINT ? p->source_len != ncells * nq
                                      : (p->source_kind == GFE_SRC_CONST && p->source_len < 1))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "quasilinear: source needs 1 or ncells*%d values",
                     nq);

  // device views: geometry, ids, state, Dirichlet values, coefficient, source
  const void *vc, *vn, *vi, *vs = nullptr, *vd = nullptr, *vk = nullptr, *vf = nullptr;
  GFE_TRY(device_view(ctx, p->node_coords, sizeof(double) * (size_t)p->nnodes * D, SCR_COORDS,
                      &vc));
  GFE_TRY(device_view(ctx, p->cell_node_ids, sizeof(int32_t) * (size_t)ncells * nv,
                      SCR_CELLNODES, &vn));
  GFE_TRY(device_view(ctx, p->cell_dof_ids, sizeof(int32_t) * (size_t)ncells * nn, SCR_CELLIDS,
                      &vi));
  if (p->nfree > 0)
    GFE_TRY(device_view(ctx, p->state, sizeof(double) * (size_t)p->nfree, SCR_VEC_X, &vs));
  const int64_t ndiri = p->dirichlet_values ? p->ndirichlet : 0;
  if (ndiri > 0)
    GFE_TRY(device_view(ctx, p->dirichlet_values, sizeof(double) * (size_t)ndiri, SCR_DIRI,
                        &vd));
  if (p->coef_kind == GFE_COEF_CONST || p->coef_kind == GFE_COEF_CELL) {
    const size_t n = p->coef_kind == GFE_COEF_CELL ? (size_t)ncells : 1;
    GFE_TRY(device_view(ctx, p->coef, sizeof(double) * n, SCR_COEF, &vk));
  }
  if (p->source_kind != GFE_SRC_NONE)
    GFE_TRY(device_view(ctx, p->source, sizeof(double) * (size_t)p->source_len, SCR_SRC, &vf));

  // tables: w | phi | dref | dphi1
  std::vector<double> phi1, dphi1, phi, dref;
  q1_shapes(D, nq, qx.data(), phi1, dphi1);
  if (q2) {
    q2_shapes(D, nq, qx.data(), phi, dref);
  } else {
    phi = phi1;
    dref = dphi1;
  }
  std::vector<double> tabs(qw);
  tabs.insert(tabs.end(), phi.begin(), phi.end());
  tabs.insert(tabs.end(), dref.begin(), dref.end());
  tabs.insert(tabs.end(), dphi1.begin(), dphi1.end());
  GFE_TRY(ctx->scratch[SCR_TMP1].reserve(sizeof(double) * tabs.size()));
  GFE_CUDA_TRY(cudaMemcpyAsync(ctx->scratch[SCR_TMP1].ptr, tabs.data(),
                               sizeof(double) * tabs.size(), cudaMemcpyHostToDevice,
                               ctx->stream));
  double* K = nullptr;
  double* bv = nullptr;
  if (A) {
    GFE_TRY(ctx->scratch[SCR_CELLMAT].reserve(sizeof(double) * (size_t)ncells * nn * nn));
    K = ctx->scratch[SCR_CELLMAT].as<double>();
  }
  if (d_b) {
    GFE_TRY(ctx->scratch[SCR_CELLVEC].reserve(sizeof(double) * (size_t)ncells * nn));
    bv = ctx->scratch[SCR_CELLVEC].as<double>();
  }
  const double* dt = ctx->scratch[SCR_TMP1].as<double>();
  const int ntab = (int)tabs.size();
  const int32_t* cv = (const int32_t*)vn;
  const double* xc = (const double*)vc;
  const int32_t* ids = (const int32_t*)vi;
  const double* st = (const double*)vs;
  const double* ud = (const double*)vd;
  const double* kc = (const double*)vk;
  const double* fs = (const double*)vf;
  if (D == 2 && !q2)
    GFE_TRY((launch_quasilinear<2, 4>(ctx, ncells, cv, xc, ids, st, p->nfree, ud, ndiri, dt, ntab,
                                      nq, p->coef_kind, kc, p->source_kind, fs, p, K, bv)));
  else if (D == 2)
    GFE_TRY((launch_quasilinear<2, 9>(ctx, ncells, cv, xc, ids, st, p->nfree, ud, ndiri, dt, ntab,
                                      nq, p->coef_kind, kc, p->source_kind, fs, p, K, bv)));
  else if (!q2)
    GFE_TRY((launch_quasilinear<3, 8>(ctx, ncells, cv, xc, ids, st, p->nfree, ud, ndiri, dt, ntab,
                                      nq, p->coef_kind, kc, p->source_kind, fs, p, K, bv)));
  else
    GFE_TRY((launch_quasilinear<3, 27>(ctx, ncells, cv, xc, ids, st, p->nfree, ud, ndiri, dt,
                                       ntab, nq, p->coef_kind, kc, p->source_kind, fs, p, K,
                                       bv)));
  GFE_TRY(check_device_error(ctx, "assemble (quasilinear cell arrays)"));
  // the host tables must outlive their copy
  GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));

  // row gathers in cell order (no Dirichlet lift: the residual already uses u's values)
  gfe_matrix tmp;
  gfe_matrix* R = A;
  tmp.cell_rows.owner = tmp.ref_ptr.owner = tmp.refs.owner = ctx;
  if (!R) {
    tmp.ctx = ctx;
    tmp.nrows = p->nfree;
    tmp.ncols = p->nfree;
    tmp.nd = nn;
    tmp.ncells = ncells;
    const size_t idsz = sizeof(int32_t) * (size_t)ncells * nn;
    GFE_TRY(tmp.cell_rows.reserve(idsz));
    GFE_CUDA_TRY(cudaMemcpyAsync(tmp.cell_rows.ptr, vi, idsz, cudaMemcpyDeviceToDevice,
                                 ctx->stream));
    GFE_TRY(build_refs(ctx, &tmp));
    R = &tmp;
  }
  StoredCells s{};
  s.mat = K;
  s.vec = bv;
  s.cs = 1;
  s.es = ncells;
  s.vcs = 1;
  s.ves = ncells;
  s.ntab = 0;
  RowArgs a = row_args(ctx, R, d_b, A != nullptr);
  a.uD = nullptr;
  a.ndiri = 0;
  if (A) {
    GFE_TRY(run_rows(ctx, a, s, A->max_width, A->pos_bytes));
  } else {
    a.rowptr = nullptr;
    a.colval = nullptr;
    a.cell_cols = nullptr;
    GFE_TRY(vector_only_rows(ctx, a, s));
  }
  return check_device_error(ctx, "assemble (quasilinear)");
}

}  // namespace gfe
