// gfe_elasticity.cu -- isotropic linear elasticity on vector P2 tetrahedra.
//
//   a(u, v) = int eps(v) : (lambda tr(eps(u)) I + 2 mu eps(u)),   l(v) = int f . v
//
// Local dofs are component-major (dof k*10 + n: node n, component k), the layout of
// Gridap's vector-valued Lagrangian reference FE. For v = phi_i e_k and u = phi_j e_l,
//   eps(v) : sigma(u) = lambda d_k phi_i d_l phi_j
//                       + mu (delta_kl grad phi_i . grad phi_j + d_l phi_i d_k phi_j).
// Cells are affine (P1 geometry), so grad phi = C grad_hat phi with C = inv(Jt) constant per
// cell and every entry is a combination of the reference integrals
//   G^{ab}_{ij} = sum_q w_q d_a phi_i(xi_q) d_b phi_j(xi_q):
// with T = C G_ij C^T,  K[(k,i),(l,j)] = |det Jt| (lambda T_kl + mu T_lk + mu delta_kl tr T).
//
// Two sources feed the row-gather assembly (gfe_rows.cuh):
//   - simplexified uniform Cartesian boxes: the 6 local tets of a cell have 6 fixed shapes,
//     so the cell matrix is lambda_c Kl[t] + mu_c Km[t] from 2 x 6 tables (built on the host
//     from Gridap's per-quadrature-point steps in extended precision);
//   - general affine tets (node coordinates + tet vertex ids): an element kernel evaluates the
//     formula above per cell, with the Jacobian, its inverse and determinant in FP64 (FP32
//     cell matrices: the tensor-core kernels of gfe_p2_tc.cu).
#include <cmath>
#include <vector>

#include "gfe_internal.h"
#include "gfe_rows.cuh"

namespace gfe {
namespace {

__global__ void k_check_finite_e(const double* __restrict__ v, int64_t n, DevError* err) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (!isfinite(v[i])) raise_err(err, GFE_ERR_NONFINITE, i);
}

__device__ __forceinline__ void lame_of(int coef_kind, const double* coef, int64_t cell,
                                        double& lam, double& mu) {
  if (coef_kind == GFE_COEF_CELL) {
    lam = __ldg(coef + 2 * cell);
    mu = __ldg(coef + 2 * cell + 1);
  } else if (coef_kind == GFE_COEF_CONST) {
    lam = __ldg(coef);
    mu = __ldg(coef + 1);
  } else {
    lam = 1.0;
    mu = 1.0;
  }
}

// Tables: Kl[6*900] | Km[6*900] | mv[6*10] (column-major 30x30 per local tet), read through
// the L1 cache rather than staged in shared memory (86 KB would cap the row kernel at one
// block per SM).
template <bool FP32>
struct CartesianElasticityP2 {
  const double* tables;
  int coef_kind;
  const double* coef;
  const double* f;  // body force (3 values) or null
  int ntab;
  struct Cell {
    int t;  // local tet 0..5 of its hexahedron
    double lam, mu;
  };
  __device__ void load_tables(double*) const {}
  __device__ __forceinline__ Cell cell(int64_t c) const {
    Cell k;
    k.t = (int)(c % 6);
    lame_of(coef_kind, coef, c, k.lam, k.mu);
    return k;
  }
  __device__ __forceinline__ double m(const double*, const Cell& k, int li, int lj, int) const {
    const int e = k.t * 900 + li + lj * 30;
    if (FP32)
      return (double)fmaf((float)k.lam, (float)__ldg(tables + e),
                          (float)k.mu * (float)__ldg(tables + 5400 + e));
    return fma(k.lam, __ldg(tables + e), k.mu * __ldg(tables + 5400 + e));
  }
  __device__ __forceinline__ double v(const double*, int64_t cell, int li) const {
    if (!f) return 0.0;
    return __ldg(f + li / 10) * __ldg(tables + 10800 + (int)(cell % 6) * 10 + li % 10);
  }
};

// One thread per tet. K entry-major: K[(li + lj*30)*ncells + cell]; b[li*ncells + cell].
template <typename T>
__global__ void __launch_bounds__(128)
    k_p2_elasticity_cells(int64_t ncells, const double* __restrict__ coords,
                          const int32_t* __restrict__ tet_vertices, int coef_kind,
                          const double* __restrict__ coef, const double* __restrict__ f,
                          const double* __restrict__ Gref, const double* __restrict__ mref,
                          T* __restrict__ K, double* __restrict__ bvec, DevError* err) {
  __shared__ T sG[900];
  for (int i = threadIdx.x; i < 900; i += blockDim.x) sG[i] = (T)Gref[i];
  __syncthreads();
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncells) return;
  double X[4][3];
  for (int a = 0; a < 4; ++a) {
    const int32_t v = __ldg(tet_vertices + cell * 4 + a);
    if (v < 1) {
      raise_err(err, GFE_ERR_INVALID_ARGUMENT, cell);
      return;
    }
    for (int d = 0; d < 3; ++d) X[a][d] = __ldg(coords + (int64_t)(v - 1) * 3 + d);
  }
  // Jt_{kl} = sum_a grad phi1_a[k] x_a[l] = x_{k+1}[l] - x_0[l] (FP64)
  double J[3][3];
  for (int k = 0; k < 3; ++k)
    for (int l = 0; l < 3; ++l) J[k][l] = X[k + 1][l] - X[0][l];
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[0][2] * J[2][1] - J[0][1] * J[2][2];
  const double c02 = J[0][1] * J[1][2] - J[0][2] * J[1][1];
  const double det = J[0][0] * c00 + J[1][0] * c01 + J[2][0] * c02;
  if (!(det != 0.0) || !isfinite(det)) {
    raise_err(err, GFE_ERR_INVALID_ARGUMENT, cell);
    return;
  }
  const double id = 1.0 / det;
  double Cd[3][3] = {
      {c00 * id, c01 * id, c02 * id},
      {(J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id, (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id,
       (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id},
      {(J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id, (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id,
       (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id}};
  T C[3][3];
  for (int k = 0; k < 3; ++k)
    for (int a = 0; a < 3; ++a) C[k][a] = (T)Cd[k][a];
  double lamd, mud;
  lame_of(coef_kind, coef, cell, lamd, mud);
  const T dJ = (T)fabs(det);
  const T lam = (T)lamd * dJ, mu = (T)mud * dJ;
  for (int i = 0; i < 10; ++i)
    for (int j = 0; j < 10; ++j) {
      // M = G_ij C^T, Tm = C M
      T M[3][3];
      for (int a = 0; a < 3; ++a)
        for (int l = 0; l < 3; ++l) {
          T s = 0;
          for (int b = 0; b < 3; ++b) s += sG[(a * 3 + b) * 100 + i * 10 + j] * C[l][b];
          M[a][l] = s;
        }
      T Tm[3][3];
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) {
          T s = 0;
          for (int a = 0; a < 3; ++a) s += C[k][a] * M[a][l];
          Tm[k][l] = s;
        }
      const T tr = Tm[0][0] + Tm[1][1] + Tm[2][2];
      for (int l = 0; l < 3; ++l)
        for (int k = 0; k < 3; ++k) {
          T e = lam * Tm[k][l] + mu * Tm[l][k];
          if (k == l) e += mu * tr;
          K[(int64_t)((k * 10 + i) + (l * 10 + j) * 30) * ncells + cell] = e;
        }
    }
  if (bvec)
    for (int k = 0; k < 3; ++k)
      for (int i = 0; i < 10; ++i)
        bvec[(int64_t)(k * 10 + i) * ncells + cell] =
            f ? __ldg(f + k) * (fabs(det) * __ldg(mref + i)) : 0.0;
}

}  // namespace

int assemble_p2_elasticity(gfe_ctx* ctx, const gfe_problem* p, gfe_matrix* A, double* d_b) {
  if (p->dim != 3 || p->ncomp != 3 || p->nd != 30 || p->form != GFE_FORM_ELASTICITY)
    return set_error(GFE_ERR_UNSUPPORTED,
                     "assemble: P2 tets are provided for 3-D vector elasticity (nd 30)");
  if (A && (A->ncells != p->ncells || A->nd != p->nd ||
            A->cols_per_cell() != p->nd))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "assemble: matrix pattern built for other cells");
  const int64_t ncells = p->ncells;
  const bool fp32 = p->precision == GFE_PREC_FP32;
  // Lame coefficients
  const double* d_coef = nullptr;
  if (p->coef_kind == GFE_COEF_CONST || p->coef_kind == GFE_COEF_CELL) {
    const size_t n = p->coef_kind == GFE_COEF_CELL ? 2 * (size_t)ncells : 2;
    const void* v;
    GFE_TRY(device_view(ctx, p->coef, sizeof(double) * n, SCR_COEF, &v));
    d_coef = (const double*)v;
    k_check_finite_e<<<grid_for((int64_t)n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
        d_coef, (int64_t)n, ctx->d_err);
    ctx->launches++;
  } else if (p->coef_kind != GFE_COEF_ONE) {
    return set_error(GFE_ERR_INVALID_ARGUMENT, "assemble: bad coefficient kind");
  }
  // body force
  const double* d_f = nullptr;
  if (p->source_kind == GFE_SRC_CONST) {
    if (p->source_len != 3)
      return set_error(GFE_ERR_INVALID_ARGUMENT, "assemble: body force needs 3 values");
    const void* v;
    GFE_TRY(device_view(ctx, p->source, sizeof(double) * 3, SCR_SRC, &v));
    d_f = (const double*)v;
    k_check_finite_e<<<1, 32, 0, ctx->stream>>>(d_f, 3, ctx->d_err);
    ctx->launches++;
  } else if (p->source_kind != GFE_SRC_NONE) {
    return set_error(GFE_ERR_UNSUPPORTED, "assemble: elasticity takes a constant body force");
  }
  GFE_CUDA_TRY(cudaGetLastError());

  // rows: the matrix's, or (vector only) references built from the cell ids
  gfe_matrix* R = A;
  gfe_matrix tmp;
  tmp.cell_rows.owner = tmp.ref_ptr.owner = tmp.refs.owner = ctx;
  if (!R) {
    tmp.ctx = ctx;
    tmp.nrows = p->nfree;
    tmp.ncols = p->nfree;
    tmp.nd = p->nd;
    tmp.ncells = ncells;
    const void* v;
    const size_t idsz = sizeof(int32_t) * (size_t)ncells * p->nd;
    GFE_TRY(device_view(ctx, p->cell_dof_ids, idsz, SCR_CELLIDS, &v));
    GFE_TRY(tmp.cell_rows.reserve(idsz));
    GFE_CUDA_TRY(cudaMemcpyAsync(tmp.cell_rows.ptr, v, idsz, cudaMemcpyDeviceToDevice,
                                 ctx->stream));
    GFE_TRY(build_refs(ctx, &tmp));
    R = &tmp;
  }
  GFE_TRY(ensure_row_refs(ctx, R));
  RowArgs a = row_args(ctx, R, d_b, A != nullptr);
  if (!A) {
    a.rowptr = nullptr;
    a.colval = nullptr;
    a.cell_cols = nullptr;
  }
  const int maxw = A ? A->max_width : 1;

  if (p->geometry == GFE_GEOM_CARTESIAN) {
    if (ncells != 6 * p->partition[0] * p->partition[1] * p->partition[2])
      return set_error(GFE_ERR_INVALID_ARGUMENT,
                       "assemble: simplexified box has 6 tets per hexahedron");
    double h[3];
    for (int d = 0; d < 3; ++d)
      h[d] = (p->domain[2 * d + 1] - p->domain[2 * d]) / (double)p->partition[d];
    std::vector<double> tab;
    GFE_TRY(elasticity_p2_tables(h, p->degree, tab));
    GFE_TRY(ctx->scratch[SCR_TMP1].reserve(sizeof(double) * tab.size()));
    GFE_CUDA_TRY(cudaMemcpyAsync(ctx->scratch[SCR_TMP1].ptr, tab.data(),
                                 sizeof(double) * tab.size(), cudaMemcpyHostToDevice,
                                 ctx->stream));
    // the host table must stay alive until the copy has run
    GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    auto go = [&](auto src) -> int {
      src.tables = ctx->scratch[SCR_TMP1].as<double>();
      src.coef_kind = p->coef_kind;
      src.coef = d_coef;
      src.f = d_f;
      src.ntab = 0;
      if (A) return run_rows(ctx, a, src, maxw, A->pos_bytes);
      return vector_only_rows(ctx, a, src);
    };
    if (fp32) GFE_TRY(go(CartesianElasticityP2<true>{}));
    else GFE_TRY(go(CartesianElasticityP2<false>{}));
    if (A) GFE_TRY(attach_p2_pmg(ctx, A, p, d_coef));
    return check_device_error(ctx, "assemble (P2 elasticity)");
  }

  if (p->geometry != GFE_GEOM_NODAL || !p->node_coords || !p->cell_node_ids || p->nnodes < 4)
    return set_error(GFE_ERR_INVALID_ARGUMENT,
                     "assemble: P2 tets need a Cartesian box or node coordinates + tet vertices");
  const void* vc;
  const void* vn;
  GFE_TRY(device_view(ctx, p->node_coords, sizeof(double) * (size_t)p->nnodes * 3, SCR_COORDS,
                      &vc));
  GFE_TRY(device_view(ctx, p->cell_node_ids, sizeof(int32_t) * (size_t)ncells * 4,
                      SCR_CELLNODES, &vn));
  std::vector<double> G, mr;
  GFE_TRY(p2tet_reference_integrals(p->degree, G, mr));
  G.insert(G.end(), mr.begin(), mr.end());
  GFE_TRY(ctx->scratch[SCR_TMP1].reserve(sizeof(double) * G.size()));
  GFE_CUDA_TRY(cudaMemcpyAsync(ctx->scratch[SCR_TMP1].ptr, G.data(), sizeof(double) * G.size(),
                               cudaMemcpyHostToDevice, ctx->stream));
  GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  const double* dG = ctx->scratch[SCR_TMP1].as<double>();
  const size_t esz = fp32 ? sizeof(float) : sizeof(double);
  const int64_t ncells16 = (ncells + 15) / 16 * 16;  // whole tiles of the tensor-core layout
  if (A) GFE_TRY(ctx->scratch[SCR_CELLMAT].reserve(esz * (size_t)ncells16 * 900));
  if (d_b) GFE_TRY(ctx->scratch[SCR_CELLVEC].reserve(sizeof(double) * (size_t)ncells * 30));
  double* bv = d_b ? ctx->scratch[SCR_CELLVEC].as<double>() : nullptr;
  const unsigned g = (unsigned)((ncells + 127) / 128);
  if (A) {
    timer_begin(ctx, GFE_KT_ELEMENT);
    if (fp32) {
      // the tensor-core cells (gfe_p2_tc.cu): split FP16 operands, FP32 accuracy
      GFE_TRY(launch_p2_cells_tc(ctx, ncells, (const double*)vc, (const int32_t*)vn,
                                 p->coef_kind, d_coef, d_f, dG + 900, G.data(),
                                 ctx->scratch[SCR_CELLMAT].as<float>(), bv));
    } else {
      k_p2_elasticity_cells<double><<<g, 128, 0, ctx->stream>>>(
          ncells, (const double*)vc, (const int32_t*)vn, p->coef_kind, d_coef, d_f, dG,
          dG + 900, ctx->scratch[SCR_CELLMAT].as<double>(), bv, ctx->d_err);
      ctx->launches++;
    }
    timer_end(ctx);
  } else if (bv) {
    // vector only: the element kernel without matrix output is not worth a separate path
    GFE_TRY(ctx->scratch[SCR_CELLMAT].reserve(sizeof(float) * (size_t)ncells * 900));
    k_p2_elasticity_cells<float><<<g, 128, 0, ctx->stream>>>(
        ncells, (const double*)vc, (const int32_t*)vn, p->coef_kind, d_coef, d_f, dG, dG + 900,
        ctx->scratch[SCR_CELLMAT].as<float>(), bv, ctx->d_err);
    ctx->launches++;
  }
  GFE_CUDA_TRY(cudaGetLastError());
  if (bv) {  // the vector through its own gather, before the matrix pass and its lift
    StoredCells vs{};
    vs.mat = nullptr;
    vs.vec = bv;
    vs.vcs = 1;
    vs.ves = ncells;
    vs.ntab = 0;
    RowArgs av = a;
    av.val = nullptr;
    GFE_TRY(vector_only_rows(ctx, av, vs));
  }
  RowArgs am = a;  // matrix pass
  am.b = nullptr;
  const bool lift = A && bv && a.uD;
  if (fp32) {
    TiledCellsF32 src{};
    src.mat = A ? ctx->scratch[SCR_CELLMAT].as<float>() : nullptr;
    src.ntab = 0;
    if (A) GFE_TRY(run_rows(ctx, am, src, maxw, A->pos_bytes));
    if (lift) GFE_TRY(dirichlet_lift(ctx, a, src));
  } else {
    StoredCells src{};
    src.mat = A ? ctx->scratch[SCR_CELLMAT].as<double>() : nullptr;
    src.cs = 1;
    src.es = ncells;
    src.vec = nullptr;
    src.ntab = 0;
    if (A) GFE_TRY(run_rows(ctx, am, src, maxw, A->pos_bytes));
    if (lift) GFE_TRY(dirichlet_lift(ctx, a, src));
  }
  return check_device_error(ctx, "assemble (P2 elasticity)");
}

}  // namespace gfe
