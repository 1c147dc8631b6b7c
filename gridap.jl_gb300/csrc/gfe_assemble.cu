// gfe_assemble.cu -- numeric assembly on the device.
//
// Gridap's numeric loop walks cells in order and adds every cell matrix entry into the
// sparse matrix (InserterCSC: binary search in the column, then `+=`), so each stored value
// is the sum of its cell contributions in ascending cell order
// (FESpaces/SparseMatrixAssemblers.jl:214-248, Algebra/SparseMatrixCSC.jl:124-150).
//
// Here every matrix row is owned by one thread. The thread walks the row's cell references
// (sorted by cell, built with the pattern), finds each contribution's column by binary search
// in the row's sorted column list and accumulates in shared memory. Each stored value thus
// receives exactly the additions Gridap makes, in the same order, with no atomics and no
// colouring: the result is deterministic and, for identical cell values, bit-identical to
// Gridap's. A block of R rows then writes its contiguous slice of the CSR values with
// coalesced stores.
//
// Cell values come from a source functor:
//   - StoredCells: cell matrices/vectors in memory (the caller's, or an element kernel's);
//   - CartesianDiffusionQ1: kappa_K * Kref on uniform Cartesian cells, where every cell has
//     Jt = diag(h) (Geometry/CartesianGrids.jl:247-276) and hence the same reference
//     stiffness; the source term from the cell's node values or quadrature-point values.
#include <cmath>

#include "gfe_internal.h"
#include "gfe_rows.cuh"


namespace gfe {

// Uniform Cartesian Q1 diffusion. Tables (built on the host, FP64):
//   Kref[nd*nd]  = sum_q (invJt grad phi_i).(invJt grad phi_j) |det Jt| w_q   (col-major)
//   Mref[nd*nd]  = sum_q phi_i phi_a |det Jt| w_q                             (col-major)
//   mref[nd]     = sum_q phi_i |det Jt| w_q
//   PW[nq*nd]    = phi_i(xi_q) |det Jt| w_q
template <int D, bool FP32>
struct CartesianDiffusionQ1 {
  static constexpr int NV = 1 << D;
  const double* tables;  // Kref | Mref | mref | PW
  int nq;
  int coef_kind;         // GFE_COEF_*
  const double* coef;
  int src_kind;          // GFE_SRC_* (SINSUM arrives here as QPOINT values)
  const double* src;
  int64_t n0, n1;        // cells per direction
  const int32_t* cell_nodes;  // optional explicit node ids
  int ntab;
  __device__ void load_tables(double* s) const {
    for (int i = threadIdx.x; i < ntab; i += blockDim.x) s[i] = tables[i];
  }
  __device__ __forceinline__ double kappa(int64_t cell) const {
    if (coef_kind == GFE_COEF_CELL) return __ldg(coef + cell);
    if (coef_kind == GFE_COEF_CONST) return __ldg(coef);
    return 1.0;
  }
  __device__ __forceinline__ double cell(int64_t c) const { return kappa(c); }
  __device__ __forceinline__ double m(const double* s, double kap, int li, int lj, int) const {
    const double k = s[li + lj * NV];
    if (coef_kind == GFE_COEF_ONE) return k;
    if (FP32) return (double)((float)kap * (float)k);
    return kap * k;
  }
  // acc + kappa Kref[li][lj] as one FP64 fused multiply-add
  __device__ __forceinline__ double madd(const double* s, double kap, int li, int lj, int,
                                         double acc) const {
    const double k = s[li + lj * NV];
    if (coef_kind == GFE_COEF_ONE) return acc + k;
    if (FP32) return acc + (double)((float)kap * (float)k);
    return fma(kap, k, acc);
  }
  // node of local vertex 0 of a Cartesian cell and the node strides of y and z: the cell id
  // is split once in 32-bit arithmetic (cell ids are below 2^31), the other vertices follow
  // by offsets (64-bit division per vertex dominated the row gather's instruction count)
  __device__ __forceinline__ int64_t node0(int64_t cell, int64_t& sy, int64_t& sz) const {
    const uint32_t c = (uint32_t)cell, u0 = (uint32_t)n0, u1 = (uint32_t)n1;
    const uint32_t r = c / u0, i = c - r * u0, k = r / u1, j = r - k * u1;
    sy = n0 + 1;
    sz = sy * (n1 + 1);
    return (int64_t)i + sy * j + sz * k;
  }
  __device__ __forceinline__ double v(const double* s, int64_t cell, int li) const {
    const double* Mref = s + NV * NV;
    const double* mref = Mref + NV * NV;
    const double* PW = mref + NV;
    if (src_kind == GFE_SRC_CONST) return __ldg(src) * mref[li];
    if (src_kind == GFE_SRC_NODAL) {
      double acc = 0.0;
#pragma unroll
      if (cell_nodes) {
#pragma unroll
        for (int a = 0; a < NV; ++a)
          acc = fma(Mref[li + a * NV], __ldg(src + (__ldg(cell_nodes + cell * NV + a) - 1)),
                    acc);
        return acc;
      }
      int64_t sy, sz;
      const int64_t b0 = node0(cell, sy, sz);
#pragma unroll
      for (int a = 0; a < NV; ++a) {
        const int64_t nd = b0 + (a & 1) + sy * ((a >> 1) & 1) + (D == 3 ? sz * (a >> 2) : 0);
        acc = fma(Mref[li + a * NV], __ldg(src + nd), acc);
      }
      return acc;
    }
    if (src_kind == GFE_SRC_QPOINT) {
      double acc = 0.0;
      for (int q = 0; q < nq; ++q) acc = fma(__ldg(src + cell * nq + q), PW[q * NV + li], acc);
      return acc;
    }
    return 0.0;
  }
};

// ---- caller-provided cell matrices (Gridap's numeric_loop_matrix!) -----------------------
int assemble_cellmats(gfe_ctx* ctx, gfe_matrix* A, const double* d_cellmats) {
  const int maxw = A->max_width;
  StoredCells src{};
  src.mat = d_cellmats;
  src.vec = nullptr;
  src.cs = (int64_t)A->nd * A->cols_per_cell();
  src.es = 1;
  src.ntab = 0;
  GFE_TRY(ensure_row_refs(ctx, A));
  RowArgs a = row_args(ctx, A, nullptr, true);
  GFE_TRY(run_rows(ctx, a, src, maxw, A->pos_bytes));
  return check_device_error(ctx, "numeric_loop_matrix");
}

// ---- caller-provided cell vectors (numeric_loop_vector!) ---------------------------------
// Builds the row references of the given cell ids in scratch, then gathers per row.
int assemble_cellvecs(gfe_ctx* ctx, int64_t ncells, int nd, const int32_t* d_rows,
                      const double* d_cellvecs, int64_t nrows, double* d_b) {
  // A temporary matrix object carries the references (no pattern needed).
  gfe_matrix T;
  T.ctx = ctx;
  T.cell_rows.owner = T.ref_ptr.owner = T.refs.owner = ctx;
  T.nrows = nrows;
  T.ncols = nrows;
  T.nd = nd;
  T.ncells = ncells;
  const size_t idsz = sizeof(int32_t) * (size_t)ncells * nd;
  GFE_TRY(T.cell_rows.reserve(idsz));
  GFE_CUDA_TRY(cudaMemcpyAsync(T.cell_rows.ptr, d_rows, idsz, cudaMemcpyDeviceToDevice,
                               ctx->stream));
  GFE_TRY(build_refs(ctx, &T));
  StoredCells src{};
  src.mat = nullptr;
  src.vec = d_cellvecs;
  src.vcs = nd;
  src.ves = 1;
  src.ntab = 0;
  RowArgs a;
  a.nrows = nrows;
  a.nd = nd;
  a.rowptr = nullptr;
  a.colval = nullptr;
  a.ref_ptr = T.ref_ptr.as<int64_t>();
  a.refs = T.refs.as<int32_t>();
  a.cell_cols = nullptr;
  a.val = nullptr;
  a.b = d_b;
  a.err = ctx->d_err;
  GFE_TRY((vector_only_rows<StoredCells, true>(ctx, a, src)));
  return check_device_error(ctx, "numeric_loop_vector");
}

// ---- element kernel: Q1 cells with nodal (possibly distorted) geometry --------------------
// One thread per cell, following the per-quadrature-point steps of Gridap's lazy cell
// arrays: Jt_q = sum_a grad phi_a(xi_q) (x) x_a (Geometry/Grids.jl:237-241), inv and det
// (TensorValues/Operations.jl:875-934), grad phi_i = invJt . grad phi_hat_i
// (Fields/FieldsInterfaces.jl:98-106), K_ij += ((kappa grad v_i) . grad u_j) |det Jt| w_q
// (Fields/FieldsInterfaces.jl:708-720). Output in entry-major layout
// K[(li + lj*nd)*ncells + cell], b[li*ncells + cell] for coalesced stores and loads.
template <int D, typename T>
__global__ void k_q1_cells_nodal(int64_t ncells, const int32_t* __restrict__ cell_nodes,
                                 const double* __restrict__ coords,
                                 const double* __restrict__ tabs, int nq, int coef_kind,
                                 const double* __restrict__ coef, int src_kind,
                                 const double* __restrict__ src, double* __restrict__ K,
                                 double* __restrict__ bvec, DevError* err) {
  constexpr int NV = 1 << D;
  extern __shared__ double st[];  // w[nq] | phi[nq*NV] | dphi[nq*NV*D]
  const int ntab = nq * (1 + NV + NV * D);
  for (int i = threadIdx.x; i < ntab; i += blockDim.x) st[i] = tabs[i];
  __syncthreads();
  const double* w = st;
  const double* phi = w + nq;
  const double* dphi = phi + nq * NV;
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncells) return;
  T x[NV][D];
  int64_t nid[NV];
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    nid[a] = (int64_t)__ldg(cell_nodes + cell * NV + a) - 1;
#pragma unroll
    for (int d = 0; d < D; ++d) x[a][d] = (T)__ldg(coords + nid[a] * D + d);
  }
  T kap = (T)1;
  if (coef_kind == GFE_COEF_CELL) kap = (T)__ldg(coef + cell);
  else if (coef_kind == GFE_COEF_CONST) kap = (T)__ldg(coef);
  T Ke[NV][NV];
  T be[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    be[i] = (T)0;
#pragma unroll
    for (int j = 0; j < NV; ++j) Ke[i][j] = (T)0;
  }
  for (int q = 0; q < nq; ++q) {
    T Jt[D][D];
#pragma unroll
    for (int k = 0; k < D; ++k)
#pragma unroll
      for (int l = 0; l < D; ++l) Jt[k][l] = (T)0;
#pragma unroll
    for (int a = 0; a < NV; ++a)
#pragma unroll
      for (int k = 0; k < D; ++k) {
        const T g = (T)dphi[(q * NV + a) * D + k];
#pragma unroll
        for (int l = 0; l < D; ++l) Jt[k][l] += g * x[a][l];
      }
    T det, iJ[D][D];
    if (D == 2) {
      det = Jt[0][0] * Jt[1][1] - Jt[0][1] * Jt[1][0];
      const T c = (T)1 / det;
      iJ[0][0] = Jt[1][1] * c;
      iJ[0][1] = -Jt[0][1] * c;
      iJ[1][0] = -Jt[1][0] * c;
      iJ[1][1] = Jt[0][0] * c;
    } else {
      const T a11 = Jt[0][0], a12 = Jt[0][1], a13 = Jt[0][2];
      const T a21 = Jt[1][0], a22 = Jt[1][1], a23 = Jt[1][2];
      const T a31 = Jt[2][0], a32 = Jt[2][1], a33 = Jt[2][2];
      det = a11 * a22 * a33 + a12 * a23 * a31 + a13 * a21 * a32 -
            (a11 * a23 * a32 + a12 * a21 * a33 + a13 * a22 * a31);
      const T c = (T)1 / det;
      iJ[0][0] = (a22 * a33 - a23 * a32) * c;
      iJ[1][0] = -(a21 * a33 - a23 * a31) * c;
      iJ[2][0] = (a21 * a32 - a22 * a31) * c;
      iJ[0][1] = -(a12 * a33 - a13 * a32) * c;
      iJ[1][1] = (a11 * a33 - a13 * a31) * c;
      iJ[2][1] = -(a11 * a32 - a12 * a31) * c;
      iJ[0][2] = (a12 * a23 - a13 * a22) * c;
      iJ[1][2] = -(a11 * a23 - a13 * a21) * c;
      iJ[2][2] = (a11 * a22 - a12 * a21) * c;
    }
    if (!(det != (T)0) || !isfinite((double)det)) {
      raise_err(err, GFE_ERR_DEGENERATE_CELL, cell);
      return;
    }
    const T dV = (det < (T)0 ? -det : det) * (T)w[q];
    T g[NV][D];
#pragma unroll
    for (int a = 0; a < NV; ++a)
#pragma unroll
      for (int k = 0; k < D; ++k) {
        T s = (T)0;
#pragma unroll
        for (int l = 0; l < D; ++l) s += iJ[k][l] * (T)dphi[(q * NV + a) * D + l];
        g[a][k] = s;
      }
#pragma unroll
    for (int j = 0; j < NV; ++j)
#pragma unroll
      for (int i = 0; i < NV; ++i) {
        T s = (T)0;
#pragma unroll
        for (int k = 0; k < D; ++k) s += (kap * g[i][k]) * g[j][k];
        Ke[i][j] += s * dV;
      }
    if (src_kind != GFE_SRC_NONE) {
      T fq = (T)0;
      if (src_kind == GFE_SRC_CONST) fq = (T)__ldg(src);
      else if (src_kind == GFE_SRC_NODAL) {
#pragma unroll
        for (int a = 0; a < NV; ++a) fq += (T)__ldg(src + nid[a]) * (T)phi[q * NV + a];
      } else if (src_kind == GFE_SRC_QPOINT) fq = (T)__ldg(src + cell * nq + q);
#pragma unroll
      for (int i = 0; i < NV; ++i) be[i] += (fq * (T)phi[q * NV + i]) * dV;
    }
  }
#pragma unroll
  for (int j = 0; j < NV; ++j)
#pragma unroll
    for (int i = 0; i < NV; ++i) K[(int64_t)(i + j * NV) * ncells + cell] = (double)Ke[i][j];
  if (bvec)
#pragma unroll
    for (int i = 0; i < NV; ++i) bvec[(int64_t)i * ncells + cell] = (double)be[i];
}

// ---- f(x) = sum_k a_k prod_d sin(pi m_kd x_d) at the quadrature points of Cartesian cells
template <int D>
__global__ void k_sinsum_qpoints(int64_t ncells, int64_t n0, int64_t n1, double x0, double y0,
                                 double z0, double hx, double hy, double hz,
                                 const double* __restrict__ qx, int nq,
                                 const double* __restrict__ terms, int nterms,
                                 double* __restrict__ fq) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= ncells * nq) return;
  const int64_t cell = idx / nq;
  const int q = (int)(idx - cell * nq);
  const int64_t I[3] = {cell % n0, (cell / n0) % n1, cell / (n0 * n1)};
  const double o[3] = {x0, y0, z0}, h[3] = {hx, hy, hz};
  double x[3];
  for (int d = 0; d < D; ++d) {
    // physical point: xi . diag(h) + cell origin (Fields/AffineMaps.jl:57-62)
    const double org = o[d] + (double)I[d] * h[d];
    x[d] = qx[q * D + d] * h[d] + org;
  }
  const double pi = 3.14159265358979323846;
  double f = 0.0;
  for (int k = 0; k < nterms; ++k) {
    const double* t = terms + k * (1 + D);
    double p = t[0];
    for (int d = 0; d < D; ++d) p *= sin(pi * t[1 + d] * x[d]);
    f += p;
  }
  fq[idx] = f;
}

// (pairs of doubles where v is 16-byte aligned; the reported index is the element's)
__global__ void k_check_finite(const double* __restrict__ v, int64_t n, DevError* err) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  int64_t done = 0;
  if ((reinterpret_cast<uintptr_t>(v) & 15) == 0) {
    const int64_t n2 = n >> 1;
    for (int64_t i = tid; i < n2; i += nth) {
      const double2 w = __ldg(reinterpret_cast<const double2*>(v) + i);
      if (!isfinite(w.x)) raise_err(err, GFE_ERR_NONFINITE, 2 * i);
      if (!isfinite(w.y)) raise_err(err, GFE_ERR_NONFINITE, 2 * i + 1);
    }
    done = 2 * n2;
  }
  for (int64_t i = done + tid; i < n; i += nth)
    if (!isfinite(v[i])) raise_err(err, GFE_ERR_NONFINITE, i);
}

// ---- host: reference tables ---------------------------------------------------------------
// Reference tables of a uniform Cartesian cell with sizes h (FP64, same steps as the
// per-cell integral with Jt = diag(h)).
static void cartesian_tables(int D, const double* h, int nq, const std::vector<double>& qx,
                             const std::vector<double>& qw, std::vector<double>& out) {
  const int nv = 1 << D;
  std::vector<double> phi, dphi;
  q1_shapes(D, nq, qx.data(), phi, dphi);
  out.assign((size_t)nv * nv * 2 + nv + (size_t)nq * nv, 0.0);
  double* K = out.data();
  double* M = K + nv * nv;
  double* m = M + nv * nv;
  double* PW = m + nv;
  double det = 1.0;
  for (int d = 0; d < D; ++d) det *= h[d];
  for (int q = 0; q < nq; ++q) {
    const double dV = std::fabs(det) * qw[q];
    double g[8][3];
    for (int a = 0; a < nv; ++a)
      for (int k = 0; k < D; ++k) g[a][k] = (1.0 / h[k]) * dphi[((size_t)q * nv + a) * D + k];
    for (int j = 0; j < nv; ++j)
      for (int i = 0; i < nv; ++i) {
        double s = 0.0;
        for (int k = 0; k < D; ++k) s += g[i][k] * g[j][k];
        K[i + j * nv] += s * dV;
        M[i + j * nv] += (phi[(size_t)q * nv + i] * phi[(size_t)q * nv + j]) * dV;
      }
    for (int i = 0; i < nv; ++i) {
      m[i] += phi[(size_t)q * nv + i] * dV;
      PW[q * nv + i] = phi[(size_t)q * nv + i] * dV;
    }
  }
}

// W[c] = Kref[0, c] of the unit cube's Q1 stiffness (degree-2 rule): the entry between two
// vertices that differ along the axes in the bit set c (bit 0 x, bit 1 y, bit 2 z).
void q1_unit_stiffness_classes(double W[8]) {
  std::vector<double> qx, qw, tabs;
  tensor_quadrature(3, 2, qx, qw);
  const double h[3] = {1.0, 1.0, 1.0};
  cartesian_tables(3, h, (int)qw.size(), qx, qw, tabs);
  for (int c = 0; c < 8; ++c) W[c] = tabs[0 + 8 * c];
}

// ---- Q2 (27-node HEX, 9-node QUAD) cell integrals ----------------------------------------
// The diffusion cell matrix on a cell with (multi)linear geometry is
//     K = B^T D B,   B[(q,k), i] = d phi_hat_i / d xi_k (xi_q)   (same for every cell),
//     D = blockdiag_q( G_q ),  G_q = kappa |det Jt_q| w_q  invJt_q^T invJt_q   (3x3 per q),
// which is Gridap's sum over q of (kappa invJt grad phi_i).(invJt grad phi_j) |det Jt| w_q
// (Fields/FieldsInterfaces.jl:708-720, Fields/ApplyOptimizations.jl:293-310) regrouped.
// Jacobians, inverses and determinants are always FP64 (distorted cells).
struct Q2Tables {
  int D, nn, nq, nv;  // dims, nodes (27/9), q-points, geometry vertices (8/4)
};

// G_q for one cell into g[q*9] (FP64); returns false on a degenerate cell.
template <int D>
__device__ bool q2_metric(const double* __restrict__ xv, const double* __restrict__ dphi1,
                          const double* __restrict__ w, int nq, double kap, double* g,
                          double* dv) {
  constexpr int NV = 1 << D;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    double Jt[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int a = 0; a < NV; ++a)
      for (int k = 0; k < D; ++k) {
        const double gk = dphi1[(q * NV + a) * D + k];
        for (int l = 0; l < D; ++l) Jt[k][l] += gk * xv[a * D + l];
      }
    double det, iJ[3][3];
    if (D == 2) {
      det = Jt[0][0] * Jt[1][1] - Jt[0][1] * Jt[1][0];
      const double c = 1.0 / det;
      iJ[0][0] = Jt[1][1] * c;
      iJ[0][1] = -Jt[0][1] * c;
      iJ[1][0] = -Jt[1][0] * c;
      iJ[1][1] = Jt[0][0] * c;
    } else {
      const double a11 = Jt[0][0], a12 = Jt[0][1], a13 = Jt[0][2];
      const double a21 = Jt[1][0], a22 = Jt[1][1], a23 = Jt[1][2];
      const double a31 = Jt[2][0], a32 = Jt[2][1], a33 = Jt[2][2];
      det = a11 * a22 * a33 + a12 * a23 * a31 + a13 * a21 * a32 -
            (a11 * a23 * a32 + a12 * a21 * a33 + a13 * a22 * a31);
      const double c = 1.0 / det;
      iJ[0][0] = (a22 * a33 - a23 * a32) * c;
      iJ[1][0] = -(a21 * a33 - a23 * a31) * c;
      iJ[2][0] = (a21 * a32 - a22 * a31) * c;
      iJ[0][1] = -(a12 * a33 - a13 * a32) * c;
      iJ[1][1] = (a11 * a33 - a13 * a31) * c;
      iJ[2][1] = -(a11 * a32 - a12 * a31) * c;
      iJ[0][2] = (a12 * a23 - a13 * a22) * c;
      iJ[1][2] = -(a11 * a23 - a13 * a21) * c;
      iJ[2][2] = (a11 * a22 - a12 * a21) * c;
    }
    if (!(det != 0.0) || !isfinite(det)) return false;
    const double s = kap * fabs(det) * w[q];
    dv[q] = fabs(det) * w[q];
    // G = s * iJ^T iJ  (grad_i . grad_j = (iJ g_i).(iJ g_j) = g_i^T iJ^T iJ g_j)
    for (int k = 0; k < D; ++k)
      for (int l = 0; l < D; ++l) {
        double t = 0.0;
        for (int m = 0; m < D; ++m) t += iJ[m][k] * iJ[m][l];
        g[q * 9 + k * 3 + l] = s * t;
      }
  }
  return true;
}

// FP64 Q2 cell matrices: one block per cell (grid-stride over cells). Output entry-major:
// K[(i + j*nn)*ncells + cell], b[i*ncells + cell].
template <int D>
__global__ void __launch_bounds__(256)
    k_q2_cells_fp64(int64_t ncells, const int32_t* __restrict__ cell_vertices,
                    const double* __restrict__ coords, const double* __restrict__ tabs, int nq,
                    int coef_kind, const double* __restrict__ coef, int src_kind,
                    const double* __restrict__ src, double* __restrict__ K,
                    double* __restrict__ bvec, DevError* err) {
  constexpr int NV = 1 << D, NN = D == 2 ? 9 : 27;
  extern __shared__ double sm[];
  // tables: w[nq] | phi2[nq*NN] | dphi1[nq*NV*D] | B[(q*D+k)*NN + i]
  const int nB = nq * D * NN;
  const int ntab = nq + nq * NN + nq * NV * D + nB;
  double* w = sm;
  double* phi2 = w + nq;
  double* dphi1 = phi2 + nq * NN;
  double* B = dphi1 + nq * NV * D;
  double* G = sm + ntab;                // nq*9
  double* dv = G + nq * 9;              // nq
  double* C = dv + nq;                  // nB: C[(q*D+k)*NN + j]
  double* xv = C + nB;                  // NV*D
  for (int i = threadIdx.x; i < ntab; i += blockDim.x) sm[i] = tabs[i];
  __syncthreads();
  for (int64_t cell = blockIdx.x; cell < ncells; cell += gridDim.x) {
    if (threadIdx.x < NV * D) {
      const int a = threadIdx.x / D, d = threadIdx.x % D;
      xv[threadIdx.x] = coords[((int64_t)cell_vertices[cell * NV + a] - 1) * D + d];
    }
    const double kap = coef_kind == GFE_COEF_CELL ? coef[cell]
                       : coef_kind == GFE_COEF_CONST ? coef[0] : 1.0;
    __syncthreads();
    const bool ok = q2_metric<D>(xv, dphi1, w, nq, kap, G, dv);
    if (!ok) raise_err(err, GFE_ERR_DEGENERATE_CELL, cell);
    __syncthreads();
    // C = D B
    for (int idx = threadIdx.x; idx < nB; idx += blockDim.x) {
      const int j = idx % NN, qk = idx / NN, q = qk / D, k = qk % D;
      double s = 0.0;
      for (int l = 0; l < D; ++l) s += G[q * 9 + k * 3 + l] * B[(q * D + l) * NN + j];
      C[idx] = s;
    }
    __syncthreads();
    // K = B^T C over the upper triangle only (i <= j), mirrored. The triangle is enumerated
    // directly -- column j holds rows 0..j, so entry t lies in column j with
    // j(j+1)/2 <= t < (j+1)(j+2)/2 -- so that no lane of an FP64 warp instruction idles.
    for (int t = threadIdx.x; t < NN * (NN + 1) / 2; t += blockDim.x) {
      int j = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
      while (j * (j + 1) / 2 > t) --j;
      while ((j + 1) * (j + 2) / 2 <= t) ++j;
      const int i = t - j * (j + 1) / 2;
      double s = 0.0;
      for (int qk = 0; qk < nq * D; ++qk) s += B[qk * NN + i] * C[qk * NN + j];
      K[(int64_t)(i + j * NN) * ncells + cell] = s;
      K[(int64_t)(j + i * NN) * ncells + cell] = s;
    }
    if (bvec)
      for (int i = threadIdx.x; i < NN; i += blockDim.x) {
        double s = 0.0;
        if (src_kind != GFE_SRC_NONE)
          for (int q = 0; q < nq; ++q) {
            const double fq = src_kind == GFE_SRC_CONST ? src[0] : src[cell * nq + q];
            s += (fq * phi2[q * NN + i]) * dv[q];
          }
        bvec[(int64_t)i * ncells + cell] = s;
      }
    __syncthreads();
  }
}


// ---- host: fused integrate + assemble -----------------------------------------------------
int assemble_problem(gfe_ctx* ctx, const gfe_problem* p, gfe_matrix* A, double* d_b) {
  // the values of a closed-form Cartesian pattern are zeroed lazily: only the class-sum
  // kernel, which writes every entry, may find them pending
  const bool lattice_candidate = A && A->val_pending && p->dim == 3 &&
                                 p->reffe == GFE_REFFE_Q1 && p->ncomp == 1 &&
                                 p->form == GFE_FORM_DIFFUSION &&
                                 p->geometry == GFE_GEOM_CARTESIAN;
  if (!lattice_candidate) GFE_TRY(ensure_values(ctx, A));
  if (A) A->zf_values = false;  // set again by the class-sum kernel when it writes them
  if (p->reffe == GFE_REFFE_P2_TET) return assemble_p2_elasticity(ctx, p, A, d_b);
  if (p->form == GFE_FORM_QUASILINEAR) return assemble_quasilinear(ctx, p, A, d_b);
  const int D = p->dim;
  if ((p->reffe != GFE_REFFE_Q1 && p->reffe != GFE_REFFE_Q2) || p->ncomp != 1 ||
      p->form != GFE_FORM_DIFFUSION)
    return set_error(GFE_ERR_UNSUPPORTED, "assemble: scalar Q1/Q2 diffusion is provided");
  if (D != 2 && D != 3) return set_error(GFE_ERR_UNSUPPORTED, "assemble: dim must be 2 or 3");
  const int nv = 1 << D;
  const bool q2 = p->reffe == GFE_REFFE_Q2;
  const int nn = q2 ? (D == 2 ? 9 : 27) : nv;
  if (p->nd != nn) return set_error(GFE_ERR_INVALID_ARGUMENT, "assemble: nd does not match the element");
  if (A && (A->ncells != p->ncells || A->nd != p->nd ||
            A->cols_per_cell() != p->nd))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "assemble: matrix pattern built for other cells");
  std::vector<double> qx, qw;
  GFE_TRY(tensor_quadrature(D, p->degree, qx, qw));
  const int nq = (int)qw.size();
  const int64_t ncells = p->ncells;
  const bool fp32 = p->precision == GFE_PREC_FP32;

  // coefficient / source to the device
  const double* d_coef = nullptr;
  if (p->coef_kind == GFE_COEF_CONST || p->coef_kind == GFE_COEF_CELL) {
    const size_t n = p->coef_kind == GFE_COEF_CELL ? (size_t)ncells : 1;
    const void* v;
    GFE_TRY(device_view(ctx, p->coef, sizeof(double) * n, SCR_COEF, &v));
    d_coef = (const double*)v;
    k_check_finite<<<grid_for((int64_t)n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(
        d_coef, (int64_t)n, ctx->d_err);
    ctx->launches++;
  }
  int src_kind = p->source_kind;
  const double* d_src = nullptr;
  if (src_kind == GFE_SRC_CONST || src_kind == GFE_SRC_NODAL || src_kind == GFE_SRC_QPOINT) {
    const void* v;
    GFE_TRY(device_view(ctx, p->source, sizeof(double) * p->source_len, SCR_SRC, &v));
    d_src = (const double*)v;
  } else if (src_kind == GFE_SRC_SINSUM) {
    if (p->geometry != GFE_GEOM_CARTESIAN)
      return set_error(GFE_ERR_UNSUPPORTED, "assemble: SINSUM source needs Cartesian cells");
    const int nterms = (int)p->source[0];
    if (nterms < 0 || p->source_len < 1 + (int64_t)nterms * (1 + D))
      return set_error(GFE_ERR_INVALID_ARGUMENT, "assemble: malformed SINSUM source");
    // terms + quadrature points to the device, evaluate f at all quadrature points
    const size_t tb = sizeof(double) * (size_t)nterms * (1 + D), qb = sizeof(double) * qx.size();
    GFE_TRY(ctx->scratch[SCR_TMP2].reserve(tb + qb + 64));
    double* dterms = ctx->scratch[SCR_TMP2].as<double>();
    double* dqx = dterms + (size_t)nterms * (1 + D);
    if (tb) GFE_CUDA_TRY(cudaMemcpyAsync(dterms, p->source + 1, tb, cudaMemcpyHostToDevice,
                                         ctx->stream));
    GFE_CUDA_TRY(cudaMemcpyAsync(dqx, qx.data(), qb, cudaMemcpyHostToDevice, ctx->stream));
    GFE_TRY(ctx->scratch[SCR_SRC].reserve(sizeof(double) * (size_t)ncells * nq));
    double h[3] = {1, 1, 1}, o[3] = {0, 0, 0};
    for (int d = 0; d < D; ++d) {
      o[d] = p->domain[2 * d];
      h[d] = (p->domain[2 * d + 1] - p->domain[2 * d]) / (double)p->partition[d];
    }
    const int64_t nt = ncells * nq;
    if (D == 2)
      k_sinsum_qpoints<2><<<grid_for(nt, 256), 256, 0, ctx->stream>>>(
          ncells, p->partition[0], p->partition[1], o[0], o[1], o[2], h[0], h[1], h[2], dqx, nq,
          dterms, nterms, ctx->scratch[SCR_SRC].as<double>());
    else
      k_sinsum_qpoints<3><<<grid_for(nt, 256), 256, 0, ctx->stream>>>(
          ncells, p->partition[0], p->partition[1], o[0], o[1], o[2], h[0], h[1], h[2], dqx, nq,
          dterms, nterms, ctx->scratch[SCR_SRC].as<double>());
    ctx->launches++;
    d_src = ctx->scratch[SCR_SRC].as<double>();
    src_kind = GFE_SRC_QPOINT;
  }
  if (d_src && src_kind != GFE_SRC_NONE) {
    const int64_t n = src_kind == GFE_SRC_QPOINT ? ncells * nq : p->source_len;
    k_check_finite<<<grid_for(n, 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(d_src, n,
                                                                              ctx->d_err);
    ctx->launches++;
  }
  GFE_CUDA_TRY(cudaGetLastError());

  // rows of the assembly: the matrix's rows, or (vector only) the problem's cell ids
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
  const int maxw = A ? A->max_width : 1;

  if (q2) {
    if (src_kind == GFE_SRC_NODAL)
      return set_error(GFE_ERR_UNSUPPORTED, "assemble: nodal sources are Q1 only");
    if (!p->node_coords || !p->cell_node_ids)
      return set_error(GFE_ERR_INVALID_ARGUMENT, "assemble: Q2 needs node coordinates and "
                                                 "cell vertex ids");
    const void* vc;
    const void* vn;
    GFE_TRY(device_view(ctx, p->node_coords, sizeof(double) * (size_t)p->nnodes * D, SCR_COORDS,
                        &vc));
    GFE_TRY(device_view(ctx, p->cell_node_ids, sizeof(int32_t) * (size_t)ncells * nv,
                        SCR_CELLNODES, &vn));
    std::vector<double> phi1, dphi1, phi2, dphi2;
    q1_shapes(D, nq, qx.data(), phi1, dphi1);
    q2_shapes(D, nq, qx.data(), phi2, dphi2);
    std::vector<double> tabs(qw);
    tabs.insert(tabs.end(), phi2.begin(), phi2.end());
    tabs.insert(tabs.end(), dphi1.begin(), dphi1.end());
    for (int q = 0; q < nq; ++q)  // B[(q*D+k)*nn + i]
      for (int k = 0; k < D; ++k)
        for (int i = 0; i < nn; ++i) tabs.push_back(dphi2[((size_t)q * nn + i) * D + k]);
    GFE_TRY(ctx->scratch[SCR_TMP1].reserve(sizeof(double) * tabs.size()));
    GFE_CUDA_TRY(cudaMemcpyAsync(ctx->scratch[SCR_TMP1].ptr, tabs.data(),
                                 sizeof(double) * tabs.size(), cudaMemcpyHostToDevice,
                                 ctx->stream));
    GFE_TRY(ctx->scratch[SCR_CELLMAT].reserve(sizeof(double) * (size_t)ncells * nn * nn));
    GFE_TRY(ctx->scratch[SCR_CELLVEC].reserve(sizeof(double) * (size_t)ncells * nn));
    if (fp32) {
      if (D != 3)
        return set_error(GFE_ERR_UNSUPPORTED, "assemble: the tensor-core Q2 path is 3-D");
      if (nq != 27)
        return set_error(GFE_ERR_UNSUPPORTED, "assemble: the tensor-core Q2 path needs degree 4");
      float* Kf = ctx->scratch[SCR_CELLMAT].as<float>();
      float* bf = ctx->scratch[SCR_CELLVEC].as<float>();
      if (src_kind == GFE_SRC_NONE)
        GFE_CUDA_TRY(cudaMemsetAsync(bf, 0, sizeof(float) * (size_t)ncells * nn, ctx->stream));
      timer_begin(ctx, GFE_KT_ELEMENT);
      GFE_TRY(launch_q2_cells_tc(ctx, ncells, (const int32_t*)vn, (const double*)vc,
                                 ctx->scratch[SCR_TMP1].as<double>(), tabs.data(),
                                 p->coef_kind, d_coef, src_kind, d_src, Kf, bf));
      timer_end(ctx);
      GFE_TRY(check_device_error(ctx, "assemble (Q2 tensor-core cell integrals)"));
      StoredCellsF32 s{};
      s.mat = Kf;
      s.vec = bf;
      s.cs = (int64_t)nn * nn;
      s.es = 1;
      s.vcs = nn;
      s.ves = 1;
      s.ntab = 0;
      GFE_TRY(ensure_row_refs(ctx, R));
      RowArgs a = row_args(ctx, R, d_b, A != nullptr);
      if (A) {
        GFE_TRY(run_rows(ctx, a, s, maxw, A->pos_bytes));
        if (D == 3) GFE_TRY(attach_q2_pmg(ctx, A, p, d_coef));
      } else {
        GFE_TRY(vector_only_rows(ctx, a, s));
      }
      return check_device_error(ctx, "assemble_matrix_and_vector");
    }
    const size_t sm = sizeof(double) * (tabs.size() + (size_t)nq * 10 + (size_t)nq * D * nn +
                                        (size_t)nv * D);
    const unsigned grid = (unsigned)std::min<int64_t>(ncells, (int64_t)ctx->num_sms * 8);
    timer_begin(ctx, GFE_KT_ELEMENT);
    if (D == 2) {
      auto kern = k_q2_cells_fp64<2>;
      GFE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)sm));
      kern<<<grid, 256, sm, ctx->stream>>>(ncells, (const int32_t*)vn, (const double*)vc,
                                           ctx->scratch[SCR_TMP1].as<double>(), nq, p->coef_kind,
                                           d_coef, src_kind, d_src,
                                           ctx->scratch[SCR_CELLMAT].as<double>(),
                                           ctx->scratch[SCR_CELLVEC].as<double>(), ctx->d_err);
    } else {
      auto kern = k_q2_cells_fp64<3>;
      GFE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)sm));
      kern<<<grid, 256, sm, ctx->stream>>>(ncells, (const int32_t*)vn, (const double*)vc,
                                           ctx->scratch[SCR_TMP1].as<double>(), nq, p->coef_kind,
                                           d_coef, src_kind, d_src,
                                           ctx->scratch[SCR_CELLMAT].as<double>(),
                                           ctx->scratch[SCR_CELLVEC].as<double>(), ctx->d_err);
    }
    timer_end(ctx);
    ctx->launches++;
    GFE_CUDA_TRY(cudaGetLastError());
    GFE_TRY(check_device_error(ctx, "assemble (Q2 cell integrals)"));
    StoredCells s{};
    s.mat = ctx->scratch[SCR_CELLMAT].as<double>();
    s.vec = ctx->scratch[SCR_CELLVEC].as<double>();
    s.cs = 1;
    s.es = ncells;
    s.vcs = 1;
    s.ves = ncells;
    s.ntab = 0;
    GFE_TRY(ensure_row_refs(ctx, R));
    RowArgs a = row_args(ctx, R, d_b, A != nullptr);
    if (A) {
      GFE_TRY(run_rows(ctx, a, s, maxw, A->pos_bytes));
      if (D == 3) GFE_TRY(attach_q2_pmg(ctx, A, p, d_coef));
    } else {
      GFE_TRY(vector_only_rows(ctx, a, s));
    }
  } else if (p->geometry == GFE_GEOM_CARTESIAN) {
    double h[3] = {1, 1, 1};
    for (int d = 0; d < D; ++d)
      h[d] = (p->domain[2 * d + 1] - p->domain[2 * d]) / (double)p->partition[d];
    std::vector<double> tabs;
    cartesian_tables(D, h, nq, qx, qw, tabs);
    GFE_TRY(ctx->scratch[SCR_TMP1].reserve(sizeof(double) * tabs.size()));
    GFE_CUDA_TRY(cudaMemcpyAsync(ctx->scratch[SCR_TMP1].ptr, tabs.data(),
                                 sizeof(double) * tabs.size(), cudaMemcpyHostToDevice,
                                 ctx->stream));
    const int32_t* cn = nullptr;
    if (p->cell_node_ids && src_kind == GFE_SRC_NODAL) {
      const void* v;
      GFE_TRY(device_view(ctx, p->cell_node_ids, sizeof(int32_t) * (size_t)ncells * nv,
                          SCR_CELLNODES, &v));
      cn = (const int32_t*)v;
    }
    // the closed-form lattice pattern of this grid: the class-sum kernel
    bool lattice_done = false;
    if (A && D == 3 && !cn) {
      // the coefficient and source checks report before the class-sum kernel, which raises
      // no device errors itself: the call then returns without waiting for it
      GFE_TRY(check_device_error(ctx, "assemble_matrix_and_vector"));
      GFE_TRY(assemble_cartesian_q1_lattice(ctx, A, p, d_coef, src_kind, d_src, tabs.data(),
                                            tabs.data() + 2 * nv * nv, d_b, &lattice_done));
    }
    if (lattice_done)
      A->val_pending = false;
    else
      GFE_TRY(ensure_values(ctx, A));
    if (!lattice_done) GFE_TRY(ensure_row_refs(ctx, R));
    RowArgs a = row_args(ctx, R, d_b, A != nullptr);
    if (!A) a.rowptr = nullptr;
#define GFE_CART(DD, F32)                                                               \
  {                                                                                     \
    CartesianDiffusionQ1<DD, F32> s;                                                    \
    s.tables = ctx->scratch[SCR_TMP1].as<double>();                                     \
    s.nq = nq;                                                                          \
    s.coef_kind = p->coef_kind;                                                         \
    s.coef = d_coef;                                                                    \
    s.src_kind = src_kind;                                                              \
    s.src = d_src;                                                                      \
    s.n0 = p->partition[0];                                                             \
    s.n1 = p->partition[1];                                                             \
    s.cell_nodes = cn;                                                                  \
    s.ntab = (int)tabs.size();                                                          \
    if (A) {                                                                            \
      GFE_TRY(run_rows(ctx, a, s, maxw, A->pos_bytes));                                 \
    } else {                                                                            \
      GFE_TRY(vector_only_rows(ctx, a, s));                                             \
    }                                                                                   \
  }
    if (lattice_done) {
    } else if (D == 2 && !fp32) GFE_CART(2, false)
    else if (D == 2) GFE_CART(2, true)
    else if (!fp32) GFE_CART(3, false)
    else GFE_CART(3, true)
#undef GFE_CART
    if (A && D == 3) GFE_TRY(attach_lattice_operator(ctx, A, p, d_coef, tabs.data()));
    if (lattice_done) {
      GFE_CUDA_TRY(cudaGetLastError());
      return GFE_OK;
    }
  } else {
    // nodal geometry: element kernel into entry-major scratch, then the row gather
    if (!p->node_coords || !p->cell_node_ids)
      return set_error(GFE_ERR_INVALID_ARGUMENT, "assemble: nodal geometry needs coordinates");
    const void* vc;
    const void* vn;
    GFE_TRY(device_view(ctx, p->node_coords, sizeof(double) * (size_t)p->nnodes * D, SCR_COORDS,
                        &vc));
    GFE_TRY(device_view(ctx, p->cell_node_ids, sizeof(int32_t) * (size_t)ncells * nv,
                        SCR_CELLNODES, &vn));
    std::vector<double> phi, dphi;
    q1_shapes(D, nq, qx.data(), phi, dphi);
    std::vector<double> tabs(qw);
    tabs.insert(tabs.end(), phi.begin(), phi.end());
    tabs.insert(tabs.end(), dphi.begin(), dphi.end());
    GFE_TRY(ctx->scratch[SCR_TMP1].reserve(sizeof(double) * tabs.size()));
    GFE_CUDA_TRY(cudaMemcpyAsync(ctx->scratch[SCR_TMP1].ptr, tabs.data(),
                                 sizeof(double) * tabs.size(), cudaMemcpyHostToDevice,
                                 ctx->stream));
    GFE_TRY(ctx->scratch[SCR_CELLMAT].reserve(sizeof(double) * (size_t)ncells * nv * nv));
    GFE_TRY(ctx->scratch[SCR_CELLVEC].reserve(sizeof(double) * (size_t)ncells * nv));
    const size_t sm = sizeof(double) * tabs.size();
    const int blk = 128;
    if (D == 2) {
      if (fp32)
        k_q1_cells_nodal<2, float><<<grid_for(ncells, blk), blk, sm, ctx->stream>>>(
            ncells, (const int32_t*)vn, (const double*)vc, ctx->scratch[SCR_TMP1].as<double>(),
            nq, p->coef_kind, d_coef, src_kind, d_src, ctx->scratch[SCR_CELLMAT].as<double>(),
            ctx->scratch[SCR_CELLVEC].as<double>(), ctx->d_err);
      else
        k_q1_cells_nodal<2, double><<<grid_for(ncells, blk), blk, sm, ctx->stream>>>(
            ncells, (const int32_t*)vn, (const double*)vc, ctx->scratch[SCR_TMP1].as<double>(),
            nq, p->coef_kind, d_coef, src_kind, d_src, ctx->scratch[SCR_CELLMAT].as<double>(),
            ctx->scratch[SCR_CELLVEC].as<double>(), ctx->d_err);
    } else {
      if (fp32)
        k_q1_cells_nodal<3, float><<<grid_for(ncells, blk), blk, sm, ctx->stream>>>(
            ncells, (const int32_t*)vn, (const double*)vc, ctx->scratch[SCR_TMP1].as<double>(),
            nq, p->coef_kind, d_coef, src_kind, d_src, ctx->scratch[SCR_CELLMAT].as<double>(),
            ctx->scratch[SCR_CELLVEC].as<double>(), ctx->d_err);
      else
        k_q1_cells_nodal<3, double><<<grid_for(ncells, blk), blk, sm, ctx->stream>>>(
            ncells, (const int32_t*)vn, (const double*)vc, ctx->scratch[SCR_TMP1].as<double>(),
            nq, p->coef_kind, d_coef, src_kind, d_src, ctx->scratch[SCR_CELLMAT].as<double>(),
            ctx->scratch[SCR_CELLVEC].as<double>(), ctx->d_err);
    }
    ctx->launches++;
    GFE_CUDA_TRY(cudaGetLastError());
    GFE_TRY(check_device_error(ctx, "assemble (cell integrals)"));
    StoredCells s{};
    s.mat = ctx->scratch[SCR_CELLMAT].as<double>();
    s.vec = ctx->scratch[SCR_CELLVEC].as<double>();
    s.cs = 1;
    s.es = ncells;
    s.vcs = 1;
    s.ves = ncells;
    s.ntab = 0;
    GFE_TRY(ensure_row_refs(ctx, R));
    RowArgs a = row_args(ctx, R, d_b, A != nullptr);
    if (A) {
      GFE_TRY(run_rows(ctx, a, s, maxw, A->pos_bytes));
    } else {
      GFE_TRY(vector_only_rows(ctx, a, s));
    }
  }
  return check_device_error(ctx, "assemble_matrix_and_vector");
}

}  // namespace gfe

