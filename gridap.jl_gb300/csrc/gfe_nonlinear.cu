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

// alpha, d alpha / d u and gamma at a point (u, |grad u|^2). p = 3 (the p-Laplacian of the
// reference tests) and p = 4 use sqrt / plain products instead of pow.
__device__ __forceinline__ void law_values(int law, double c0, double c1, double c2, double u,
                                           double n2, double* al, double* be, double* ga) {
  if (law == GFE_LAW_POLY) {
    *al = c0 + c1 * u + c2 * u * u;
    *be = c1 + 2.0 * c2 * u;
    *ga = 0.0;
    return;
  }
  const double s = c1 + n2;  // eps2 + |grad u|^2
  *be = 0.0;
  if (c0 == 3.0) {
    const double r = sqrt(s);
    *al = r;
    *ga = 1.0 / r;
  } else if (c0 == 4.0) {
    *al = s;
    *ga = 2.0;
  } else if (c0 == 2.0) {
    *al = 1.0;
    *ga = 0.0;
  } else {
    *al = pow(s, 0.5 * (c0 - 2.0));
    *ga = (c0 - 2.0) * pow(s, 0.5 * (c0 - 4.0));
  }
}

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
      law_values(law, c0, c1, c2, u, n2, &al, &be, &ga);
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

// Q1 cells: one thread per cell with the cell arrays in registers (2^D nodes), the same
// per-point steps as the block-per-cell kernel.
template <int D>
__global__ void __launch_bounds__(128)
    k_quasilinear_q1(int64_t ncells, const int32_t* __restrict__ cell_vertices,
                     const double* __restrict__ coords, const int32_t* __restrict__ cell_ids,
                     const double* __restrict__ state, int64_t nfree,
                     const double* __restrict__ uD, int64_t ndiri,
                     const double* __restrict__ tabs, int nq, int coef_kind,
                     const double* __restrict__ coef, int src_kind,
                     const double* __restrict__ src, int law, double c0, double c1, double c2,
                     double* __restrict__ K, double* __restrict__ bvec, DevError* err) {
  constexpr int NV = 1 << D;
  extern __shared__ double st[];  // w[nq] | phi[nq*NV] | dref[nq*NV*D] (| dphi1 = dref)
  const int ntab = nq * (1 + NV + NV * D);
  for (int i = threadIdx.x; i < ntab; i += blockDim.x) st[i] = tabs[i];
  __syncthreads();
  const double* w = st;
  const double* phi = w + nq;
  const double* dref = phi + nq * NV;
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncells) return;
  double x[NV][D], uc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const int64_t nid = (int64_t)__ldg(cell_vertices + cell * NV + v) - 1;
#pragma unroll
    for (int d = 0; d < D; ++d) x[v][d] = __ldg(coords + nid * D + d);
    const int32_t id = __ldg(cell_ids + cell * NV + v);
    double u = 0.0;
    if (id > 0 && id <= nfree) {
      u = __ldg(state + id - 1);
    } else if (id < 0 && -(int64_t)id <= ndiri) {
      u = __ldg(uD - (int64_t)id - 1);
    } else if (id != 0 && !(id < 0 && ndiri == 0)) {
      raise_err(err, GFE_ERR_INVALID_ARGUMENT, cell);
    }
    uc[v] = u;
  }
  const double kap = coef_kind == GFE_COEF_CELL ? __ldg(coef + cell)
                     : coef_kind == GFE_COEF_CONST ? __ldg(coef) : 1.0;
  double Ke[NV][NV], be[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    be[i] = 0.0;
#pragma unroll
    for (int j = 0; j < NV; ++j) Ke[i][j] = 0.0;
  }
  for (int q = 0; q < nq; ++q) {
    double Jt[D][D];
#pragma unroll
    for (int k = 0; k < D; ++k)
#pragma unroll
      for (int l = 0; l < D; ++l) Jt[k][l] = 0.0;
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
      for (int k = 0; k < D; ++k) {
        const double gr = dref[(q * NV + v) * D + k];
#pragma unroll
        for (int l = 0; l < D; ++l) Jt[k][l] += gr * x[v][l];
      }
    double det, iJ[D][D];
    if (D == 2) {
      det = Jt[0][0] * Jt[1][1] - Jt[0][1] * Jt[1][0];
      iJ[0][0] = Jt[1][1] / det;
      iJ[0][1] = -Jt[0][1] / det;
      iJ[1][0] = -Jt[1][0] / det;
      iJ[1][1] = Jt[0][0] / det;
    } else {
      const double c00 = Jt[1][1] * Jt[2][2] - Jt[1][2] * Jt[2][1];
      const double c01 = Jt[1][2] * Jt[2][0] - Jt[1][0] * Jt[2][2];
      const double c02 = Jt[1][0] * Jt[2][1] - Jt[1][1] * Jt[2][0];
      det = Jt[0][0] * c00 + Jt[0][1] * c01 + Jt[0][2] * c02;
      iJ[0][0] = c00 / det;
      iJ[0][1] = (Jt[0][2] * Jt[2][1] - Jt[0][1] * Jt[2][2]) / det;
      iJ[0][2] = (Jt[0][1] * Jt[1][2] - Jt[0][2] * Jt[1][1]) / det;
      iJ[1][0] = c01 / det;
      iJ[1][1] = (Jt[0][0] * Jt[2][2] - Jt[0][2] * Jt[2][0]) / det;
      iJ[1][2] = (Jt[0][2] * Jt[1][0] - Jt[0][0] * Jt[1][2]) / det;
      iJ[2][0] = c02 / det;
      iJ[2][1] = (Jt[0][1] * Jt[2][0] - Jt[0][0] * Jt[2][1]) / det;
      iJ[2][2] = (Jt[0][0] * Jt[1][1] - Jt[0][1] * Jt[1][0]) / det;
    }
    if (!(det != 0.0) || !isfinite(det)) raise_err(err, GFE_ERR_DEGENERATE_CELL, cell);
    const double dV = w[q] * fabs(det);
    double g[NV][D], u = 0.0, gu[D];
#pragma unroll
    for (int k = 0; k < D; ++k) gu[k] = 0.0;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      u += phi[q * NV + v] * uc[v];
#pragma unroll
      for (int k = 0; k < D; ++k) {
        double s = 0.0;
#pragma unroll
        for (int l = 0; l < D; ++l) s += iJ[k][l] * dref[(q * NV + v) * D + l];
        g[v][k] = s;
        gu[k] += s * uc[v];
      }
    }
    double n2 = 0.0;
#pragma unroll
    for (int k = 0; k < D; ++k) n2 += gu[k] * gu[k];
    double al, be_, ga;
    law_values(law, c0, c1, c2, u, n2, &al, &be_, &ga);
    const double kd = kap * dV;
    const double ca = kd * al, cb = kd * be_, cg = kd * ga;
    if (!isfinite(ca) || !isfinite(cb) || !isfinite(cg)) raise_err(err, GFE_ERR_NONFINITE, cell);
    double f = 0.0;
    if (src_kind == GFE_SRC_CONST) f = __ldg(src);
    else if (src_kind == GFE_SRC_QPOINT) f = __ldg(src + cell * nq + q);
    const double fd = f * dV;
    double a[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < D; ++k) s += gu[k] * g[v][k];
      a[v] = s;
    }
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      be[i] += ca * a[i] - fd * phi[q * NV + i];
#pragma unroll
      for (int j = 0; j < NV; ++j) {
        double gg = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) gg += g[i][k] * g[j][k];
        Ke[i][j] += ca * gg + cb * a[i] * phi[q * NV + j] + cg * a[i] * a[j];
      }
    }
  }
  if (K)
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
      for (int j = 0; j < NV; ++j) K[(int64_t)(i + j * NV) * ncells + cell] = Ke[i][j];
  if (bvec)
#pragma unroll
    for (int i = 0; i < NV; ++i) bvec[(int64_t)i * ncells + cell] = be[i];
}

// Uniform Cartesian Q1 cells: the physical gradients g, their products G[q][i][j] = g_i.g_j
// and dV are the same in every cell (host tables), so a cell costs the state-dependent part
// only. SYM (no d alpha/d u term): the Jacobian is symmetric and only j >= i is formed.
template <int D, bool SYM>
__global__ void __launch_bounds__(128)
    k_quasilinear_q1_cart(int64_t ncells, const int32_t* __restrict__ cell_ids,
                          const double* __restrict__ state, int64_t nfree,
                          const double* __restrict__ uD, int64_t ndiri,
                          const double* __restrict__ tabs, int nq, int coef_kind,
                          const double* __restrict__ coef, int src_kind,
                          const double* __restrict__ src, int law, double c0, double c1,
                          double c2, double* __restrict__ K, double* __restrict__ bvec,
                          DevError* err) {
  constexpr int NV = 1 << D;
  extern __shared__ double st[];  // dV[nq] | phi[nq*NV] | g[nq*NV*D] | G[nq*NV*NV]
  const int ntab = nq * (1 + NV + NV * D + NV * NV);
  for (int i = threadIdx.x; i < ntab; i += blockDim.x) st[i] = tabs[i];
  __syncthreads();
  const double* dVq = st;
  const double* phi = dVq + nq;
  const double* gt = phi + nq * NV;
  const double* GG = gt + nq * NV * D;
  const int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncells) return;
  double uc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const int32_t id = __ldg(cell_ids + cell * NV + v);
    double u = 0.0;
    if (id > 0 && id <= nfree) {
      u = __ldg(state + id - 1);
    } else if (id < 0 && -(int64_t)id <= ndiri) {
      u = __ldg(uD - (int64_t)id - 1);
    } else if (id != 0 && !(id < 0 && ndiri == 0)) {
      raise_err(err, GFE_ERR_INVALID_ARGUMENT, cell);
    }
    uc[v] = u;
  }
  const double kap = coef_kind == GFE_COEF_CELL ? __ldg(coef + cell)
                     : coef_kind == GFE_COEF_CONST ? __ldg(coef) : 1.0;
  double Ke[NV][NV], be[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    be[i] = 0.0;
#pragma unroll
    for (int j = 0; j < NV; ++j) Ke[i][j] = 0.0;
  }
  for (int q = 0; q < nq; ++q) {
    double u = 0.0, gu[D];
#pragma unroll
    for (int k = 0; k < D; ++k) gu[k] = 0.0;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      u += phi[q * NV + v] * uc[v];
#pragma unroll
      for (int k = 0; k < D; ++k) gu[k] += gt[(q * NV + v) * D + k] * uc[v];
    }
    double n2 = 0.0;
#pragma unroll
    for (int k = 0; k < D; ++k) n2 += gu[k] * gu[k];
    double al, be_, ga;
    law_values(law, c0, c1, c2, u, n2, &al, &be_, &ga);
    const double kd = kap * dVq[q];
    const double ca = kd * al, cb = kd * be_, cg = kd * ga;
    if (!isfinite(ca) || !isfinite(cb) || !isfinite(cg)) raise_err(err, GFE_ERR_NONFINITE, cell);
    double f = 0.0;
    if (src_kind == GFE_SRC_CONST) f = __ldg(src);
    else if (src_kind == GFE_SRC_QPOINT) f = __ldg(src + cell * nq + q);
    const double fd = f * dVq[q];
    double a[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < D; ++k) s += gu[k] * gt[(q * NV + v) * D + k];
      a[v] = s;
    }
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      be[i] += ca * a[i] - fd * phi[q * NV + i];
      if (K) {
        const double cga = cg * a[i];
#pragma unroll
        for (int j = SYM ? i : 0; j < NV; ++j) {
          double t = ca * GG[(q * NV + i) * NV + j] + cga * a[j];
          if (!SYM) t += cb * a[i] * phi[q * NV + j];
          Ke[i][j] += t;
        }
      }
    }
  }
  if (K)
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
      for (int j = 0; j < NV; ++j)
        K[(int64_t)(i + j * NV) * ncells + cell] = (SYM && j < i) ? Ke[j][i] : Ke[i][j];
  if (bvec)
#pragma unroll
    for (int i = 0; i < NV; ++i) bvec[(int64_t)i * ncells + cell] = be[i];
}

template <int D>
int launch_quasilinear_cart(gfe_ctx* ctx, const gfe_problem* p, int64_t ncells,
                            const int32_t* ids, const double* st, int64_t nfree,
                            const double* uD, int64_t ndiri, const std::vector<double>& qw,
                            const std::vector<double>& phi1, const std::vector<double>& dphi1,
                            const double* coef, const double* src, double* K, double* bv) {
  constexpr int NV = 1 << D;
  const int nq = (int)qw.size();
  double h[3], vol = 1.0;
  for (int d = 0; d < D; ++d) {
    h[d] = (p->domain[2 * d + 1] - p->domain[2 * d]) / (double)p->partition[d];
    vol *= h[d];
  }
  std::vector<double> t;
  for (int q = 0; q < nq; ++q) t.push_back(qw[q] * vol);
  t.insert(t.end(), phi1.begin(), phi1.end());
  std::vector<double> g((size_t)nq * NV * D);
  for (int q = 0; q < nq; ++q)
    for (int v = 0; v < NV; ++v)
      for (int k = 0; k < D; ++k)
        g[((size_t)q * NV + v) * D + k] = dphi1[((size_t)q * NV + v) * D + k] / h[k];
  t.insert(t.end(), g.begin(), g.end());
  for (int q = 0; q < nq; ++q)
    for (int i = 0; i < NV; ++i)
      for (int j = 0; j < NV; ++j) {
        double s = 0.0;
        for (int k = 0; k < D; ++k)
          s += g[((size_t)q * NV + i) * D + k] * g[((size_t)q * NV + j) * D + k];
        t.push_back(s);
      }
  GFE_TRY(ctx->scratch[SCR_TMP0].reserve(sizeof(double) * t.size()));
  double* dt = ctx->scratch[SCR_TMP0].as<double>();
  GFE_CUDA_TRY(cudaMemcpyAsync(dt, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice,
                               ctx->stream));
  const size_t sm = sizeof(double) * t.size();
  const bool sym =
      p->law == GFE_LAW_POWER || (p->law_params[1] == 0.0 && p->law_params[2] == 0.0);
  auto kern = sym ? k_quasilinear_q1_cart<D, true> : k_quasilinear_q1_cart<D, false>;
  if (sm > 48 * 1024)
    GFE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  timer_begin(ctx, GFE_KT_ELEMENT);
  kern<<<grid_for(ncells, 128), 128, sm, ctx->stream>>>(
      ncells, ids, st, nfree, uD, ndiri, dt, nq, p->coef_kind, coef, p->source_kind, src, p->law,
      p->law_params[0], p->law_params[1], p->law_params[2], K, bv, ctx->d_err);
  timer_end(ctx);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  // the host table must outlive its copy
  GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GFE_OK;
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
  if (NN == NV) {  // Q1: thread per cell, tables only in shared memory
    const size_t smq = sizeof(double) * (size_t)nq * (1 + NV + NV * D);
    auto kq = k_quasilinear_q1<D>;
    if (smq > 48 * 1024)
      GFE_CUDA_TRY(cudaFuncSetAttribute(kq, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smq));
    timer_begin(ctx, GFE_KT_ELEMENT);
    kq<<<grid_for(ncells, 128), 128, smq, ctx->stream>>>(
        ncells, vn, vc, ids, st, nfree, uD, ndiri, tabs, nq, coef_kind, coef, src_kind, src,
        p->law, p->law_params[0], p->law_params[1], p->law_params[2], K, bv, ctx->d_err);
    timer_end(ctx);
    ctx->launches++;
    GFE_CUDA_TRY(cudaGetLastError());
    return GFE_OK;
  }
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
  if (A && (A->ncells != p->ncells || A->nd != p->nd ||
            A->cols_per_cell() != p->nd))
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
  if (!q2 && p->geometry == GFE_GEOM_CARTESIAN) {
    if (D == 2)
      GFE_TRY(launch_quasilinear_cart<2>(ctx, p, ncells, ids, st, p->nfree, ud, ndiri, qw, phi1,
                                         dphi1, kc, fs, K, bv));
    else
      GFE_TRY(launch_quasilinear_cart<3>(ctx, p, ncells, ids, st, p->nfree, ud, ndiri, qw, phi1,
                                         dphi1, kc, fs, K, bv));
  } else if (D == 2 && !q2)
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
  GFE_TRY(ensure_row_refs(ctx, R));
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
