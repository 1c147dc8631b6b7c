// gfe_assemble_lattice.cu -- the numeric assembly of uniform Cartesian Q1 diffusion in 3-D
// (kappa per cell or constant, source per node or constant) into the closed-form lattice
// pattern: the rows are the interior nodes in node order and each row's columns are its
// interior neighbours among the 27 around it, in (dz, dy, dx) order.
//
// On a uniform grid every cell has the same reference stiffness Kref, and Kref[a, b] depends
// only on the set of axes along which local vertices a and b differ (8 classes; the Q1
// stiffness is a sum of tensor products of 1-D matrices [[p, q], [q, p]]). The entry of row r
// and its neighbour r + d therefore is
//     A[r, r + d] = W[class(d)] * S(d),   S(d) = sum of kappa over the cells r and r + d share,
// the cells being a box of 1 or 2 cells per axis (1 along each axis where d is nonzero). This
// equals Gridap's cell-ordered sum of kappa_K Kref[l_r, l_c] (FESpaces/SparseMatrixAssemblers.jl:
// 214-248 with the cell matrices of CellData/CellQuadratures.jl:138-170) up to rounding: the
// parity bar for fused values is 1e-12 of the row maximum. The load vector of a nodal source
// f is the mass matrix applied to f, and the Q1 mass matrix of a uniform grid is separable:
//     b_r = hx hy hz / 216 * sum_d prod_axes w(d_axis) f_{r + d},  w(0) = 4, w(+-1) = 1.
//
// Work per row in FP64 (the pipe that bounds this kernel on GB300, 1/64 of the FP32 rate):
// a thread marches up one (i, j) column of nodes; each step loads the next cell layer's four
// kappa, forms its five partial sums (x-pairs, y-pairs, quad), combines them with the layer
// below (9 sums), and multiplies 18 entries (the 9 entries towards the layer below are the
// products formed one step earlier for the layer above); the load vector takes 11 operations
// (x-, y- and z-passes of the separable stencil). 43 FP64 operations per row against 128 in the
// generic row gather; 34 on cubic cells, whose face classes carry no weight (their entries are
// stored as zeros without forming the sums). Both rows of a symmetric pair form the same sums in the same order, so the
// matrix is exactly symmetric.
//
// Stores: a warp holds 32 consecutive rows (one x-line), whose CSR slice is contiguous; the
// lanes write their entries into a shared-memory stage at their row offsets and the warp then
// copies the slice out with coalesced stores.
#include "gfe_internal.h"

namespace gfe {
namespace {

constexpr int kCqKZ = 8;             // node planes per block (marching depth)
constexpr int kCqStage = 32 * 27;    // stage doubles per warp
constexpr int kCqBlock = 256;        // 32 x 8 columns

struct CartQ1Lattice {
  int n0, n1, n2;  // cells per direction
  int m0, m1, m2;  // interior nodes per direction (= rows per direction)
  const int32_t* rowptr;
  double* val;      // null: vector only
  double* b;        // null: matrix only
  const double* kap;  // per cell (Gridap cell order), or null for kconst
  double kconst;
  int src_kind;       // GFE_SRC_NONE / CONST / NODAL
  const double* f;    // nodal values ((n0+1)(n1+1)(n2+1), node order) for NODAL
  double fscale;      // NODAL: hx hy hz / 216; CONST: f hx hy hz (the whole row value)
  double W[8];        // Kref[0, c] for the axis set c (bit 0 x, bit 1 y, bit 2 z)
};

// kappa sums of one cell layer around a node column: the four cells (i + cx, j + cy) and
// the boxes of the 9 (dx, dy) offsets, indexed e = (dx + 1) + 3 (dy + 1)
struct LayerSums {
  double s00, s10, s01, s11, X0, X1, Y0, Y1, Q;
  __device__ __forceinline__ double box(int e) const {
    switch (e) {
      case 0: return s00;
      case 1: return X0;
      case 2: return s10;
      case 3: return Y0;
      case 4: return Q;
      case 5: return Y1;
      case 6: return s01;
      case 7: return X1;
      default: return s11;
    }
  }
};

// ZF: the face classes 1, 2 and 4 (vertices differing along one axis) carry no weight, as
// on cubic cells; their entries are stored as zeros without forming S (21 % of the FP64
// operations per row).
template <bool ZF>
__global__ void __launch_bounds__(kCqBlock) k_assemble_cart_q1(const CartQ1Lattice a) {
  extern __shared__ double stage_all[];
  const int lane = (int)(threadIdx.x & 31), warp = (int)(threadIdx.x >> 5);
  double* stage = stage_all + warp * kCqStage;
  const int i = (int)blockIdx.x * 32 + lane, j = (int)blockIdx.y * 8 + warp;
  const int k0 = (int)blockIdx.z * kCqKZ;
  if (j >= a.m1) return;  // the whole warp
  const bool act = i < a.m0;
  const int ic = act ? i : a.m0 - 1;  // lanes past the line compute on a clamped column, store nothing
  const int64_t sy = a.n0, sz = (int64_t)a.n0 * a.n1;
  auto kap = [&](int cx, int cy, int kk) -> double {
    if (!a.kap) return a.kconst;
    return __ldg(a.kap + (int64_t)(ic + cx) + sy * (j + cy) + sz * kk);
  };
  auto layer = [&](int kk, LayerSums& L) {
    L.s00 = kap(0, 0, kk);
    L.s10 = kap(1, 0, kk);
    L.s01 = kap(0, 1, kk);
    L.s11 = kap(1, 1, kk);
    L.X0 = L.s00 + L.s10;
    L.X1 = L.s01 + L.s11;
    L.Y0 = L.s00 + L.s01;
    L.Y1 = L.s10 + L.s11;
    L.Q = L.X0 + L.X1;
  };
  // y- and x-passes of the mass stencil on node plane Kp: nodes (ic .. ic+2, j .. j+2, Kp)
  const int64_t fy = a.n0 + 1, fz = (int64_t)(a.n0 + 1) * (a.n1 + 1);
  auto uplane = [&](int Kp) -> double {
    const double* fp = a.f + fz * Kp + fy * j + ic;
    double t[3];
#pragma unroll
    for (int dy = 0; dy < 3; ++dy) {
      const double* q = fp + fy * dy;
      t[dy] = fma(4.0, __ldg(q + 1), __ldg(q) + __ldg(q + 2));
    }
    return fma(4.0, t[1], t[0] + t[2]);
  };
  const bool nodal = a.src_kind == GFE_SRC_NODAL && a.b;
  const bool xm = i > 0, xp = i < a.m0 - 1, ym = j > 0, yp = j < a.m1 - 1;

  LayerSums lo, up;
  layer(k0, lo);
  double carry[9];  // dz = -1 entries: W[class | z] * box of the layer below
  // the entry of class cls from box sum S: W[cls] * S, or 0 for a weightless class
  auto entry = [&](int cls, double S) -> double {
    if (ZF && (cls == 1 || cls == 2 || cls == 4)) return 0.0;
    return a.W[cls] * S;
  };
#pragma unroll
  for (int e = 0; e < 9; ++e) {
    const int cls = (e % 3 != 1 ? 1 : 0) | (e / 3 != 1 ? 2 : 0) | 4;
    carry[e] = entry(cls, lo.box(e));
  }
  double u0 = 0.0, u1 = 0.0;
  if (nodal) {
    u0 = uplane(k0);
    u1 = uplane(k0 + 1);
  }
  for (int t = 0; t < kCqKZ; ++t) {
    const int k = k0 + t;
    if (k >= a.m2) break;  // uniform over the block
    const int64_t r = (int64_t)ic + (int64_t)a.m0 * (j + (int64_t)a.m1 * k);
    layer(k + 1, up);
    if (a.val) {
      int32_t rp = 0, rpn = 0;
      if (act) {
        rp = __ldg(a.rowptr + r);
        rpn = __ldg(a.rowptr + r + 1);
      }
      const int32_t rp0 = __shfl_sync(0xffffffffu, rp, 0);
      int32_t rend = rpn;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) rend = max(rend, __shfl_xor_sync(0xffffffffu, rend, off));
      const bool zm = k > 0, zp = k < a.m2 - 1;
      int pos = rp - rp0;
      auto put = [&](bool ok, double v) {
        if (act && ok) stage[pos++] = v;
      };
#pragma unroll
      for (int e = 0; e < 9; ++e) {  // dz = -1
        const int dx = e % 3 - 1, dy = e / 3 - 1;
        const bool okxy = (dx < 0 ? xm : dx > 0 ? xp : true) && (dy < 0 ? ym : dy > 0 ? yp : true);
        put(zm && okxy, carry[e]);
      }
#pragma unroll
      for (int e = 0; e < 9; ++e) {  // dz = 0: both layers
        const int dx = e % 3 - 1, dy = e / 3 - 1;
        const bool okxy = (dx < 0 ? xm : dx > 0 ? xp : true) && (dy < 0 ? ym : dy > 0 ? yp : true);
        const int cls = (dx ? 1 : 0) | (dy ? 2 : 0);
        put(okxy, ZF && (cls == 1 || cls == 2) ? 0.0 : a.W[cls] * (lo.box(e) + up.box(e)));
      }
#pragma unroll
      for (int e = 0; e < 9; ++e) {  // dz = +1: the layer above; kept for the next plane
        const int dx = e % 3 - 1, dy = e / 3 - 1;
        const bool okxy = (dx < 0 ? xm : dx > 0 ? xp : true) && (dy < 0 ? ym : dy > 0 ? yp : true);
        const int cls = (dx ? 1 : 0) | (dy ? 2 : 0) | 4;
        const double v = entry(cls, up.box(e));
        carry[e] = v;
        put(zp && okxy, v);
      }
      __syncwarp();
      for (int q = lane; q < rend - rp0; q += 32) a.val[rp0 + q] = stage[q];
      __syncwarp();
    } else {
#pragma unroll
      for (int e = 0; e < 9; ++e) {
        const int cls = (e % 3 != 1 ? 1 : 0) | (e / 3 != 1 ? 2 : 0) | 4;
        carry[e] = entry(cls, up.box(e));
      }
    }
    if (a.b) {
      double bv = 0.0;
      if (nodal) {
        const double u2 = uplane(k + 2);
        bv = a.fscale * fma(4.0, u1, u0 + u2);
        u0 = u1;
        u1 = u2;
      } else if (a.src_kind == GFE_SRC_CONST) {
        bv = a.fscale;
      }
      if (act) a.b[r] = bv;
    }
    lo = up;
  }
}

}  // namespace

// The fused numeric assembly above, when the matrix carries the closed-form lattice pattern of
// this problem's grid and the form is one the kernel covers; *done tells the caller.
int assemble_cartesian_q1_lattice(gfe_ctx* ctx, gfe_matrix* A, const gfe_problem* p,
                                  const double* d_coef, int src_kind, const double* d_src,
                                  const double* Kref, const double* mref, double* d_b,
                                  bool* done) {
  *done = false;
  if (!A || p->dim != 3 || p->reffe != GFE_REFFE_Q1 || p->geometry != GFE_GEOM_CARTESIAN ||
      p->precision != GFE_PREC_FP64 || ctx->lift_uD)
    return GFE_OK;
  if (!A->cart_lattice && !A->cart_checked) {
    // a pattern from the general symbolic loop over the interior-node numbering is the
    // closed form too: recognise it once, so that every assembly of the same ids takes this
    // kernel and re-assembly reproduces a fresh assembly bit for bit
    A->cart_checked = true;
    bool ok = false;
    GFE_TRY(cartesian_ids_match(ctx, A, p->partition[0], p->partition[1], p->partition[2], &ok));
    if (ok) {
      A->cart_lattice = true;
      for (int d = 0; d < 3; ++d) A->cart_n[d] = p->partition[d];
    }
  }
  if (!A->cart_lattice || A->cart_n[0] != p->partition[0] || A->cart_n[1] != p->partition[1] ||
      A->cart_n[2] != p->partition[2])
    return GFE_OK;
  if (src_kind != GFE_SRC_NONE && src_kind != GFE_SRC_CONST && src_kind != GFE_SRC_NODAL)
    return GFE_OK;
  if (src_kind == GFE_SRC_NODAL && (p->cell_node_ids || !d_src)) return GFE_OK;
  if (p->coef_kind == GFE_COEF_CELL && !d_coef) return GFE_OK;
  CartQ1Lattice a{};
  a.n0 = (int)p->partition[0];
  a.n1 = (int)p->partition[1];
  a.n2 = (int)p->partition[2];
  a.m0 = a.n0 - 1;
  a.m1 = a.n1 - 1;
  a.m2 = a.n2 - 1;
  a.rowptr = A->rowptr.as<int32_t>();
  a.val = A->val.as<double>();
  a.b = d_b;
  a.kap = p->coef_kind == GFE_COEF_CELL ? d_coef : nullptr;
  if (p->coef_kind == GFE_COEF_CONST) {
    if (!p->coef) return GFE_OK;
    double kc = 0.0;
    GFE_TRY(copy_out(ctx, &kc, d_coef, sizeof(double)));
    a.kconst = kc;
  } else {
    a.kconst = 1.0;
  }
  a.src_kind = d_b ? src_kind : GFE_SRC_NONE;
  double h[3];
  for (int d = 0; d < 3; ++d) h[d] = (p->domain[2 * d + 1] - p->domain[2 * d]) / (double)p->partition[d];
  if (src_kind == GFE_SRC_NODAL) {
    a.f = d_src;
    a.fscale = h[0] * h[1] * h[2] / 216.0;
  } else if (src_kind == GFE_SRC_CONST) {
    double fc = 0.0;
    GFE_TRY(copy_out(ctx, &fc, d_src, sizeof(double)));
    double m = 0.0;  // sum over the 8 cells of the node's shape-function integral
    for (int c = 0; c < 8; ++c) m += mref[c];
    a.fscale = fc * m;
  }
  double wmax = 0.0;
  for (int c = 0; c < 8; ++c) {
    a.W[c] = Kref[0 + 8 * c];
    wmax = std::max(wmax, std::fabs(a.W[c]));
  }
  // cubic cells: the face-class weights vanish up to the rounding of the reference integral
  // (|W| below 1e-13 of the largest weight), and their entries are stored as exact zeros
  const bool zf = std::fabs(a.W[1]) <= 1e-13 * wmax && std::fabs(a.W[2]) <= 1e-13 * wmax &&
                  std::fabs(a.W[4]) <= 1e-13 * wmax;
  auto kern = zf ? k_assemble_cart_q1<true> : k_assemble_cart_q1<false>;
  const size_t smem = sizeof(double) * kCqStage * (kCqBlock / 32);
  GFE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const dim3 grid((unsigned)((a.m0 + 31) / 32), (unsigned)((a.m1 + 7) / 8),
                  (unsigned)((a.m2 + kCqKZ - 1) / kCqKZ));
  timer_begin(ctx, GFE_KT_ASSEMBLE);
  kern<<<grid, kCqBlock, smem, ctx->stream>>>(a);
  timer_end(ctx);
  A->zf_values = zf;
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  *done = true;
  return GFE_OK;
}

}  // namespace gfe
