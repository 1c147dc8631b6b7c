// gfe_mg.cu -- geometric multigrid V-cycle on the lattice operator, a preconditioner for the
// flexible CG (gfe_solve_fcg with GFE_PC_MG). Gridap has no multigrid; this is the GPU
// counterpart of a LinearSolver plug-in preconditioner for the uniform Cartesian Q1 problems
// the lattice operator covers.
//
// Levels halve the cell counts while they stay even (at least 4 cells per direction). Each
// level is again a lattice operator: kappa of a coarse cell is the mean of its 8 children and
// the reference stiffness doubles (a Q1 stiffness on a box of sizes 2h is twice the one on h,
// in 3-D), which for piecewise-constant kappa equals the Galerkin product P^T A P of the
// nested Q1 spaces. Transfers are trilinear interpolation P and its transpose R = P^T (full
// weighting 1, 1/2, 1/4, 1/8). Smoothing is Chebyshev-paired damped Jacobi (two sweeps before and
// after, the first from zero), each later sweep fused into one pass over the lattice stencil;
// the coarsest level takes five sweeps. Levels of at most 512 rows run their part of the
// cycle in one block, out of shared memory. All vectors are FP32 in the lattice row order;
// every kernel returns at once when the solver's done flag is set. The cycle's kernels are
// chained by programmatic dependent launch; the solver records them into its own loop graph,
// or replays the cycle as a graph captured once.
#include <utility>
#include <vector>

#include "gfe_internal.h"

namespace gfe {
#include "gfe_lattice.cuh"
#include "gfe_reduce.cuh"
#include "gfe_pdl.cuh"

namespace {

constexpr int kMgBlock = 256;
// Smoothing runs in pairs of damped Jacobi sweeps whose factors are the reciprocals of the
// roots of the degree-2 Chebyshev polynomial on [kChebLo B, kChebHi B]: the pair's error
// polynomial (1 - w1 l)(1 - w2 l) is the minimax one of degree 2 on that interval. B bounds the
// spectrum of D^-1 A for every kappa >= 0: x^T A x = sum_K kappa_K x_K^T Kref x_K <=
// lmax(Kref) sum_K kappa_K |x_K|^2 = (lmax(Kref) / Kref_00) x^T D x, so B = lmax(Kref) / Kref_00,
// 1.5 on cubes (the high-frequency modes of the constant-coefficient stencil span 0.5 .. 1.5)
// and larger on elongated boxes; on [0, B] the pair's factor is at most 1 in magnitude.
// Every level shares B (coarsening halves every axis and doubles Kref). On the 128^3
// lognormal problem the flexible CG needs 7 iterations with these pairs against 8 with damped
// Jacobi (omega 0.8 or 1).
constexpr float kChebLo = 0.4f / 1.5f, kChebHi = 1.6f / 1.5f;

// the two factors of the pair for the spectral bound B
struct SweepPair {
  float w1, w2;
  __host__ __device__ float at(int s) const { return (s & 1) ? w2 : w1; }  // sweep s (0 first)
};
SweepPair sweep_pair(double B) {
  const double lo = kChebLo * B, hi = kChebHi * B;
  const double th = 0.5 * (hi + lo), de = 0.5 * (hi - lo) * 0.70710678118654752;
  return SweepPair{(float)(1.0 / (th + de)), (float)(1.0 / (th - de))};
}

// B = lmax(Kref) / Kref_00 of a box Q1 stiffness (Kref[li + 8 lj]): its eigenvectors are the
// 8 tensor-product sign patterns over the vertices
double stiffness_spectral_bound(const float* K) {
  double best = 0.0;
  for (int s = 0; s < 8; ++s) {
    double v[8], q = 0.0;
    for (int a = 0; a < 8; ++a) {
      v[a] = 1.0;
      for (int d = 0; d < 3; ++d)
        if (((s >> d) & 1) && ((a >> d) & 1)) v[a] = -v[a];
    }
    for (int a = 0; a < 8; ++a)
      for (int b = 0; b < 8; ++b) q += v[a] * (double)K[a + 8 * b] * v[b];
    best = std::max(best, q / 8.0);
  }
  return K[0] > 0.f ? best / (double)K[0] : 2.0;
}
constexpr int kPreSweeps = 2, kPostSweeps = 2, kCoarseSweeps = 4;
// On deep lattices (the march of kLatK planes per thread) the first sweep from zero runs as a
// pass of its own followed by a plain sweep: the fused pass, which forms omega D^-1 b at every
// neighbour, loads twice the vectors per row and measured slower there.
constexpr bool kFusePreDeep = false;

// Every kernel of the cycle is launched with programmatic stream serialisation (launch_pdl)
// and waits in stop() for the kernel before it; each returns at once when the solver's done
// flag is set.
__device__ __forceinline__ bool stop(const int* done) {
  pdl_wait();
  return done && *done;
}

// One damped Jacobi sweep fused into the lattice apply: xo = x + w D^-1 (b - A x)
// (xo != x: the sweep reads the old neighbours). Same arithmetic as an apply into t followed
// by the update x += omega D^-1 (b - t).
template <int KZ>
__global__ void __launch_bounds__(kMgBlock)
    k_mg_smooth(LatticeQ1Op op, const float* __restrict__ x, const float* __restrict__ b,
                const float* __restrict__ dinv, float* __restrict__ xo, float w,
                const int* done) {
  if (stop(done)) return;
  auto epi = [&](int64_t row, float xc, float acc) {
    xo[row] = fmaf(w * __ldg(dinv + row), __ldg(b + row) - acc, xc);
  };
  lattice_rows<false, decltype(epi), KZ>(op, (int)blockIdx.x, (int)blockIdx.y,
                                         (int)blockIdx.z, x, epi);
}

// The cycle's last sweep, with the dot product the caller asked for: xo as k_mg_smooth, and
// *d.out = -(xo . d.v) / *d.den (0 when *d.den is 0), FP32 per thread and FP64 across the
// block's warps, the block partials added in block order by the last block.
template <int KZ>
__global__ void __launch_bounds__(kMgBlock)
    k_mg_smooth_dot(LatticeQ1Op op, const float* __restrict__ x, const float* __restrict__ b,
                    const float* __restrict__ dinv, float* __restrict__ xo, float w,
                    const int* done, MgDot d) {
  __shared__ double sh[kMgBlock / 32];
  if (stop(done)) return;
  float s = 0.f;
  auto epi = [&](int64_t row, float xc, float acc) {
    const float v = fmaf(w * __ldg(dinv + row), __ldg(b + row) - acc, xc);
    xo[row] = v;
    s = fmaf(v, __ldg(d.v + row), s);
  };
  lattice_rows<false, decltype(epi), KZ>(op, (int)blockIdx.x, (int)blockIdx.y,
                                         (int)blockIdx.z, x, epi);
  const double bs = block_sum_f<kMgBlock>(s, sh);
  if (threadIdx.x == 0) d.partials[block_linear()] = bs;
  double tot[1];
  if (last_block_reduce<kMgBlock, 1>(d.ticket, d.partials, (int)grid_blocks(), tot, sh) &&
      threadIdx.x == 0) {
    const double den = *d.den;
    *d.out = den != 0.0 ? -tot[0] / den : 0.0;
  }
}

// The first two sweeps in one pass: x0 = w0 D^-1 b (the sweep from zero, formed on the fly at
// the neighbours) and xo = x0 + w1 D^-1 (b - A x0). x0 itself is not stored: the cycle reads
// only xo afterwards.
template <int KZ>
__global__ void __launch_bounds__(kMgBlock)
    k_mg_pre(LatticeQ1Op op, const float* __restrict__ b, const float* __restrict__ dinv,
             float* __restrict__ xo, float w0, float w1, const int* done) {
  if (stop(done)) return;
  const LatticeLoadJacobi0 x0{b, dinv, w0};
  auto epi = [&](int64_t row, float xc, float acc) {
    xo[row] = fmaf(w1 * __ldg(dinv + row), __ldg(b + row) - acc, xc);
  };
  lattice_rows_f<false, decltype(epi), KZ>(op, (int)blockIdx.x, (int)blockIdx.y,
                                           (int)blockIdx.z, x0, epi);
}

// r = b - A x (the residual the restriction takes to the coarse level)
template <int KZ>
__global__ void __launch_bounds__(kMgBlock)
    k_mg_residual(LatticeQ1Op op, const float* __restrict__ x, const float* __restrict__ b,
                  float* __restrict__ r, const int* done) {
  if (stop(done)) return;
  auto epi = [&](int64_t row, float, float acc) { r[row] = __ldg(b + row) - acc; };
  lattice_rows<false, decltype(epi), KZ>(op, (int)blockIdx.x, (int)blockIdx.y,
                                         (int)blockIdx.z, x, epi);
}

// x = w D^-1 b  (first sweep from zero)
__global__ void k_mg_jacobi0(int64_t n, const float* __restrict__ b,
                             const float* __restrict__ dinv, float* __restrict__ x, float w,
                             const int* done) {
  if (stop(done)) return;
  for (int64_t i = (int64_t)blockIdx.x * kMgBlock + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kMgBlock)
    x[i] = w * dinv[i] * b[i];
}

// b_c = R r_f: coarse interior node (I, J, K) sits on fine interior node (2I+1, 2J+1, 2K+1);
// weights prod_d (1 - |delta_d| / 2) over its 27 fine neighbours, all interior (m_f = 2 m_c +
// 1). A block covers a 32 x 8 tile of coarse (I, J) and KZ coarse planes; each thread marches
// up its column, the weighted 3 x 3 sum of the fine plane between two coarse planes formed
// once for both.
template <int KZ>
__global__ void __launch_bounds__(kMgBlock)
    k_mg_restrict(int mf0, int mf1, int mc0, int mc1, int mc2, const float* __restrict__ rf,
                  float* __restrict__ bc, const int* done) {
  if (stop(done)) return;
  const int I = (int)blockIdx.x * 32 + (int)(threadIdx.x & 31);
  const int J = (int)blockIdx.y * 8 + (int)(threadIdx.x >> 5);
  if (I >= mc0 || J >= mc1) return;
  const int K0 = (int)blockIdx.z * KZ;
  const int64_t fs2 = (int64_t)mf0 * mf1;
  const float* col = rf + (2 * I + 1) + (int64_t)mf0 * (2 * J + 1);  // fine (2I+1, 2J+1, 0)
  auto plane = [&](int kz) {
    const float* q = col + fs2 * kz;
    const float r0 = fmaf(0.5f, q[-mf0 - 1] + q[-mf0 + 1], q[-mf0]);
    const float r1 = fmaf(0.5f, q[-1] + q[1], q[0]);
    const float r2 = fmaf(0.5f, q[mf0 - 1] + q[mf0 + 1], q[mf0]);
    return fmaf(0.5f, r0 + r2, r1);
  };
  float lo = plane(2 * K0);
#pragma unroll
  for (int t = 0; t < KZ; ++t) {
    const int K = K0 + t;
    if (K >= mc2) break;
    const float mid = plane(2 * K + 1), hi = plane(2 * K + 2);
    bc[I + (int64_t)mc0 * (J + (int64_t)mc1 * K)] = fmaf(0.5f, lo + hi, mid);
    lo = hi;
  }
}

// xo = x_f + P x_c at the fine interior nodes: per axis, an even lattice position 2Q takes
// coarse position Q, an odd one the mean of Q and Q + 1 (coarse boundary positions 0 and
// m_c + 1 hold zero). A block covers a 32 x 8 tile of fine (i, j) and KZ fine planes; each
// thread forms the (x, y)-interpolated value of a coarse plane once and marches up its column.
// xo may be xf: each thread reads and writes its own rows only.
template <int KZ>
__global__ void __launch_bounds__(kMgBlock)
    k_mg_prolong(int mf0, int mf1, int mf2, int mc0, int mc1, int mc2,
                 const float* __restrict__ xc, const float* xf, float* xo, const int* done) {
  if (stop(done)) return;
  const int i = (int)blockIdx.x * 32 + (int)(threadIdx.x & 31);
  const int j = (int)blockIdx.y * 8 + (int)(threadIdx.x >> 5);
  if (i >= mf0 || j >= mf1) return;
  // the two coarse interior indices along an axis and their weights (lattice position p);
  // indices out of range are clamped and weighted 0
  auto axis = [](int p, int mc, int& a0, int& a1, float& w0, float& w1) {
    a0 = p / 2 - 1;
    a1 = p / 2;
    w0 = (p & 1) ? 0.5f : 1.f;
    w1 = (p & 1) ? 0.5f : 0.f;
    if (a0 < 0) {
      a0 = 0;
      w0 = 0.f;
    }
    if (a1 >= mc) {
      a1 = mc - 1;
      w1 = 0.f;
    }
  };
  int ax0, ax1, ay0, ay1;
  float wx0, wx1, wy0, wy1;
  axis(i + 1, mc0, ax0, ax1, wx0, wx1);
  axis(j + 1, mc1, ay0, ay1, wy0, wy1);
  const int o00 = ax0 + mc0 * ay0, o10 = ax1 + mc0 * ay0;
  const int o01 = ax0 + mc0 * ay1, o11 = ax1 + mc0 * ay1;
  const int64_t cs2 = (int64_t)mc0 * mc1;
  auto cplane = [&](int q) -> float {  // coarse lattice plane q (interior: 1 .. mc2)
    if (q < 1 || q > mc2) return 0.f;
    const float* c = xc + cs2 * (q - 1);
    return fmaf(wy1, fmaf(wx1, c[o11], wx0 * c[o01]), wy0 * fmaf(wx1, c[o10], wx0 * c[o00]));
  };
  const int k0 = (int)blockIdx.z * KZ;
  int q = (k0 + 1) >> 1;  // the coarse plane at or below fine lattice position k + 1
  float vlo = cplane(q), vhi = cplane(q + 1);
  const int64_t base = i + (int64_t)mf0 * j, fs2 = (int64_t)mf0 * mf1;
#pragma unroll
  for (int t = 0; t < KZ; ++t) {
    const int k = k0 + t;
    if (k >= mf2) break;
    const int pz = k + 1;
    if ((pz >> 1) != q) {
      ++q;
      vlo = vhi;
      vhi = cplane(q + 1);
    }
    const float v = (pz & 1) ? 0.5f * (vlo + vhi) : vlo;
    const int64_t row = base + fs2 * k;
    xo[row] = xf[row] + v;
  }
}

// One level's refresh in one pass over its interior nodes (i, j, k) = (32 bx + lane, 8 by +
// warp, bz): D^-1 of the node, D = sum of kappa_K Kref[l, l] over the 8 cells around it, and
// at even (i, j, k) kappa of the coarse cell (i/2, j/2, k/2), the mean of its 8 children
// (kc null on the coarsest level; cc1, cc2 its row and plane strides). Each level's pass is
// launched after the one above with programmatic serialisation and waits for its kappa.
__global__ void __launch_bounds__(kMgBlock)
    k_mg_refresh(LatticeQ1Op op, float* __restrict__ dinv, float* __restrict__ kc, int cc1,
                 int64_t cc2) {
  if (stop(nullptr)) return;
  const int m0 = op.n0 - 1, m1 = op.n1 - 1;
  const int i = (int)blockIdx.x * 32 + (int)(threadIdx.x & 31);
  const int j = (int)blockIdx.y * 8 + (int)(threadIdx.x >> 5);
  const int k = (int)blockIdx.z;
  if (i >= m0 || j >= m1) return;
  const float* kap = op.kap + ((int64_t)i + (int64_t)op.c1 * j + (int64_t)op.c2 * k);
  float d = 0.f;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int cx = e & 1, cy = (e >> 1) & 1, cz = e >> 2;
    const int lr = (1 - cx) + 2 * (1 - cy) + 4 * (1 - cz);
    d += kap[cx + (int64_t)op.c1 * cy + (int64_t)op.c2 * cz] * op.K[lr + 8 * lr];
  }
  dinv[i + (int64_t)m0 * (j + (int64_t)m1 * k)] = d > 0.f ? 1.f / d : 0.f;
  if (kc && !((i | j | k) & 1)) {
    float s = 0.f;
#pragma unroll
    for (int e = 0; e < 8; ++e)
      s += kap[(e & 1) + (int64_t)op.c1 * ((e >> 1) & 1) + (int64_t)op.c2 * (e >> 2)];
    kc[(i >> 1) + (int64_t)cc1 * (j >> 1) + cc2 * (k >> 1)] = 0.125f * s;
  }
}

// ---- the coarse levels in one block ------------------------------------------------------
// Levels of at most kCoarseRows rows run their whole V-cycle inside one block of kCoarseBlock
// threads: on such lattices a launch costs more than its work. The block copies kappa and
// D^-1 of these levels and b of the first one into shared memory, runs every step there
// (a barrier between steps; x, b and t of every level live in shared memory only) and writes
// x of the first level back. x and t are held with a zero halo (so that no neighbour needs a
// bounds check); a thread takes a segment of `ks` rows up one (i, j) column and marches it
// with three x-planes and the kappa box sums of two cell layers in registers.
constexpr int64_t kCoarseRows = 512;
constexpr int kCoarseBlock = kCoarseRows > 512 ? 1024 : 512;
constexpr int kMaxCoarse = 6;

// one level of the block: float offsets of its arrays in the shared buffer
struct MgCoarseLevel {
  int m0, m1, m2, n;       // interior nodes per direction, rows
  int q0, q1;              // strides of the zero-halo layout of x and t: m0 + 2, q0 (m1 + 2)
  int c1, c2, ncell;       // kappa strides (as in LatticeQ1Op), kappa entries c2 * n2
  int ks, nseg;            // rows per column segment, segments per column
  int x, t, b, dinv, kap;  // offsets into the shared buffer (x, t: q1 (m2 + 2) entries)
  float W[8];              // class weights Kref[0][c]
  const float* gkap;       // kappa and D^-1 in global memory
  const float* gdinv;
};

struct CoarseLevels {
  int nl;
  SweepPair w;      // smoothing factors
  int floats;       // shared buffer size
  const float* b0;  // b of the first level
  float* x0;        // its result
  MgCoarseLevel L[kMaxCoarse];
};

// The rows of one phase on level L: every (column, segment) item; `epi(row, padded index, x
// at the row, (A x)_row)` receives each row of the item. x is a zero-halo vector in shared
// memory. (A x)_r in class-sum form as the lattice rows: sum_c W[c] sum_{d in c} S(d) x_{r+d},
// S(d) the kappa sum over the cells r and r + d share.
template <class Epi>
__device__ __forceinline__ void coarse_rows(const MgCoarseLevel& L, const float* sm,
                                            const float* x, Epi epi) {
  const float* kap = sm + L.kap;
  const int items = L.m0 * L.m1 * L.nseg;
  for (int it = (int)threadIdx.x; it < items; it += kCoarseBlock) {
    const int col = it / L.nseg, seg = it - col * L.nseg;
    const int j = col / L.m0, i = col - j * L.m0;
    const int k0 = seg * L.ks, k1 = min(k0 + L.ks, L.m2);
    // x at padded (i + 1 + dx, j + 1 + dy, kk + 1), dx, dy in -1 .. 1
    const float* xc = x + (i + 1) + L.q0 * (j + 1);
    auto xplane = [&](int kk, float* v) {
      const float* p = xc + L.q1 * (kk + 1);
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) v[(dx + 1) + 3 * (dy + 1)] = p[dx + L.q0 * dy];
    };
    // box sums of cell layer kk (cells (i + cx, j + cy, kk)), indexed (dx + 1) + 3 (dy + 1)
    const float* kc = kap + i + L.c1 * j;
    auto layer = [&](int kk, float* Lb) {
      const float* q = kc + L.c2 * kk;
      const float v0 = q[0], v1 = q[1], v2 = q[L.c1], v3 = q[L.c1 + 1];
      const float X0 = v0 + v1, X1 = v2 + v3;
      Lb[0] = v0;
      Lb[1] = X0;
      Lb[2] = v1;
      Lb[3] = v0 + v2;
      Lb[4] = X0 + X1;
      Lb[5] = v1 + v3;
      Lb[6] = v2;
      Lb[7] = X1;
      Lb[8] = v3;
    };
    float xa[9], xb[9], xn[9], la[9], lb[9];
    xplane(k0 - 1, xa);
    xplane(k0, xb);
    layer(k0, la);
    for (int k = k0; k < k1; ++k) {
      xplane(k + 1, xn);
      layer(k + 1, lb);
      float T[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) T[c] = 0.f;
#pragma unroll
      for (int e = 0; e < 9; ++e) {
        const int cl = (e % 3 != 1 ? 1 : 0) | (e / 3 != 1 ? 2 : 0);
        T[cl | 4] = fmaf(la[e], xa[e], T[cl | 4]);
        T[cl] = fmaf(la[e] + lb[e], xb[e], T[cl]);
        T[cl | 4] = fmaf(lb[e], xn[e], T[cl | 4]);
      }
      float acc = 0.f;
#pragma unroll
      for (int c = 0; c < 8; ++c) acc = fmaf(L.W[c], T[c], acc);
      epi(i + L.m0 * (j + L.m1 * k), (i + 1) + L.q0 * (j + 1) + L.q1 * (k + 1), xb[4], acc);
#pragma unroll
      for (int e = 0; e < 9; ++e) {
        xa[e] = xb[e];
        xb[e] = xn[e];
        la[e] = lb[e];
      }
    }
  }
}

// the V-cycle of levels 0 .. nl-1 of `c` (b of level 0 given, its result written to x0); the
// same steps, sweep counts and buffer roles as the multi-launch cycle
__global__ void __launch_bounds__(kCoarseBlock)
    k_mg_coarse(const __grid_constant__ CoarseLevels c, const int* done) {
  if (stop(done)) return;
  extern __shared__ float sm[];
  const int t0 = threadIdx.x;
  // zero-halo x and t (whole arrays), kappa, D^-1 and the first level's b
  for (int l = 0; l < c.nl; ++l) {
    const MgCoarseLevel& L = c.L[l];
    const int np = L.q1 * (L.m2 + 2);
    for (int e = t0; e < 2 * np; e += kCoarseBlock) sm[L.x + e] = 0.f;  // t follows x
    for (int e = t0; e < L.ncell; e += kCoarseBlock) sm[L.kap + e] = L.gkap[e];
    for (int r = t0; r < L.n; r += kCoarseBlock) sm[L.dinv + r] = L.gdinv[r];
  }
  for (int r = t0; r < c.L[0].n; r += kCoarseBlock) sm[c.L[0].b + r] = c.b0[r];
  __syncthreads();
  // the interior rows of level L: f(row, padded index)
  auto rows = [&](const MgCoarseLevel& L, auto f) {
    for (int r = t0; r < L.n; r += kCoarseBlock) {
      const int jk = r / L.m0, i = r - jk * L.m0;
      const int k = jk / L.m1, j = jk - k * L.m1;
      f(r, (i + 1) + L.q0 * (j + 1) + L.q1 * (k + 1), i, j, k);
    }
  };
  auto sweep = [&](const MgCoarseLevel& L, int xi, int xo, float w) {
    float* out = sm + xo;
    const float* b = sm + L.b;
    const float* dv = sm + L.dinv;
    coarse_rows(L, sm, sm + xi, [&](int r, int pr, float xc, float acc) {
      out[pr] = fmaf(w * dv[r], b[r] - acc, xc);
    });
    __syncthreads();
  };
  // down
  for (int l = 0; l < c.nl; ++l) {
    const MgCoarseLevel& L = c.L[l];
    rows(L, [&](int r, int pr, int, int, int) {  // the sweep from zero
      sm[L.x + pr] = c.w.at(0) * sm[L.dinv + r] * sm[L.b + r];
    });
    __syncthreads();
    if (l + 1 == c.nl) {  // coarsest: four more sweeps, ending in x
      for (int s = 0; s < kCoarseSweeps; s += 2) {
        sweep(L, L.x, L.t, c.w.at(s + 1));
        sweep(L, L.t, L.x, c.w.at(s + 2));
      }
      break;
    }
    sweep(L, L.x, L.t, c.w.at(1));
    {  // residual into x
      float* out = sm + L.x;
      const float* b = sm + L.b;
      coarse_rows(L, sm, sm + L.t,
                  [&](int r, int pr, float, float acc) { out[pr] = b[r] - acc; });
    }
    __syncthreads();
    const MgCoarseLevel& C = c.L[l + 1];
    rows(C, [&](int q, int, int I, int J, int K) {  // restriction from the fine x
      const float* f = sm + L.x + (2 * I + 2) + L.q0 * (2 * J + 2) + L.q1 * (2 * K + 2);
      auto plane = [&](const float* p) {
        const float r0 = fmaf(0.5f, p[-L.q0 - 1] + p[-L.q0 + 1], p[-L.q0]);
        const float r1 = fmaf(0.5f, p[-1] + p[1], p[0]);
        const float r2 = fmaf(0.5f, p[L.q0 - 1] + p[L.q0 + 1], p[L.q0]);
        return fmaf(0.5f, r0 + r2, r1);
      };
      sm[C.b + q] = fmaf(0.5f, plane(f - L.q1) + plane(f + L.q1), plane(f));
    });
    __syncthreads();
  }
  // up: x = t + P x_c (trilinear over the zero-halo coarse x: an even lattice position p
  // reads coarse position p / 2 twice, an odd one p / 2 and p / 2 + 1), then two sweeps
  for (int l = c.nl - 2; l >= 0; --l) {
    const MgCoarseLevel& L = c.L[l];
    const MgCoarseLevel& C = c.L[l + 1];
    const float* xc = sm + C.x;
    rows(L, [&](int, int pr, int i, int j, int k) {
      const int a0 = (i + 1) >> 1, a1 = (i + 2) >> 1;
      const int b0 = C.q0 * ((j + 1) >> 1), b1 = C.q0 * ((j + 2) >> 1);
      const int g0 = C.q1 * ((k + 1) >> 1), g1 = C.q1 * ((k + 2) >> 1);
      const float v0 = (xc[a0 + b0 + g0] + xc[a1 + b0 + g0]) + (xc[a0 + b1 + g0] + xc[a1 + b1 + g0]);
      const float v1 = (xc[a0 + b0 + g1] + xc[a1 + b0 + g1]) + (xc[a0 + b1 + g1] + xc[a1 + b1 + g1]);
      sm[L.x + pr] = fmaf(0.125f, v0 + v1, sm[L.t + pr]);
    });
    __syncthreads();
    sweep(L, L.x, L.t, c.w.at(0));
    sweep(L, L.t, L.x, c.w.at(1));
  }
  const MgCoarseLevel& L0 = c.L[0];
  rows(L0, [&](int r, int pr, int, int, int) { c.x0[r] = sm[L0.x + pr]; });
}

}  // namespace

struct LatticeMG {
  struct Level {
    LatticeQ1Op op;
    int m0, m1, m2;
    int64_t n;
    float *x, *b, *t, *dinv;
  };
  gfe_ctx* ctx;
  std::vector<Level> lv;
  DevBuf buf;
  // the V-cycle's launches, captured once per (r, z, done) and replayed
  cudaGraphExec_t exec = nullptr;
  const float* cap_r = nullptr;
  float* cap_z = nullptr;
  const int* cap_done = nullptr;
  long long nodes = 0;
  MgDot cap_dot{};
  gfe_learned_pc* learned = nullptr;  // the fine level's smoother when set
  SweepPair w{0.8f, 0.8f};             // smoothing factors of every level
  MgDot dot{};                         // formed by the cycle's last sweep when dot.v is set
  explicit LatticeMG(gfe_ctx* c) : ctx(c), buf(c) {}
  ~LatticeMG() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

namespace {

unsigned vgrid(gfe_ctx* ctx, int64_t n) {
  return (unsigned)std::max<int64_t>(
      1, std::min<int64_t>((n + kMgBlock - 1) / kMgBlock, (int64_t)ctx->num_sms * 8));
}

// whether level l and all coarser ones run in one block
bool coarse_from(const LatticeMG* mg, size_t l) {
  return mg->lv[l].n <= kCoarseRows && mg->lv.size() - l <= (size_t)kMaxCoarse;
}

// the block's view of levels l .. end: shared-memory offsets, weights and global sources
CoarseLevels coarse_levels(const LatticeMG* mg, size_t l) {
  CoarseLevels c{};
  c.nl = (int)(mg->lv.size() - l);
  int off = 0;
  for (int q = 0; q < c.nl; ++q) {
    const LatticeMG::Level& Q = mg->lv[l + q];
    MgCoarseLevel& S = c.L[q];
    S.m0 = Q.m0;
    S.m1 = Q.m1;
    S.m2 = Q.m2;
    S.n = (int)Q.n;
    S.q0 = Q.m0 + 2;
    S.q1 = S.q0 * (Q.m1 + 2);
    S.c1 = Q.op.c1;
    S.c2 = Q.op.c2;
    S.ncell = Q.op.c2 * Q.op.n2;
    // segments: enough (column, segment) items for the block, at most 8 rows each
    const int cols = Q.m0 * Q.m1;
    S.ks = std::max(1, std::min(8, cols * Q.m2 / kCoarseBlock));
    S.nseg = (Q.m2 + S.ks - 1) / S.ks;
    const int np = S.q1 * (Q.m2 + 2);
    S.x = off;
    S.t = off + np;
    S.b = off + 2 * np;
    S.dinv = S.b + S.n;
    S.kap = S.dinv + S.n;
    off = S.kap + S.ncell;
    for (int e = 0; e < 8; ++e) S.W[e] = Q.op.K[8 * e];
    S.gkap = Q.op.kap;
    S.gdinv = Q.dinv;
  }
  c.floats = off;
  c.w = mg->w;
  c.b0 = mg->lv[l].b;
  c.x0 = mg->lv[l].x;
  return c;
}

// The V-cycle of level l: b in L.b, the result in L.x. Sweeps alternate between L.x and L.t
// (a fused sweep cannot run in place); the sweep counts keep the result in L.x: the first
// sweep from zero writes L.x, one more pre-sweep moves it to L.t, the residual goes to L.x,
// prolongation writes L.x from L.t, and the two post-sweeps return to L.x. The coarsest
// level takes the first sweep and four more.
int vcycle(LatticeMG* mg, size_t l, const int* done) {
  gfe_ctx* ctx = mg->ctx;
  cudaStream_t st = ctx->stream;
  LatticeMG::Level& L = mg->lv[l];
  const unsigned g = vgrid(ctx, L.n);
  const dim3 ga = L.op.grid(L.n);
  const bool coarsest = l + 1 == mg->lv.size();
  const int pre = coarsest ? kCoarseSweeps + 1 : kPreSweeps;
  if (coarse_from(mg, l)) {  // this level and all coarser ones in one block
    const CoarseLevels c = coarse_levels(mg, l);
    GFE_CUDA_TRY(launch_pdl(k_mg_coarse, dim3(1), kCoarseBlock, sizeof(float) * c.floats, st,
                            c, done));
    ctx->launches++;
    return GFE_OK;
  }
  float* cur = L.x;
  float* oth = L.t;
  // lattices too small for 4 blocks per SM march one k-plane per thread
  const bool deep = (int64_t)ga.x * ga.y * ga.z >= 4 * (int64_t)ctx->num_sms;
  const dim3 ga1 = L.op.grid_k(1);
  auto smooth = [&](const float* xi, float* xo, float w) -> int {
    if (deep)
      GFE_CUDA_TRY(launch_pdl(k_mg_smooth<kLatK>, ga, kMgBlock, 0, st, L.op, xi, L.b, L.dinv,
                              xo, w, done));
    else
      GFE_CUDA_TRY(launch_pdl(k_mg_smooth<1>, ga1, kMgBlock, 0, st, L.op, xi, L.b, L.dinv,
                              xo, w, done));
    ctx->launches++;
    return GFE_OK;
  };
  // the last sweep of the fine level, with the caller's dot product
  auto smooth_dot = [&](const float* xi, float* xo, float w) -> int {
    if (deep)
      GFE_CUDA_TRY(launch_pdl(k_mg_smooth_dot<kLatK>, ga, kMgBlock, 0, st, L.op, xi, L.b,
                              L.dinv, xo, w, done, mg->dot));
    else
      GFE_CUDA_TRY(launch_pdl(k_mg_smooth_dot<1>, ga1, kMgBlock, 0, st, L.op, xi, L.b, L.dinv,
                              xo, w, done, mg->dot));
    ctx->launches++;
    return GFE_OK;
  };
  auto residual = [&](const float* x, float* r) -> int {
    if (deep)
      GFE_CUDA_TRY(launch_pdl(k_mg_residual<kLatK>, ga, kMgBlock, 0, st, L.op, x, L.b, r,
                              done));
    else
      GFE_CUDA_TRY(launch_pdl(k_mg_residual<1>, ga1, kMgBlock, 0, st, L.op, x, L.b, r, done));
    ctx->launches++;
    return GFE_OK;
  };
  auto restrict_to = [&](const LatticeMG::Level& C, const float* r) -> int {
    const dim3 gc = C.op.grid(C.n);
    if ((int64_t)gc.x * gc.y * gc.z >= 4 * (int64_t)ctx->num_sms)
      GFE_CUDA_TRY(launch_pdl(k_mg_restrict<kLatK>, gc, kMgBlock, 0, st, L.m0, L.m1, C.m0,
                              C.m1, C.m2, r, C.b, done));
    else
      GFE_CUDA_TRY(launch_pdl(k_mg_restrict<1>, C.op.grid_k(1), kMgBlock, 0, st, L.m0, L.m1,
                              C.m0, C.m1, C.m2, r, C.b, done));
    ctx->launches++;
    return GFE_OK;
  };
  auto prolong = [&](const LatticeMG::Level& C, const float* xf, float* xo) -> int {
    if (deep)
      GFE_CUDA_TRY(launch_pdl(k_mg_prolong<kLatK>, ga, kMgBlock, 0, st, L.m0, L.m1, L.m2,
                              C.m0, C.m1, C.m2, (const float*)C.x, xf, xo, done));
    else
      GFE_CUDA_TRY(launch_pdl(k_mg_prolong<1>, ga1, kMgBlock, 0, st, L.m0, L.m1, L.m2, C.m0,
                              C.m1, C.m2, (const float*)C.x, xf, xo, done));
    ctx->launches++;
    return GFE_OK;
  };
  if (l == 0 && mg->learned && !coarsest) {
    // learned smoothing on the fine level: x = M(b); r = b - A x to the coarse level;
    // t = x + P x_c; x = t + M(b - A t)
    LatticeMG::Level& C = mg->lv[l + 1];
    GFE_TRY(learned_apply_into(ctx, mg->learned, L.b, nullptr, L.x, done, false));
    GFE_TRY(residual(L.x, L.t));
    GFE_TRY(restrict_to(C, L.t));
    GFE_TRY(vcycle(mg, l + 1, done));
    GFE_TRY(prolong(C, L.x, L.t));
    GFE_TRY(residual(L.t, L.x));
    return learned_apply_into(ctx, mg->learned, L.x, L.t, L.x, done, false);
  }
  const bool fuse_pre = pre >= 2 && (kFusePreDeep || !deep);
  if (fuse_pre) {  // the sweep from zero and the next one in one pass
    if (deep)
      GFE_CUDA_TRY(launch_pdl(k_mg_pre<kLatK>, ga, kMgBlock, 0, st, L.op, (const float*)L.b,
                              (const float*)L.dinv, oth, mg->w.at(0), mg->w.at(1), done));
    else
      GFE_CUDA_TRY(launch_pdl(k_mg_pre<1>, ga1, kMgBlock, 0, st, L.op, (const float*)L.b,
                              (const float*)L.dinv, oth, mg->w.at(0), mg->w.at(1), done));
    std::swap(cur, oth);
  } else {
    GFE_CUDA_TRY(launch_pdl(k_mg_jacobi0, dim3(g), kMgBlock, 0, st, L.n, (const float*)L.b,
                            (const float*)L.dinv, cur, mg->w.at(0), done));
  }
  ctx->launches++;
  for (int s = fuse_pre ? 2 : 1; s < pre; ++s) {
    GFE_TRY(smooth(cur, oth, mg->w.at(s)));
    std::swap(cur, oth);
  }
  if (coarsest) return cur == L.x ? GFE_OK
                                  : set_error(GFE_ERR_UNSUPPORTED, "multigrid: sweep parity");
  LatticeMG::Level& C = mg->lv[l + 1];
  GFE_TRY(residual(cur, oth));
  GFE_TRY(restrict_to(C, oth));
  GFE_TRY(vcycle(mg, l + 1, done));
  // x + P x_c into the buffer that the post-sweeps then leave the result in L.x from (in
  // place when that is where x already is)
  float* post0 = kPostSweeps % 2 == 0 ? L.x : L.t;
  GFE_TRY(prolong(C, cur, post0));
  cur = post0;
  oth = post0 == L.x ? L.t : L.x;
  for (int s = 0; s < kPostSweeps; ++s) {
    if (l == 0 && mg->dot.v && s + 1 == kPostSweeps)
      GFE_TRY(smooth_dot(cur, oth, mg->w.at(s)));
    else
      GFE_TRY(smooth(cur, oth, mg->w.at(s)));
    std::swap(cur, oth);
  }
  return cur == L.x ? GFE_OK : set_error(GFE_ERR_UNSUPPORTED, "multigrid: sweep parity");
}

}  // namespace

// Levels below the fine lattice operator; the fine level's b and x are set per apply.
int mg_create(gfe_ctx* ctx, const LatticeQ1Op& fine, LatticeMG** out) {
  LatticeMG* mg = new LatticeMG(ctx);
  *out = mg;
  mg->w = sweep_pair(stiffness_spectral_bound(fine.K));
  std::vector<LatticeQ1Op> ops{fine};
  while (ops.size() < 12) {
    const LatticeQ1Op& f = ops.back();
    if ((f.n0 & 1) || (f.n1 & 1) || (f.n2 & 1) || f.n0 < 8 || f.n1 < 8 || f.n2 < 8) break;
    LatticeQ1Op c = f;
    c.n0 = f.n0 / 2;
    c.n1 = f.n1 / 2;
    c.n2 = f.n2 / 2;
    c.s1 = c.n0 - 1;
    c.s2 = (c.n0 - 1) * (c.n1 - 1);
    c.c1 = (c.n0 + 3) & ~3;
    c.c2 = c.c1 * c.n1;
    c.p1 = (c.n0 + 1 + 3) & ~3;
    c.p2 = c.p1 * (c.n1 + 1);
    for (int e = 0; e < 64; ++e) c.K[e] = 2.f * f.K[e];
    c.kap = nullptr;
    ops.push_back(c);
  }
  // one buffer: per level x, b, t, dinv (+ kappa below the fine level), 256-byte aligned
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t total = 0;
  for (size_t l = 0; l < ops.size(); ++l) {
    const int64_t n = (int64_t)(ops[l].n0 - 1) * (ops[l].n1 - 1) * (ops[l].n2 - 1);
    total += 4 * al(sizeof(float) * n);
    if (l) total += al(sizeof(float) * (size_t)ops[l].c2 * ops[l].n2);
  }
  GFE_TRY(mg->buf.reserve(total));
  char* p = (char*)mg->buf.ptr;
  for (size_t l = 0; l < ops.size(); ++l) {
    LatticeMG::Level L;
    L.op = ops[l];
    L.m0 = L.op.n0 - 1;
    L.m1 = L.op.n1 - 1;
    L.m2 = L.op.n2 - 1;
    L.n = (int64_t)L.m0 * L.m1 * L.m2;
    const size_t vb = al(sizeof(float) * L.n);
    L.x = (float*)p;
    L.b = (float*)(p + vb);
    L.t = (float*)(p + 2 * vb);
    L.dinv = (float*)(p + 3 * vb);
    p += 4 * vb;
    if (l) {
      L.op.kap = (float*)p;  // kappa of this level, formed by mg_refresh
      p += al(sizeof(float) * (size_t)L.op.c2 * L.op.n2);
    }
    mg->lv.push_back(L);
  }
  // the coarse kappa arrays' padding columns (every refresh writes the cells only)
  for (size_t l = 1; l < mg->lv.size(); ++l)
    GFE_CUDA_TRY(cudaMemsetAsync(const_cast<float*>(mg->lv[l].op.kap), 0,
                                 sizeof(float) * (size_t)mg->lv[l].op.c2 * mg->lv[l].op.n2,
                                 ctx->stream));
  GFE_TRY(mg_refresh(mg, fine));
  for (size_t l = 0; l < mg->lv.size(); ++l) {
    if (!coarse_from(mg, l)) continue;
    const size_t bytes = sizeof(float) * (size_t)coarse_levels(mg, l).floats;
    if (bytes > 48 * 1024)
      GFE_CUDA_TRY(cudaFuncSetAttribute(k_mg_coarse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)bytes));
    break;
  }
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

// The coarse kappa and D^-1 of every level from the fine operator's kappa (the same
// dimensions and kappa array as the hierarchy was created for; its values may have changed)
int mg_refresh(LatticeMG* mg, const LatticeQ1Op& fine) {
  gfe_ctx* ctx = mg->ctx;
  mg->lv[0].op.kap = fine.kap;
  for (size_t l = 0; l < mg->lv.size(); ++l) {
    const LatticeMG::Level& L = mg->lv[l];
    const LatticeQ1Op* C = l + 1 < mg->lv.size() ? &mg->lv[l + 1].op : nullptr;
    GFE_CUDA_TRY(launch_pdl(k_mg_refresh, dim3((unsigned)((L.m0 + 31) / 32),
                                              (unsigned)((L.m1 + 7) / 8), (unsigned)L.m2),
                            kMgBlock, 0, ctx->stream, L.op, L.dinv,
                            C ? const_cast<float*>(C->kap) : nullptr, C ? C->c1 : 0,
                            C ? (int64_t)C->c2 : (int64_t)0));
    ctx->launches++;
  }
  return GFE_OK;
}

bool mg_fuses_dot(const LatticeMG* mg) {
  return !mg->learned && mg->lv.size() > 1 && !coarse_from(mg, 0);
}

namespace {
MgDot dot_or_none(const LatticeMG* mg, const MgDot* dot) {
  return dot && mg_fuses_dot(mg) ? *dot : MgDot{};
}
bool same_dot(const MgDot& a, const MgDot& b) {
  return a.v == b.v && a.partials == b.partials && a.ticket == b.ticket && a.den == b.den &&
         a.out == b.out;
}
}  // namespace

// z = V-cycle(r) on the fine lattice rows
int mg_apply(LatticeMG* mg, const float* r, float* z, const int* done, const MgDot* dot) {
  gfe_ctx* ctx = mg->ctx;
  const MgDot d = dot_or_none(mg, dot);
  if (!mg->exec || mg->cap_r != r || mg->cap_z != z || mg->cap_done != done ||
      !same_dot(mg->cap_dot, d)) {
    if (mg->exec) {
      cudaGraphExecDestroy(mg->exec);
      mg->exec = nullptr;
    }
    mg->lv[0].b = const_cast<float*>(r);
    mg->lv[0].x = z;
    mg->dot = d;
    const long long l0 = ctx->launches;
    cudaGraph_t graph = nullptr;
    GFE_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int st = vcycle(mg, 0, done);
    const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    ctx->launches = l0;  // counted when replayed
    if (st != GFE_OK || ce != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return st != GFE_OK ? st
                          : set_error(GFE_ERR_CUDA, "multigrid: graph capture failed: %s",
                                      cudaGetErrorString(ce));
    }
    const cudaError_t ie = cudaGraphInstantiate(&mg->exec, graph, 0);
    size_t nodes = 0;
    cudaGraphGetNodes(graph, nullptr, &nodes);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess)
      return set_error(GFE_ERR_CUDA, "multigrid: graph instantiate failed: %s",
                       cudaGetErrorString(ie));
    mg->cap_r = r;
    mg->cap_z = z;
    mg->cap_done = done;
    mg->cap_dot = d;
    mg->nodes = (long long)nodes;
  }
  timer_begin(ctx, GFE_KT_PRECOND);
  GFE_CUDA_TRY(cudaGraphLaunch(mg->exec, ctx->stream));
  timer_end(ctx);
  ctx->launches += mg->nodes;
  return GFE_OK;
}

int mg_record(LatticeMG* mg, const float* r, float* z, const int* done, const MgDot* dot) {
  mg->lv[0].b = const_cast<float*>(r);
  mg->lv[0].x = z;
  mg->dot = dot_or_none(mg, dot);
  return vcycle(mg, 0, done);
}

int mg_set_learned(LatticeMG* mg, gfe_learned_pc* pc) {
  if (pc && learned_ndofs(pc) != mg->lv[0].n)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "multigrid: the learned smoother covers %lld "
                     "dofs, the fine level %lld", (long long)learned_ndofs(pc),
                     (long long)mg->lv[0].n);
  if (mg->learned != pc && mg->exec) {
    cudaGraphExecDestroy(mg->exec);
    mg->exec = nullptr;
  }
  mg->learned = pc;
  return GFE_OK;
}

void mg_destroy(LatticeMG* mg) { delete mg; }

}  // namespace gfe
