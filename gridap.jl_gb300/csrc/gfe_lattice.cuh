// gfe_lattice.cuh -- the matrix-free FP32 operator of uniform Cartesian Q1 diffusion (the
// lattice operator) and its row kernel, shared by the CG solvers (gfe_solve.cu) and the
// geometric multigrid preconditioner (gfe_mg.cu). Included inside namespace gfe.
#pragma once

// Matrix-free FP32 operator of uniform Cartesian Q1 diffusion on (n0, n1, n2) cells with rows
// = interior nodes in node order (the CLagrangian numbering with every boundary node
// Dirichlet): (A x)_r = sum over the 8 cells K around node r of kappa_K sum_c Kref[l_r, c]
// x[node(K, c)], boundary nodes contributing 0 -- the cell-wise sum the assembled matrix
// stores, applied with FP32 element matrices (kappa_K Kref). It reads kappa (4 B per cell)
// and x instead of 27 values per row. Applied by k_lattice_spmv: a block covers a 32 x 8 tile
// of (i, j) and kLatK consecutive k-planes; each thread marches up its k-column keeping the
// three x-planes and two kappa-planes around its node in registers, so a row costs 9 x and 4
// kappa loads.
constexpr int kLatK = 8;

struct LatticeQ1Op {
  const float* kap;
  int n0, n1, n2;   // cells per direction
  int s1, s2;       // row strides of j and k: m0 and m0*m1 (m = n - 1 interior nodes)
  int c1, c2;       // cell strides of j and k: n0 rounded up to 4, and c1*n1
  int p1, p2;       // strides of the zero-halo padded layout: m0 + 2 rounded up to 4, p1*(m1+2)
  float K[64];      // Kref[li + 8 lj], symmetric
  // padded index of interior node (i, j, k): halo of one zero entry on every side
  __host__ __device__ int64_t pad_index(int i, int j, int k) const {
    return (int64_t)(i + 1) + (int64_t)p1 * (j + 1) + (int64_t)p2 * (k + 1);
  }
  int64_t padded_size() const { return (int64_t)p2 * (n2 + 1); }
  __host__ __device__ dim3 grid(int64_t) const {
    return dim3((unsigned)((n0 - 1 + 31) / 32), (unsigned)((n1 - 1 + 7) / 8),
                (unsigned)((n2 - 1 + kLatK - 1) / kLatK));
  }
  // grid of the tensor-map kernel: k-tiles of kz planes
  dim3 grid_k(int kz) const {
    return dim3((unsigned)((n0 - 1 + 31) / 32), (unsigned)((n1 - 1 + 7) / 8),
                (unsigned)((n2 - 1 + kz - 1) / kz));
  }
  unsigned blocks(int64_t n) const {  // covers both grids (partials are sized from it)
    const dim3 g = grid(n);
    return g.x * g.y * g.z * (kLatK / 2);
  }
};

// p at a row index (the x of the apply)
struct LatticeLoad {
  const float* __restrict__ p;
  __device__ __forceinline__ float operator()(int64_t idx) const { return __ldg(p + idx); }
};

// x0 = omega D^-1 b at a row index (the first Jacobi sweep from zero, formed on the fly)
struct LatticeLoadJacobi0 {
  const float* __restrict__ b;
  const float* __restrict__ dinv;
  float omega;
  __device__ __forceinline__ float operator()(int64_t idx) const {
    return omega * __ldg(dinv + idx) * __ldg(b + idx);
  }
};

// The rows of one tile: (i, j) = (32 bx + lane, 8 by + warp), k-planes KZ bz .. + KZ (KZ = 1
// for small lattices: more blocks, shorter per-thread chains). For every row the epilogue
// receives (row index, p at the row, (A p)_row); `load(index)` gives p.
template <bool PAD, class Epi, int KZ = kLatK, class Load = LatticeLoad>
__device__ __forceinline__ void lattice_rows_f(const LatticeQ1Op& op, int bx, int by, int bz,
                                               const Load& load, Epi& epi) {
  const int m0 = op.n0 - 1, m1 = op.n1 - 1, m2 = op.n2 - 1;
  const int i = bx * 32 + (int)(threadIdx.x & 31);
  const int j = by * 8 + (int)(threadIdx.x >> 5);
  const int k0 = bz * KZ;
  if (i < m0 && j < m1) {
    const bool okx[3] = {i > 0, true, i < m0 - 1};
    const bool oky[3] = {j > 0, true, j < m1 - 1};
    // row (or padded index) of (i, j, 0) and the strides between neighbours
    const int64_t col = PAD ? op.pad_index(i, j, 0) : (int64_t)i + (int64_t)op.s1 * j;
    const int sy = PAD ? op.p1 : op.s1, sz = PAD ? op.p2 : op.s2;
    const float* kcol = op.kap + ((int64_t)i + (int64_t)op.c1 * j);
    // x-plane kk (9 values around (i, j)); 0 outside the interior
    auto xplane = [&](int kk, float* v) {
      const bool okz = PAD || (kk >= 0 && kk < m2);
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
          float t = 0.f;
          if (PAD || (okz && okx[dx + 1] && oky[dy + 1]))
            t = load(col + (int64_t)sz * kk + dx + sy * dy);
          v[(dx + 1) + 3 * (dy + 1)] = t;
        }
    };
    // kappa-plane of cell layer kk: cells (i + cx, j + cy, kk)
    auto kplane = [&](int kk, float* v) {
#pragma unroll
      for (int cy = 0; cy < 2; ++cy)
#pragma unroll
        for (int cx = 0; cx < 2; ++cx)
          v[cx + 2 * cy] = __ldg(kcol + (int64_t)op.c2 * kk + cx + op.c1 * cy);
    };
    // Kref[a][b] depends only on the axes along which local vertices a and b differ (the Q1
    // stiffness of a box is a sum of tensor products of 1-D [[p, q], [q, p]] matrices), so
    //   (A x)_r = sum over the 8 axis classes c of W[c] sum_{d in c} S(d) x_{r+d},
    // S(d) the kappa sum over the cells r and r + d share (a box of 1 or 2 cells per axis).
    // Per row: 5 adds for the new cell layer's box sums, 9 to merge it with the layer below,
    // 27 multiply-adds over the neighbours and 8 over the classes (49 FP32 operations
    // instead of the 72 of a cell-by-cell Kref product).
    float W[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) W[c] = op.K[8 * c];
    // box sums of cell layer kk, indexed e = (dx + 1) + 3 (dy + 1)
    auto layer = [&](int kk, float* L) {
      float v[4];
      kplane(kk, v);
      const float X0 = v[0] + v[1], X1 = v[2] + v[3];
      L[0] = v[0];
      L[1] = X0;
      L[2] = v[1];
      L[3] = v[0] + v[2];
      L[4] = X0 + X1;
      L[5] = v[1] + v[3];
      L[6] = v[2];
      L[7] = X1;
      L[8] = v[3];
    };
    float xa[9], xb[9], xc[9], la[9], lb[9];
    xplane(k0 - 1, xa);
    xplane(k0, xb);
    layer(k0, la);
#pragma unroll
    for (int t = 0; t < KZ; ++t) {
      const int k = k0 + t;
      if (k < m2) {
        xplane(k + 1, xc);
        layer(k + 1, lb);
        float T[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) T[c] = 0.f;
#pragma unroll
        for (int e = 0; e < 9; ++e) {
          const int cl = (e % 3 != 1 ? 1 : 0) | (e / 3 != 1 ? 2 : 0);
          T[cl | 4] = fmaf(la[e], xa[e], T[cl | 4]);
          T[cl] = fmaf(la[e] + lb[e], xb[e], T[cl]);
          T[cl | 4] = fmaf(lb[e], xc[e], T[cl | 4]);
        }
        float acc = 0.f;
#pragma unroll
        for (int c = 0; c < 8; ++c) acc = fmaf(W[c], T[c], acc);
        epi(col + (int64_t)sz * k, xb[4], acc);
      }
#pragma unroll
      for (int e = 0; e < 9; ++e) {
        xa[e] = xb[e];
        xb[e] = xc[e];
        la[e] = lb[e];
      }
    }
  }
}

template <bool PAD, class Epi, int KZ = kLatK>
__device__ __forceinline__ void lattice_rows(const LatticeQ1Op& op, int bx, int by, int bz,
                                             const float* __restrict__ p, Epi& epi) {
  lattice_rows_f<PAD, Epi, KZ>(op, bx, by, bz, LatticeLoad{p}, epi);
}

// q = A p over one tile; adds p.q (and p.r for flexible CG) of the thread's rows to d1 (d2).
template <bool FCG, bool PAD>
__device__ __forceinline__ void lattice_tile(const LatticeQ1Op& op, int bx, int by, int bz,
                                             const float* __restrict__ p, float* __restrict__ q,
                                             const float* __restrict__ rr, float& d1,
                                             float& d2) {
  auto epi = [&](int64_t row, float pc, float acc) {
    q[row] = acc;
    d1 = fmaf(pc, acc, d1);
    if (FCG) d2 = fmaf(pc, __ldg(rr + row), d2);
  };
  lattice_rows<PAD>(op, bx, by, bz, p, epi);
}
