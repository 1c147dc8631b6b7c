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
// weighting 1, 1/2, 1/4, 1/8). Smoothing is damped Jacobi (omega 0.8, two sweeps before and
// after, the first from zero), each later sweep fused into one pass over the lattice stencil;
// the coarsest level takes five sweeps. Levels of at most 512 rows run their part of the
// cycle in one block. All vectors are FP32 in the lattice row order; every kernel returns at
// once when the solver's done flag is set.
#include <utility>
#include <vector>

#include "gfe_internal.h"

namespace gfe {
#include "gfe_lattice.cuh"

namespace {

constexpr int kMgBlock = 256;
constexpr float kOmega = 0.8f;
constexpr int kPreSweeps = 2, kPostSweeps = 2, kCoarseSweeps = 4;

__device__ __forceinline__ bool stop(const int* done) { return done && *done; }

// One damped Jacobi sweep fused into the lattice apply: xo = x + omega D^-1 (b - A x)
// (xo != x: the sweep reads the old neighbours). Same arithmetic as an apply into t followed
// by the update x += omega D^-1 (b - t).
template <int KZ>
__global__ void __launch_bounds__(kMgBlock)
    k_mg_smooth(LatticeQ1Op op, const float* __restrict__ x, const float* __restrict__ b,
                const float* __restrict__ dinv, float* __restrict__ xo, const int* done) {
  if (stop(done)) return;
  auto epi = [&](int64_t row, float xc, float acc) {
    xo[row] = fmaf(kOmega * __ldg(dinv + row), __ldg(b + row) - acc, xc);
  };
  lattice_rows<false, decltype(epi), KZ>(op, (int)blockIdx.x, (int)blockIdx.y,
                                         (int)blockIdx.z, x, epi);
}

// The first two sweeps in one pass: x0 = omega D^-1 b (the sweep from zero, formed on the fly
// at the neighbours) and xo = x0 + omega D^-1 (b - A x0). x0 itself is not stored: the cycle
// reads only xo afterwards.
template <int KZ>
__global__ void __launch_bounds__(kMgBlock)
    k_mg_pre(LatticeQ1Op op, const float* __restrict__ b, const float* __restrict__ dinv,
             float* __restrict__ xo, const int* done) {
  if (stop(done)) return;
  const LatticeLoadJacobi0 x0{b, dinv, kOmega};
  auto epi = [&](int64_t row, float xc, float acc) {
    xo[row] = fmaf(kOmega * __ldg(dinv + row), __ldg(b + row) - acc, xc);
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

// x = omega D^-1 b  (first sweep from zero)
__global__ void k_mg_jacobi0(int64_t n, const float* __restrict__ b,
                             const float* __restrict__ dinv, float* __restrict__ x,
                             const int* done) {
  if (stop(done)) return;
  for (int64_t i = (int64_t)blockIdx.x * kMgBlock + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kMgBlock)
    x[i] = kOmega * dinv[i] * b[i];
}

// b_c = R r_f: coarse interior node (I, J, K) sits on fine interior node (2I+1, 2J+1, 2K+1);
// weights prod_d (1 - |delta_d| / 2) over the 27 fine neighbours
__global__ void k_mg_restrict(int mf0, int mf1, int mc0, int mc1, int mc2,
                              const float* __restrict__ rf, float* __restrict__ bc,
                              const int* done) {
  if (stop(done)) return;
  const int64_t nc = (int64_t)mc0 * mc1 * mc2;
  for (int64_t c = (int64_t)blockIdx.x * kMgBlock + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * kMgBlock) {
    // 32-bit index split (levels hold fewer than 2^31 rows)
    const uint32_t cu = (uint32_t)c, rest = cu / (uint32_t)mc0;
    const int I = (int)(cu - rest * (uint32_t)mc0);
    const int K = (int)(rest / (uint32_t)mc1), J = (int)(rest - (uint32_t)K * (uint32_t)mc1);
    float s = 0.f;
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
          const float w = (dx ? 0.5f : 1.f) * (dy ? 0.5f : 1.f) * (dz ? 0.5f : 1.f);
          const int64_t f = (int64_t)(2 * I + 1 + dx) +
                            (int64_t)mf0 * ((2 * J + 1 + dy) + (int64_t)mf1 * (2 * K + 1 + dz));
          s = fmaf(w, rf[f], s);
        }
    bc[c] = s;
  }
}

// (P x_c) at fine interior node (i, j, k): trilinear, coarse boundary nodes are zero
__device__ __forceinline__ float prolong_value(int i, int j, int k, int mc0, int mc1, int mc2,
                                               const float* __restrict__ xc) {
  int ci[2], cj[2], ck[2];
  float wi[2], wj[2], wk[2];
  auto axis = [](int p, int mc, int* cc, float* ww) {  // p = lattice position (1-based)
    if ((p & 1) == 0) {
      cc[0] = p / 2 - 1;
      ww[0] = 1.f;
      cc[1] = -1;
      ww[1] = 0.f;
    } else {
      cc[0] = p / 2 - 1;  // coarse interior index of lattice p/2 (-1: boundary)
      cc[1] = p / 2;      // of lattice p/2 + 1 (mc: boundary)
      ww[0] = ww[1] = 0.5f;
      if (cc[1] >= mc) cc[1] = -1;
    }
  };
  axis(i + 1, mc0, ci, wi);
  axis(j + 1, mc1, cj, wj);
  axis(k + 1, mc2, ck, wk);
  float s = 0.f;
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int bb = 0; bb < 2; ++bb)
#pragma unroll
      for (int cc = 0; cc < 2; ++cc) {
        if (ci[a] < 0 || cj[bb] < 0 || ck[cc] < 0) continue;
        const float w = wi[a] * wj[bb] * wk[cc];
        if (w == 0.f) continue;
        s = fmaf(w, xc[(int64_t)ci[a] + (int64_t)mc0 * (cj[bb] + (int64_t)mc1 * ck[cc])], s);
      }
  return s;
}

// xo_f = x_f + P x_c (xo may be xf: each thread reads and writes its own rows only)
__global__ void k_mg_prolong(int mf0, int mf1, int mf2, int mc0, int mc1, int mc2,
                             const float* __restrict__ xc, const float* xf, float* xo,
                             const int* done) {
  if (stop(done)) return;
  const int64_t nf = (int64_t)mf0 * mf1 * mf2;
  for (int64_t f = (int64_t)blockIdx.x * kMgBlock + threadIdx.x; f < nf;
       f += (int64_t)gridDim.x * kMgBlock) {
    const uint32_t fu = (uint32_t)f, rest = fu / (uint32_t)mf0;
    const int i = (int)(fu - rest * (uint32_t)mf0);
    const int k = (int)(rest / (uint32_t)mf1), j = (int)(rest - (uint32_t)k * (uint32_t)mf1);
    xo[f] = xf[f] + prolong_value(i, j, k, mc0, mc1, mc2, xc);
  }
}

// coarse kappa = mean of the 8 children (padded row strides cf1, cc1)
__global__ void k_mg_kappa(int nc0, int nc1, int nc2, int cf1, int nf1, int cc1,
                           const float* __restrict__ kf, float* __restrict__ kc) {
  const int64_t n = (int64_t)nc0 * nc1 * nc2;
  for (int64_t c = (int64_t)blockIdx.x * kMgBlock + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * kMgBlock) {
    const int I = (int)(c % nc0);
    const int64_t rest = c / nc0;
    const int J = (int)(rest % nc1), K = (int)(rest / nc1);
    float s = 0.f;
    for (int e = 0; e < 8; ++e) {
      const int i = 2 * I + (e & 1), j = 2 * J + ((e >> 1) & 1), k = 2 * K + (e >> 2);
      s += kf[(int64_t)i + (int64_t)cf1 * (j + (int64_t)nf1 * k)];
    }
    kc[(int64_t)I + (int64_t)cc1 * (J + (int64_t)nc1 * K)] = 0.125f * s;
  }
}

// D^-1 of a lattice operator: D_r = sum of kappa_K Kref[l_r, l_r] over the 8 cells around r
__global__ void k_mg_diag(LatticeQ1Op op, float* __restrict__ dinv) {
  const int m0 = op.n0 - 1, m1 = op.n1 - 1, m2 = op.n2 - 1;
  const int64_t n = (int64_t)m0 * m1 * m2;
  for (int64_t r = (int64_t)blockIdx.x * kMgBlock + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * kMgBlock) {
    const int i = (int)(r % m0);
    const int64_t rest = r / m0;
    const int j = (int)(rest % m1), k = (int)(rest / m1);
    float d = 0.f;
    for (int e = 0; e < 8; ++e) {
      const int cx = e & 1, cy = (e >> 1) & 1, cz = e >> 2;
      const int lr = (1 - cx) + 2 * (1 - cy) + 4 * (1 - cz);
      d += op.kap[(int64_t)(i + cx) + (int64_t)op.c1 * (j + cy) + (int64_t)op.c2 * (k + cz)] *
           op.K[lr + 8 * lr];
    }
    dinv[r] = d > 0.f ? 1.f / d : 0.f;
  }
}

// ---- the coarse levels in one block ------------------------------------------------------
// Levels of at most kCoarseRows rows run their whole V-cycle inside one block of kCoarseBlock
// threads (block-stride loops, a barrier between steps): on such lattices a launch costs
// more than its work. The row operator below follows lattice_rows' loop order exactly. (With
// 15^3-row levels inside, the one block's issue rate made the cycle slower than launches.)
constexpr int kCoarseBlock = 512;
constexpr int64_t kCoarseRows = 512;
constexpr int kMaxCoarse = 6;

struct MgLevelView {
  LatticeQ1Op op;
  int m0, m1, m2;
  int64_t n;
  float *x, *b, *t, *dinv;
};

struct CoarseLevels {
  int nl;
  MgLevelView L[kMaxCoarse];
};

// (A p)_r at interior node (i, j, k): its 27 neighbours loaded once (0 outside the interior),
// then the 8 cells around it, 8 local columns each, in lattice_rows' order (32-bit indexing:
// these levels are small). `load(row)` gives p at a row.
template <class Load>
__device__ __forceinline__ float lattice_row_value_f(const LatticeQ1Op& op, int i, int j, int k,
                                                     const Load& load) {
  const int m0 = op.n0 - 1, m1 = op.n1 - 1, m2 = op.n2 - 1;
  float v[27];
#pragma unroll
  for (int dz = 0; dz < 3; ++dz)
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) {
        const int ii = i - 1 + dx, jj = j - 1 + dy, kk = k - 1 + dz;
        const bool in = ii >= 0 && ii < m0 && jj >= 0 && jj < m1 && kk >= 0 && kk < m2;
        v[dx + 3 * dy + 9 * dz] = in ? load(ii + op.s1 * jj + op.s2 * kk) : 0.f;
      }
  float acc = 0.f;
#pragma unroll
  for (int cz = 0; cz < 2; ++cz)
#pragma unroll
    for (int cy = 0; cy < 2; ++cy)
#pragma unroll
      for (int cx = 0; cx < 2; ++cx) {
        const int lr = (1 - cx) + 2 * (1 - cy) + 4 * (1 - cz);
        float s = 0.f;
#pragma unroll
        for (int lc = 0; lc < 8; ++lc)
          s = fmaf(op.K[lr + 8 * lc],
                   v[(cx + (lc & 1)) + 3 * (cy + ((lc >> 1) & 1)) + 9 * (cz + (lc >> 2))], s);
        acc = fmaf(op.kap[(i + cx) + op.c1 * (j + cy) + op.c2 * (k + cz)], s, acc);
      }
  return acc;
}

__device__ __forceinline__ float lattice_row_value(const LatticeQ1Op& op, int i, int j, int k,
                                                   const float* __restrict__ p) {
  return lattice_row_value_f(op, i, j, k, [p](int row) { return p[row]; });
}

__device__ __forceinline__ void row_ijk(const MgLevelView& L, int64_t r, int& i, int& j,
                                        int& k) {
  const uint32_t ru = (uint32_t)r, rest = ru / (uint32_t)L.m0;
  i = (int)(ru - rest * (uint32_t)L.m0);
  k = (int)(rest / (uint32_t)L.m1);
  j = (int)(rest - (uint32_t)k * (uint32_t)L.m1);
}

// the V-cycle of levels 0 .. nl-1 of `c` (level 0's b is given, its result lands in its x);
// same steps, sweep counts and buffer roles as the multi-launch cycle
__global__ void __launch_bounds__(kCoarseBlock)
    k_mg_coarse(const __grid_constant__ CoarseLevels c, const int* done) {
  if (stop(done)) return;
  const int t0 = threadIdx.x;
  auto sweep = [&](const MgLevelView& L, const float* xi, float* xo) {
    for (int64_t r = t0; r < L.n; r += kCoarseBlock) {
      int i, j, k;
      row_ijk(L, r, i, j, k);
      const float acc = lattice_row_value(L.op, i, j, k, xi);
      xo[r] = fmaf(kOmega * L.dinv[r], L.b[r] - acc, xi[r]);
    }
    __syncthreads();
  };
  auto first = [&](const MgLevelView& L) {
    for (int64_t r = t0; r < L.n; r += kCoarseBlock) L.x[r] = kOmega * L.dinv[r] * L.b[r];
    __syncthreads();
  };
  // down
  for (int l = 0; l < c.nl; ++l) {
    const MgLevelView& L = c.L[l];
    first(L);
    if (l + 1 == c.nl) {  // coarsest: four more sweeps, ending in x
      for (int s = 0; s < kCoarseSweeps; s += 2) {
        sweep(L, L.x, L.t);
        sweep(L, L.t, L.x);
      }
      break;
    }
    sweep(L, L.x, L.t);
    for (int64_t r = t0; r < L.n; r += kCoarseBlock) {  // residual into x
      int i, j, k;
      row_ijk(L, r, i, j, k);
      L.x[r] = L.b[r] - lattice_row_value(L.op, i, j, k, L.t);
    }
    __syncthreads();
    const MgLevelView& C = c.L[l + 1];
    for (int64_t q = t0; q < C.n; q += kCoarseBlock) {  // restriction
      int I, J, K;
      row_ijk(C, q, I, J, K);
      float s = 0.f;
#pragma unroll
      for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
          for (int dx = -1; dx <= 1; ++dx) {
            const float w = (dx ? 0.5f : 1.f) * (dy ? 0.5f : 1.f) * (dz ? 0.5f : 1.f);
            const int64_t f =
                (int64_t)(2 * I + 1 + dx) +
                (int64_t)L.m0 * ((2 * J + 1 + dy) + (int64_t)L.m1 * (2 * K + 1 + dz));
            s = fmaf(w, L.x[f], s);
          }
      C.b[q] = s;
    }
    __syncthreads();
  }
  // up: x = t + P x_c, then two sweeps back into x
  for (int l = c.nl - 2; l >= 0; --l) {
    const MgLevelView& L = c.L[l];
    const MgLevelView& C = c.L[l + 1];
    for (int64_t r = t0; r < L.n; r += kCoarseBlock) {
      int i, j, k;
      row_ijk(L, r, i, j, k);
      L.x[r] = L.t[r] + prolong_value(i, j, k, C.m0, C.m1, C.m2, C.x);
    }
    __syncthreads();
    sweep(L, L.x, L.t);
    sweep(L, L.t, L.x);
  }
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
  gfe_learned_pc* learned = nullptr;  // the fine level's smoother when set
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

// The V-cycle of level l: b in L.b, the result in L.x. Sweeps alternate between L.x and L.t
// (a fused sweep cannot run in place); the sweep counts keep the result in L.x: the first
// sweep from zero writes L.x, one more pre-sweep moves it to L.t, the residual goes to L.x,
// prolongation writes L.x from L.t, and the two post-sweeps return to L.x. The coarsest
// level takes the first sweep and four more.
int vcycle(LatticeMG* mg, size_t l, const int* done) {
  gfe_ctx* ctx = mg->ctx;
  LatticeMG::Level& L = mg->lv[l];
  const unsigned g = vgrid(ctx, L.n);
  const dim3 ga = L.op.grid(L.n);
  const bool coarsest = l + 1 == mg->lv.size();
  const int pre = coarsest ? kCoarseSweeps + 1 : kPreSweeps;
  if (L.n <= kCoarseRows && mg->lv.size() - l <= (size_t)kMaxCoarse) {
    // this level and all coarser ones in one block
    CoarseLevels c{};
    c.nl = (int)(mg->lv.size() - l);
    for (int q = 0; q < c.nl; ++q) {
      const LatticeMG::Level& Q = mg->lv[l + q];
      c.L[q] = MgLevelView{Q.op, Q.m0, Q.m1, Q.m2, Q.n, Q.x, Q.b, Q.t, Q.dinv};
    }
    k_mg_coarse<<<1, kCoarseBlock, 0, ctx->stream>>>(c, done);
    ctx->launches++;
    return GFE_OK;
  }
  float* cur = L.x;
  float* oth = L.t;
  // lattices too small for 4 blocks per SM march one k-plane per thread
  const bool deep = (int64_t)ga.x * ga.y * ga.z >= 4 * (int64_t)ctx->num_sms;
  const dim3 ga1 = L.op.grid_k(1);
  auto smooth = [&](const float* xi, float* xo) {
    if (deep)
      k_mg_smooth<kLatK><<<ga, kMgBlock, 0, ctx->stream>>>(L.op, xi, L.b, L.dinv, xo, done);
    else
      k_mg_smooth<1><<<ga1, kMgBlock, 0, ctx->stream>>>(L.op, xi, L.b, L.dinv, xo, done);
    ctx->launches++;
  };
  if (l == 0 && mg->learned && !coarsest) {
    // learned smoothing on the fine level: x = M(b); r = b - A x to the coarse level;
    // t = x + P x_c; x = t + M(b - A t)
    LatticeMG::Level& C = mg->lv[l + 1];
    GFE_TRY(learned_apply_into(ctx, mg->learned, L.b, nullptr, L.x, done, false));
    if (deep)
      k_mg_residual<kLatK><<<ga, kMgBlock, 0, ctx->stream>>>(L.op, L.x, L.b, L.t, done);
    else
      k_mg_residual<1><<<ga1, kMgBlock, 0, ctx->stream>>>(L.op, L.x, L.b, L.t, done);
    k_mg_restrict<<<vgrid(ctx, C.n), kMgBlock, 0, ctx->stream>>>(L.m0, L.m1, C.m0, C.m1, C.m2,
                                                                 L.t, C.b, done);
    ctx->launches += 2;
    GFE_TRY(vcycle(mg, l + 1, done));
    k_mg_prolong<<<g, kMgBlock, 0, ctx->stream>>>(L.m0, L.m1, L.m2, C.m0, C.m1, C.m2, C.x, L.x,
                                                  L.t, done);
    if (deep)
      k_mg_residual<kLatK><<<ga, kMgBlock, 0, ctx->stream>>>(L.op, L.t, L.b, L.x, done);
    else
      k_mg_residual<1><<<ga1, kMgBlock, 0, ctx->stream>>>(L.op, L.t, L.b, L.x, done);
    ctx->launches += 2;
    return learned_apply_into(ctx, mg->learned, L.x, L.t, L.x, done, false);
  }
  if (pre >= 2) {  // the sweep from zero and the next one in one pass
    if (deep)
      k_mg_pre<kLatK><<<ga, kMgBlock, 0, ctx->stream>>>(L.op, L.b, L.dinv, oth, done);
    else
      k_mg_pre<1><<<ga1, kMgBlock, 0, ctx->stream>>>(L.op, L.b, L.dinv, oth, done);
    std::swap(cur, oth);
  } else {
    k_mg_jacobi0<<<g, kMgBlock, 0, ctx->stream>>>(L.n, L.b, L.dinv, cur, done);
  }
  ctx->launches++;
  for (int s = 2; s < pre; ++s) {
    smooth(cur, oth);
    std::swap(cur, oth);
  }
  if (coarsest) return cur == L.x ? GFE_OK
                                  : set_error(GFE_ERR_UNSUPPORTED, "multigrid: sweep parity");
  LatticeMG::Level& C = mg->lv[l + 1];
  if (deep)
    k_mg_residual<kLatK><<<ga, kMgBlock, 0, ctx->stream>>>(L.op, cur, L.b, oth, done);
  else
    k_mg_residual<1><<<ga1, kMgBlock, 0, ctx->stream>>>(L.op, cur, L.b, oth, done);
  k_mg_restrict<<<vgrid(ctx, C.n), kMgBlock, 0, ctx->stream>>>(L.m0, L.m1, C.m0, C.m1, C.m2,
                                                               oth, C.b, done);
  ctx->launches += 2;
  GFE_TRY(vcycle(mg, l + 1, done));
  // x + P x_c into the buffer that the post-sweeps then leave the result in L.x from (in
  // place when that is where x already is)
  float* post0 = kPostSweeps % 2 == 0 ? L.x : L.t;
  k_mg_prolong<<<g, kMgBlock, 0, ctx->stream>>>(L.m0, L.m1, L.m2, C.m0, C.m1, C.m2, C.x, cur,
                                                post0, done);
  ctx->launches++;
  cur = post0;
  oth = post0 == L.x ? L.t : L.x;
  for (int s = 0; s < kPostSweeps; ++s) {
    smooth(cur, oth);
    std::swap(cur, oth);
  }
  return cur == L.x ? GFE_OK : set_error(GFE_ERR_UNSUPPORTED, "multigrid: sweep parity");
}

}  // namespace

// Levels below the fine lattice operator; the fine level's b and x are set per apply.
int mg_create(gfe_ctx* ctx, const LatticeQ1Op& fine, LatticeMG** out) {
  LatticeMG* mg = new LatticeMG(ctx);
  *out = mg;
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
      float* kc = (float*)p;
      p += al(sizeof(float) * (size_t)L.op.c2 * L.op.n2);
      const LatticeQ1Op& f = mg->lv.back().op;
      GFE_CUDA_TRY(cudaMemsetAsync(kc, 0, sizeof(float) * (size_t)L.op.c2 * L.op.n2,
                                   ctx->stream));
      k_mg_kappa<<<vgrid(ctx, (int64_t)L.op.n0 * L.op.n1 * L.op.n2), kMgBlock, 0,
                   ctx->stream>>>(L.op.n0, L.op.n1, L.op.n2, f.c1, f.n1, L.op.c1, f.kap, kc);
      ctx->launches++;
      L.op.kap = kc;
    }
    k_mg_diag<<<vgrid(ctx, L.n), kMgBlock, 0, ctx->stream>>>(L.op, L.dinv);
    ctx->launches++;
    mg->lv.push_back(L);
  }
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

// z = V-cycle(r) on the fine lattice rows
int mg_apply(LatticeMG* mg, const float* r, float* z, const int* done) {
  gfe_ctx* ctx = mg->ctx;
  if (!mg->exec || mg->cap_r != r || mg->cap_z != z || mg->cap_done != done) {
    if (mg->exec) {
      cudaGraphExecDestroy(mg->exec);
      mg->exec = nullptr;
    }
    mg->lv[0].b = const_cast<float*>(r);
    mg->lv[0].x = z;
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
    mg->nodes = (long long)nodes;
  }
  timer_begin(ctx, GFE_KT_PRECOND);
  GFE_CUDA_TRY(cudaGraphLaunch(mg->exec, ctx->stream));
  timer_end(ctx);
  ctx->launches += mg->nodes;
  return GFE_OK;
}

int mg_record(LatticeMG* mg, const float* r, float* z, const int* done) {
  mg->lv[0].b = const_cast<float*>(r);
  mg->lv[0].x = z;
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
