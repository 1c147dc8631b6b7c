// gfe_batch.cu -- many independent Q1 diffusion problems assembled and solved in one
// persistent launch.
//
// The problems (unit cubes with their own partitions (n, n, n), per-cell kappa, constant
// source, homogeneous Dirichlet on the boundary) are uniform Cartesian Q1 grids, so each one's
// assembled operator is the class-sum form of the lattice assembly: A[r, r + d] =
// W[class(d)] * S(d), S(d) the kappa sum over the cells rows r and r + d share, W the entries of
// the reference stiffness by the set of axes along which two vertices differ. Every
// equation is divided by h^3 (which changes neither a solution nor its relative residuals):
// the cells carry kappa / h^2 and the unit-cube tables, and the load of constant f is f at
// every row.
//
// One launch solves all problems: thread blocks take problems from a work counter (atomicAdd,
// largest first; no block ever waits on another) and each runs a whole mixed-precision
// Jacobi-PCG on its problem: FP32 iterations on the operator applied matrix-free from FP32
// kappa (27 neighbours, class sums), FP64 reliable updates (x accumulates in FP64, the true
// residual b - A x is formed in FP64 from the FP64 kappa and replaces the FP32 one whenever
// the FP32 residual has dropped by delta, and decides convergence). Reductions are block
// reductions in a fixed order, so results do not depend on which block took which problem.
// The launch shape (threads per CTA, CTAs per problem) is chosen once per batch by timing the
// first solve with each of six candidates (gfe_batch_set_shape fixes one instead).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gfe_internal.h"

namespace gfe {
namespace batch {

constexpr float kDelta = 0.01f;  // FP32 residual reduction between reliable updates

struct BProb {
  int32_t n;       // cells per direction
  int32_t pad;
  int64_t cell0;   // first cell in the concatenated coefficient array
  int64_t xoff;    // first free dof in the concatenated solution
};

struct PArgs {
  int32_t nproblems;
  const BProb* probs;
  const int32_t* order;   // problems by decreasing size
  int* counter;           // work counter of the large problems (zeroed before the launch)
  int* counter2;          // work counter of the small problems
  int32_t nlarge;         // order[0 .. nlarge) are solved by clusters, the rest by single CTAs
  const double* coef;     // kappa / h^2 per cell, problems one after the other
  double f;               // the load at every row (constant source)
  double rtol2;
  int32_t maxit;
  float* scratch;         // per CTA: kap32 | d | x | r | p | q (a cluster uses its rank 0's)
  int64_t cell_stride, row_stride;
  double* x;              // FP64 solutions, problems one after the other
  int32_t* iters;
  int32_t* conv;
  DevError* err;
  double W64[8];
  float W32[8];
};

// (A x)_r of a uniform Q1 lattice in class-sum form: T the arithmetic type, kap the cell
// coefficients (n^3, Gridap cell order), x the row vector (m^3 interior nodes, node order)
// (x may be written elsewhere in the launch: plain pointers, no read-only cache path)
template <typename T, typename KT, typename XT>
__device__ __forceinline__ T class_apply(int i, int j, int k, int m, int n, const KT* kap,
                                         const XT* x, const T* W) {
  T kv[2][2][2];
#pragma unroll
  for (int cz = 0; cz < 2; ++cz)
#pragma unroll
    for (int cy = 0; cy < 2; ++cy)
#pragma unroll
      for (int cx = 0; cx < 2; ++cx)
        kv[cz][cy][cx] = (T)kap[(i + cx) + (int64_t)n * ((j + cy) + (int64_t)n * (k + cz))];
  T acc[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) acc[c] = (T)0;
  const int64_t r = (int64_t)i + (int64_t)m * (j + (int64_t)m * k);
#pragma unroll
  for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx) {
        const int ii = i + dx, jj = j + dy, kk = k + dz;
        if (ii < 0 || ii >= m || jj < 0 || jj >= m || kk < 0 || kk >= m) continue;
        // kappa sum over the shared cells: cx in {0} (dx=-1), {1} (dx=+1), {0,1} (dx=0)
        T sum = (T)0;
#pragma unroll
        for (int cz = 0; cz < 2; ++cz)
#pragma unroll
          for (int cy = 0; cy < 2; ++cy)
#pragma unroll
            for (int cx = 0; cx < 2; ++cx) {
              const bool in = (dx == 0 || cx == (dx > 0)) && (dy == 0 || cy == (dy > 0)) &&
                              (dz == 0 || cz == (dz > 0));
              if (in) sum += kv[cz][cy][cx];
            }
        const int cl = (dx ? 1 : 0) | (dy ? 2 : 0) | (dz ? 4 : 0);
        acc[cl] += sum * (T)x[r + dx + (int64_t)m * (dy + (int64_t)m * dz)];
      }
  T y = (T)0;
#pragma unroll
  for (int c = 0; c < 8; ++c) y += W[c] * acc[c];
  return y;
}

// ---- thread-block clusters ----------------------------------------------------------------
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// every thread of every CTA of the cluster; orders all memory operations before it (shared,
// distributed shared and global) before those after it, cluster-wide
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// a double in CTA `rank`'s shared memory, at the address of `p` in this CTA
__device__ __forceinline__ double dsmem_ld(const double* p, uint32_t rank) {
  const uint32_t local = (uint32_t)__cvta_generic_to_shared(p);
  uint32_t remote;
  double v;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(rank));
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(remote) : "memory");
  return v;
}

template <int CS>
__device__ __forceinline__ void group_sync() {
  if constexpr (CS > 1)
    cluster_sync();
  else
    __syncthreads();
}

// Shared state of one CTA: the block reduction, the two reduction slots its peers read, and
// the broadcast task.
template <int NT>
struct BShared {
  double red[2 * (NT / 32)];
  double slot[2][2];
  double bc[2];
  int task;
};

// (a, b) summed over the CTA's threads, then over the cluster's CTAs in rank order: every
// thread gets the same two doubles, whichever CTA it is in. `k` alternates the slot, so a
// slot is rewritten only after the barrier of the next reduction, which its readers reach
// after reading it.
template <int NT, int CS>
__device__ __forceinline__ void group_sum2(double& a, double& b, BShared<NT>& sh, int& k) {
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, off);
    b += __shfl_down_sync(0xffffffffu, b, off);
  }
  if ((threadIdx.x & 31) == 0) {
    sh.red[2 * (threadIdx.x >> 5)] = a;
    sh.red[2 * (threadIdx.x >> 5) + 1] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int w = 0; w < NT / 32; ++w) {
      s0 += sh.red[2 * w];
      s1 += sh.red[2 * w + 1];
    }
    sh.slot[k][0] = s0;
    sh.slot[k][1] = s1;
  }
  group_sync<CS>();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    if constexpr (CS > 1) {
      for (uint32_t r = 0; r < (uint32_t)CS; ++r) {
        s0 += dsmem_ld(&sh.slot[k][0], r);
        s1 += dsmem_ld(&sh.slot[k][1], r);
      }
    } else {
      s0 = sh.slot[k][0];
      s1 = sh.slot[k][1];
    }
    sh.bc[0] = s0;
    sh.bc[1] = s1;
  }
  __syncthreads();
  a = sh.bc[0];
  b = sh.bc[1];
  k ^= 1;
}

__device__ __forceinline__ void row_ijk3(int r, int m, int& i, int& j, int& k) {
  const uint32_t ru = (uint32_t)r, t = ru / (uint32_t)m;
  i = (int)(ru - t * (uint32_t)m);
  k = (int)(t / (uint32_t)m);
  j = (int)(t - (uint32_t)k * (uint32_t)m);
}

constexpr int kBZ = 8;  // k-planes a thread marches per tile
constexpr int kU = 4;   // rows a thread keeps in flight in the vector phases

// q = A p over one tile of one problem, FP32 class sums: the thread's (i, j) column, planes
// kz0 .. kz0 + kBZ, the x- and kappa-planes around the node kept in registers (per row 9 x
// and 4 kappa loads, 49 FP32 operations). kap: FP32 cells with row stride c1 = n rounded up
// to 4. Plain loads: p and kap are rewritten inside the launch (no read-only cache path).
// Returns the thread's p.q over its rows.
template <int NT>
__device__ __forceinline__ float march_tile(int n, int c1, int bx, int by, int kz0,
                                            const float* kap, const float* p, float* q,
                                            const float* W) {
  const int m = n - 1;
  const int i = bx * 32 + (int)(threadIdx.x & 31);
  const int j = by * (NT / 32) + (int)(threadIdx.x >> 5);
  float pq = 0.f;
  if (i >= m || j >= m) return pq;
  const bool okx[3] = {i > 0, true, i < m - 1};
  const bool oky[3] = {j > 0, true, j < m - 1};
  const int64_t col = (int64_t)i + (int64_t)m * j, sz = (int64_t)m * m;
  const int64_t c2 = (int64_t)c1 * n;
  const float* kcol = kap + ((int64_t)i + (int64_t)c1 * j);
  auto xplane = [&](int kk, float* v) {
    const bool okz = kk >= 0 && kk < m;
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx) {
        float t = 0.f;
        if (okz && okx[dx + 1] && oky[dy + 1]) t = p[col + sz * kk + dx + (int64_t)m * dy];
        v[(dx + 1) + 3 * (dy + 1)] = t;
      }
  };
  auto layer = [&](int kk, float* L) {
    const float* kc = kcol + c2 * kk;
    const float v0 = kc[0], v1 = kc[1], v2 = kc[c1], v3 = kc[c1 + 1];
    const float X0 = v0 + v1, X1 = v2 + v3;
    L[0] = v0;
    L[1] = X0;
    L[2] = v1;
    L[3] = v0 + v2;
    L[4] = X0 + X1;
    L[5] = v1 + v3;
    L[6] = v2;
    L[7] = X1;
    L[8] = v3;
  };
  float xa[9], xb[9], xc[9], la[9], lb[9];
  xplane(kz0 - 1, xa);
  xplane(kz0, xb);
  layer(kz0, la);
#pragma unroll 1
  for (int t = 0; t < kBZ; ++t) {
    const int k = kz0 + t;
    if (k >= m) break;
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
    q[col + sz * k] = acc;
    pq = fmaf(xb[4], acc, pq);
#pragma unroll
    for (int e = 0; e < 9; ++e) {
      xa[e] = xb[e];
      xb[e] = xc[e];
      la[e] = lb[e];
    }
  }
  return pq;
}

// One problem solved by a group of CS CTAs (a cluster; CS = 1: one CTA): the operator phase
// splits the problem's tiles between the group's CTAs (tile t to rank t mod CS), the vector
// phases its rows (contiguous ranges). Every branch depends only on group-wide sums, which
// all CTAs form in the same order, so all CTAs of a group take the same path through the
// same barriers. base: the group's scratch (kap32 | d | x | r | p | q).
template <int NT, int CS>
__device__ __forceinline__ void solve_one(const PArgs& a, BShared<NT>& sh, int& slot,
                                          uint32_t rank, float* base, int pi) {
  const int tid = threadIdx.x;
  float* kap32 = base;
  float* dv = kap32 + a.cell_stride;
  float* x32 = dv + a.row_stride;
  float* r32 = x32 + a.row_stride;
  float* p32 = r32 + a.row_stride;
  float* q32 = p32 + a.row_stride;
  const float* W = a.W32;  // kernel parameter space, read through the constant cache
  const BProb P = a.probs[pi];
  const int n = P.n, m = n - 1;
  const int c1 = (n + 3) & ~3;
  const int R = m * m * m;  // < 2^31 (n <= 1024)
  const double* kap = a.coef + P.cell0;
  double* x64 = a.x + P.xoff;
  const int r0 = (int)((int64_t)R * rank / CS), r1 = (int)((int64_t)R * (rank + 1) / CS);
  const int tx = (m + 31) / 32, ty = (m + NT / 32 - 1) / (NT / 32), tz = (m + kBZ - 1) / kBZ;
  const int ntile = tx * ty * tz;
  int iters = 0, converged = 0;
  if (R > 0) {
    // set-up: FP32 kappa (this CTA's cell layers), Jacobi diagonal, x = 0, r = b = f,
    // p = D^-1 r
    const int64_t nlay = (int64_t)n * n;
    for (int64_t c = (int64_t)rank * nlay * n / CS + tid;
         c < ((int64_t)rank + 1) * nlay * n / CS; c += NT) {
      const int64_t ck = c / nlay, rest = c - ck * nlay, cj = rest / n, ci = rest - cj * n;
      kap32[ci + (int64_t)c1 * (cj + (int64_t)n * ck)] = (float)kap[c];
    }
    double rz = 0.0, bb = 0.0;
    const float fb = (float)a.f;
    for (int r = r0 + tid; r < r1; r += NT) {
      int i, j, k;
      row_ijk3(r, m, i, j, k);
      float ks = 0.f;
#pragma unroll
      for (int e = 0; e < 8; ++e)
        ks += (float)kap[(i + (e & 1)) + (int64_t)n * ((j + ((e >> 1) & 1)) +
                                                        (int64_t)n * (k + (e >> 2)))];
      const float d = 1.f / (W[0] * ks);
      dv[r] = d;
      x64[r] = 0.0;
      x32[r] = 0.f;
      r32[r] = fb;
      p32[r] = d * fb;
      rz += (double)fb * (double)(d * fb);
      bb += a.f * a.f;
    }
    group_sum2<NT, CS>(rz, bb, sh, slot);  // also publishes kap32 and p32 to the cluster
    const double tol2 = a.rtol2 * bb;
    double rmax2 = bb;
    bool done = !(bb > 0.0);
    converged = done;
    while (!done) {
      // q = A p over this CTA's tiles; p.q
      double pq = 0.0, unused = 0.0;
      for (int t = (int)rank; t < ntile; t += CS) {
        const int bx = t % tx, by = (t / tx) % ty, bz = t / (tx * ty);
        pq += (double)march_tile<NT>(n, c1, bx, by, bz * kBZ, kap32, p32, q32, W);
      }
      group_sum2<NT, CS>(pq, unused, sh, slot);
      const float alpha = (float)(rz / pq);
      // x += alpha p, r -= alpha q over this CTA's rows; r.z and r.r
      double rzn = 0.0, rr = 0.0;
      for (int base = r0 + tid; base < r1; base += kU * NT) {
        // kU rows a thread: all loads issued before the first use
        float xv[kU], pv[kU], qv[kU], rv[kU], dd[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int r = base + u * NT;
          if (r < r1) {
            xv[u] = x32[r];
            pv[u] = p32[r];
            qv[u] = q32[r];
            rv[u] = r32[r];
            dd[u] = dv[r];
          }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int r = base + u * NT;
          if (r < r1) {
            x32[r] = fmaf(alpha, pv[u], xv[u]);
            const float ri = fmaf(-alpha, qv[u], rv[u]);
            r32[r] = ri;
            rzn += (double)ri * (double)(dd[u] * ri);
            rr += (double)ri * ri;
          }
        }
      }
      group_sum2<NT, CS>(rzn, rr, sh, slot);
      ++iters;
      if (!isfinite(rr) || !isfinite(rzn) || !isfinite(pq)) {
        if (tid == 0 && rank == 0 && atomicCAS(&a.err->code, 0, GFE_ERR_NONFINITE) == 0)
          a.err->index = pi;
        break;
      }
      if (rr <= (double)kDelta * kDelta * rmax2 || rr <= tol2 || iters >= a.maxit) {
        // reliable update: x64 += x32, then r = b - A x64 in FP64 from the FP64 kappa
        for (int base = r0 + tid; base < r1; base += kU * NT) {
          double xv[kU];
          float xs[kU];
#pragma unroll
          for (int u = 0; u < kU; ++u) {
            const int r = base + u * NT;
            if (r < r1) {
              xv[u] = x64[r];
              xs[u] = x32[r];
            }
          }
#pragma unroll
          for (int u = 0; u < kU; ++u) {
            const int r = base + u * NT;
            if (r < r1) {
              x64[r] = xv[u] + (double)xs[u];
              x32[r] = 0.f;
            }
          }
        }
        group_sync<CS>();
        double rr64 = 0.0;
        rzn = 0.0;
        for (int r = r0 + tid; r < r1; r += NT) {
          int i, j, k;
          row_ijk3(r, m, i, j, k);
          const double res = a.f - class_apply<double>(i, j, k, m, n, kap, x64, a.W64);
          const float rf = (float)res;
          r32[r] = rf;
          rr64 += res * res;
          rzn += (double)rf * (double)(dv[r] * rf);
        }
        group_sum2<NT, CS>(rr64, rzn, sh, slot);
        rmax2 = rr64;
        if (rr64 <= tol2) {
          converged = 1;
          break;
        }
        if (iters >= a.maxit) break;
      }
      const float beta = (float)(rzn / rz);
      rz = rzn;
      for (int base = r0 + tid; base < r1; base += kU * NT) {
        float pv[kU], dd[kU], rv[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int r = base + u * NT;
          if (r < r1) {
            pv[u] = p32[r];
            dd[u] = dv[r];
            rv[u] = r32[r];
          }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int r = base + u * NT;
          if (r < r1) p32[r] = fmaf(beta, pv[u], dd[u] * rv[u]);
        }
      }
      group_sync<CS>();
    }
  } else {
    converged = 1;
  }
  if (tid == 0 && rank == 0) {
    a.iters[pi] = iters;
    a.conv[pi] = converged;
  }
  // the next problem's set-up rewrites this group's scratch, which peers may still read
  group_sync<CS>();
}

// The solve of every problem in one launch. Phase 1: each cluster of CS CTAs takes the large
// problems (order[0 .. nlarge)) from the first work counter and solves them together. Phase
// 2 (once that counter is exhausted for the cluster): every CTA takes the small problems
// from the second counter and solves each alone, with CTA barriers only. A cluster leaves
// phase 1 together (the task is broadcast) and its CTAs touch no peer's shared memory after
// that, so none waits on another CTA in phase 2.
template <int NT, int CS>
__global__ void __launch_bounds__(NT, (1024 / NT > 0 ? 1024 / NT : 1))
    k_b_solve(const __grid_constant__ PArgs a) {
  __shared__ BShared<NT> sh;
  const int tid = threadIdx.x;
  const uint32_t rank = CS > 1 ? cluster_rank() : 0u;
  const int64_t stride = a.cell_stride + 5 * a.row_stride;
  int slot = 0;
  float* gbase = a.scratch + ((int64_t)blockIdx.x - rank) * stride;
  for (;;) {
    if (tid == 0 && rank == 0) sh.task = atomicAdd(a.counter, 1);
    group_sync<CS>();
    int task;
    if constexpr (CS > 1) {
      if (tid == 0) {
        const uint32_t local = (uint32_t)__cvta_generic_to_shared(&sh.task);
        uint32_t remote;
        int v;
        asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(0));
        asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(remote) : "memory");
        sh.bc[0] = (double)v;
      }
      __syncthreads();
      task = (int)sh.bc[0];
      group_sync<CS>();  // rank 0 rewrites its task only after every CTA has read it
    } else {
      task = sh.task;
      __syncthreads();
    }
    if (task >= a.nlarge) break;
    solve_one<NT, CS>(a, sh, slot, rank, gbase, a.order[task]);
  }
  if constexpr (CS > 1) {
    float* cbase = a.scratch + (int64_t)blockIdx.x * stride;
    for (;;) {
      if (tid == 0) sh.task = atomicAdd(a.counter2, 1);
      __syncthreads();
      const int task = a.nlarge + sh.task;
      __syncthreads();
      if (task >= a.nproblems) break;
      solve_one<NT, 1>(a, sh, slot, 0u, cbase, a.order[task]);
    }
  }
}

}  // namespace batch
}  // namespace gfe

struct gfe_batch {
  gfe_ctx* ctx = nullptr;
  int32_t nproblems = 0;
  int64_t ncells = 0, nfree_total = 0;
  int64_t cell_stride = 0, row_stride = 0;  // per-block scratch: largest problem, rounded to 32
  std::vector<int64_t> nfree;               // per problem
  std::vector<int64_t> nfree_sorted;        // the same, largest first
  int64_t rmax = 0;                         // the largest problem's rows
  gfe::DevBuf coef, probs, order, counter, status, xbuf, scratch;
  int nt = 0, cs = 0;                       // tuned threads per CTA and CTAs per problem
  float large = 0.f;                        // and the cluster threshold (relative rows)
  double W64[8] = {0};
  float W32[8] = {0};
};

namespace gfe {

// the schedules the autotuner times: threads per CTA, CTAs per problem (cluster size) and the
// row count, relative to the largest problem's, from which a problem goes to a cluster (the
// smaller ones go to single CTAs once the clusters have run out of large problems; 0: every
// problem to a cluster)
struct Schedule {
  int nt, cs;
  float large;
};
static const Schedule kShapes[] = {{256, 1, 0.f},  {1024, 1, 0.f},  {1024, 2, 0.f},
                                   {512, 4, 0.f},  {512, 4, 0.3f},  {1024, 4, 0.3f},
                                   {1024, 8, 0.f}, {1024, 8, 0.3f}};
constexpr int kNumShapes = (int)(sizeof(kShapes) / sizeof(kShapes[0]));
constexpr size_t kScratchCap = (size_t)8 << 30;  // scratch bytes the launch may hold at most

template <int NT, int CS>
static int launch_shape(gfe_ctx* ctx, const batch::PArgs& a, int64_t groups, bool query,
                        int64_t* max_groups) {
  auto kern = batch::k_b_solve<NT, CS>;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = ctx->stream;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (query) {
    int occ = 0;
    if (CS > 1) {
      cfg.gridDim = dim3((unsigned)(ctx->num_sms / CS * CS));
      if (cudaOccupancyMaxActiveClusters(&occ, kern, &cfg) != cudaSuccess) occ = 0;
    } else {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, NT, 0) != cudaSuccess)
        occ = 0;
      occ *= ctx->num_sms;
    }
    cudaGetLastError();
    *max_groups = occ;
    return GFE_OK;
  }
  cfg.gridDim = dim3((unsigned)(groups * CS));
  GFE_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, a));
  return GFE_OK;
}

static int dispatch_shape(gfe_ctx* ctx, int s, const batch::PArgs& a, int64_t groups,
                          bool query, int64_t* max_groups) {
  const int nt = kShapes[s].nt, cs = kShapes[s].cs;
  if (nt == 256 && cs == 1) return launch_shape<256, 1>(ctx, a, groups, query, max_groups);
  if (nt == 1024 && cs == 1) return launch_shape<1024, 1>(ctx, a, groups, query, max_groups);
  if (nt == 1024 && cs == 2) return launch_shape<1024, 2>(ctx, a, groups, query, max_groups);
  if (nt == 512 && cs == 4) return launch_shape<512, 4>(ctx, a, groups, query, max_groups);
  if (nt == 1024 && cs == 4) return launch_shape<1024, 4>(ctx, a, groups, query, max_groups);
  return launch_shape<1024, 8>(ctx, a, groups, query, max_groups);
}

// problem groups (CTAs, or clusters) of one launch of schedule s: as many as can be
// resident, at most one per problem and within the scratch cap (scratch is per CTA); 0 if the
// schedule cannot run here
static int64_t batch_groups(gfe_ctx* ctx, const gfe_batch* B, int s) {
  int64_t res = 0;
  batch::PArgs dummy{};
  dispatch_shape(ctx, s, dummy, 0, true, &res);
  if (res < 1) return 0;
  const int64_t grp_bytes =
      (int64_t)sizeof(float) * (B->cell_stride + 5 * B->row_stride) * kShapes[s].cs;
  const int64_t cap =
      std::max<int64_t>(1, (int64_t)(kScratchCap / (size_t)std::max<int64_t>(grp_bytes, 1)));
  return std::max<int64_t>(1, std::min<int64_t>({res, (int64_t)B->nproblems, cap}));
}

// problems that schedule s gives to clusters: a prefix of the largest-first order
static int32_t batch_nlarge(const gfe_batch* B, int s) {
  if (kShapes[s].cs == 1 || !(kShapes[s].large > 0.f)) return B->nproblems;
  const double t = (double)kShapes[s].large * (double)B->rmax;
  int32_t k = 0;
  while (k < B->nproblems && (double)B->nfree_sorted[k] >= t) ++k;
  return k;
}

// One launch solving every problem with schedule s into x (device, nfree_total entries).
static int batch_launch(gfe_ctx* ctx, gfe_batch* B, int s, double source, double rtol,
                        int32_t maxit, double* x) {
  using namespace batch;
  const int64_t groups = batch_groups(ctx, B, s);
  if (groups < 1)
    return set_error(GFE_ERR_UNSUPPORTED, "batch: launch schedule %d cannot run", s);
  GFE_TRY(B->scratch.reserve(sizeof(float) * (size_t)(groups * kShapes[s].cs) *
                             (size_t)(B->cell_stride + 5 * B->row_stride)));
  GFE_CUDA_TRY(cudaMemsetAsync(B->counter.ptr, 0, 2 * sizeof(int), ctx->stream));
  PArgs a;
  a.nproblems = B->nproblems;
  a.probs = B->probs.as<BProb>();
  a.order = B->order.as<int32_t>();
  a.counter = B->counter.as<int>();
  a.counter2 = a.counter + 1;
  a.nlarge = batch_nlarge(B, s);
  a.coef = B->coef.as<double>();
  a.f = source;
  a.rtol2 = rtol * rtol;
  a.maxit = maxit;
  a.scratch = B->scratch.as<float>();
  a.cell_stride = B->cell_stride;
  a.row_stride = B->row_stride;
  a.x = x;
  a.iters = B->status.as<int32_t>();
  a.conv = a.iters + B->nproblems;
  a.err = ctx->d_err;
  for (int c = 0; c < 8; ++c) {
    a.W64[c] = B->W64[c];
    a.W32[c] = B->W32[c];
  }
  int64_t unused = 0;
  GFE_TRY(dispatch_shape(ctx, s, a, groups, false, &unused));
  ctx->launches++;
  return GFE_OK;
}

}  // namespace gfe

using namespace gfe;

extern "C" int gfe_batch_create(gfe_ctx* ctx, int32_t nproblems, const int64_t* partitions,
                                const double* kappa, gfe_batch** out) {
  clear_error();
  if (!ctx || nproblems < 1 || !partitions || !kappa || !out)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_batch_create: bad arguments");
  std::vector<batch::BProb> probs(nproblems);
  std::vector<int64_t> nfree(nproblems);
  int64_t cells = 0, nf_total = 0, cmax = 0, rmax = 0;
  for (int32_t p = 0; p < nproblems; ++p) {
    const int64_t nx = partitions[3 * p], ny = partitions[3 * p + 1], nz = partitions[3 * p + 2];
    if (nx < 1 || ny < 1 || nz < 1)
      return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_batch_create: partition of problem %d",
                       (int)p);
    if (nx != ny || ny != nz)  // the unit-cell tables assume cubic cells
      return set_error(GFE_ERR_UNSUPPORTED,
                       "gfe_batch_create: problem %d: partition must be (n, n, n)", (int)p);
    if (nx > 1024)
      return set_error(GFE_ERR_UNSUPPORTED,
                       "gfe_batch_create: problem %d: n = %lld above 1024 (solve it alone)",
                       (int)p, (long long)nx);
    const int64_t nf = (nx - 1) * (nx - 1) * (nx - 1), nc = nx * nx * nx;
    probs[p].n = (int32_t)nx;
    probs[p].pad = 0;
    probs[p].cell0 = cells;
    probs[p].xoff = nf_total;
    nfree[p] = nf;
    cells += nc;
    nf_total += nf;
    cmax = std::max(cmax, ((nx + 3) & ~3) * nx * nx);  // FP32 copy: rows padded to 4
    rmax = std::max(rmax, nf);
  }
  // kappa / h^2 per cell (the equations divided by h^3)
  std::vector<double> coef((size_t)cells);
  for (int32_t p = 0; p < nproblems; ++p) {
    const double inv_h2 = (double)probs[p].n * (double)probs[p].n;
    const int64_t nc = (int64_t)probs[p].n * probs[p].n * probs[p].n;
    for (int64_t c = 0; c < nc; ++c)
      coef[probs[p].cell0 + c] = kappa[probs[p].cell0 + c] * inv_h2;
  }
  // largest problems first: the last problems to start are the short ones
  std::vector<int32_t> order(nproblems);
  for (int32_t p = 0; p < nproblems; ++p) order[p] = p;
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b) { return nfree[a] > nfree[b]; });
  gfe_batch* B = new gfe_batch();
  B->ctx = ctx;
  B->nproblems = nproblems;
  B->ncells = cells;
  B->nfree_total = nf_total;
  B->nfree = nfree;
  B->rmax = rmax;
  for (int32_t p = 0; p < nproblems; ++p) B->nfree_sorted.push_back(nfree[order[p]]);
  B->cell_stride = (cmax + 31) / 32 * 32;
  B->row_stride = (rmax + 31) / 32 * 32;
  q1_unit_stiffness_classes(B->W64);
  for (int c = 0; c < 8; ++c) B->W32[c] = (float)B->W64[c];
  for (DevBuf* d : {&B->coef, &B->probs, &B->order, &B->counter, &B->status, &B->xbuf,
                    &B->scratch})
    d->owner = ctx;
  int st = GFE_OK;
  auto up = [&](DevBuf& d, const void* src, size_t nb) {
    if (st != GFE_OK) return;
    st = d.reserve(nb);
    if (st == GFE_OK &&
        cudaMemcpyAsync(d.ptr, src, nb, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
      st = set_error(GFE_ERR_CUDA, "gfe_batch_create: copy failed");
  };
  up(B->coef, coef.data(), coef.size() * sizeof(double));
  up(B->probs, probs.data(), probs.size() * sizeof(batch::BProb));
  up(B->order, order.data(), order.size() * sizeof(int32_t));
  if (st == GFE_OK) st = B->counter.reserve(2 * sizeof(int));
  if (st == GFE_OK) st = B->status.reserve(sizeof(int32_t) * 2 * (size_t)nproblems);
  if (st == GFE_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    st = set_error(GFE_ERR_CUDA, "gfe_batch_create: sync failed");
  if (st != GFE_OK) {
    delete B;
    return st;
  }
  *out = B;
  return GFE_OK;
}

extern "C" int gfe_batch_destroy(gfe_batch* B) {
  if (!B) return GFE_OK;
  delete B;
  return GFE_OK;
}

extern "C" int gfe_batch_info(gfe_batch* B, int64_t* nrows, int64_t* nfree, int64_t* ncells) {
  clear_error();
  if (!B) return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_batch_info: NULL");
  if (nrows) *nrows = B->nfree_total;
  if (nfree) *nfree = B->nfree_total;
  if (ncells) *ncells = B->ncells;
  return GFE_OK;
}

extern "C" int gfe_batch_shape(gfe_batch* B, int32_t* threads, int32_t* ctas_per_problem,
                               double* cluster_threshold) {
  clear_error();
  if (!B) return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_batch_shape: NULL");
  if (threads) *threads = B->nt;
  if (ctas_per_problem) *ctas_per_problem = B->cs;
  if (cluster_threshold) *cluster_threshold = B->large;
  return GFE_OK;
}

// Fixes the launch schedule (one of the autotuner's candidates) instead of tuning it; (0, 0)
// re-enables the autotuner. Schedules sum in different orders, so fixing one makes results
// reproducible across batches.
extern "C" int gfe_batch_set_shape(gfe_batch* B, int32_t threads, int32_t ctas_per_problem,
                                   double cluster_threshold) {
  clear_error();
  if (!B) return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_batch_set_shape: NULL");
  if (threads == 0 && ctas_per_problem == 0) {
    B->nt = B->cs = 0;
    B->large = 0.f;
    return GFE_OK;
  }
  for (int s = 0; s < kNumShapes; ++s)
    if (kShapes[s].nt == threads && kShapes[s].cs == ctas_per_problem &&
        std::fabs((double)kShapes[s].large - cluster_threshold) < 1e-6) {
      if (batch_groups(B->ctx, B, s) < 1)
        return set_error(GFE_ERR_UNSUPPORTED, "gfe_batch_set_shape: (%d, %d) cannot run on "
                         "this device", (int)threads, (int)ctas_per_problem);
      B->nt = threads;
      B->cs = ctas_per_problem;
      B->large = kShapes[s].large;
      return GFE_OK;
    }
  return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_batch_set_shape: (%d, %d, %g) is not a "
                   "candidate schedule", (int)threads, (int)ctas_per_problem, cluster_threshold);
}

// Assembles and solves every problem (one persistent launch; see the file comment). x (host
// or device memory of the context's device) receives the free-dof solutions of the problems
// one after the other (nfree_total entries). iterations[nproblems] (optional, host) gets each
// problem's iteration count; *nconverged the number of problems that reached rtol.
extern "C" int gfe_batch_assemble_solve(gfe_batch* B, double source, double rtol,
                                        int32_t maxiter, double* x, int32_t* iterations,
                                        int32_t* nconverged) {
  gfe::NvtxRange nvtx_range("gfe_batch_assemble_solve");
  clear_error();
  if (!B || !x || !(rtol > 0.0) || !std::isfinite(source))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_batch_assemble_solve: bad arguments");
  gfe_ctx* ctx = B->ctx;
  const int32_t maxit = maxiter > 0 ? maxiter : 100000;
  cudaPointerAttributes pa;
  const bool xdev = cudaPointerGetAttributes(&pa, x) == cudaSuccess &&
                    pa.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  if (xdev && pa.device != ctx->device)
    return set_error(GFE_ERR_INVALID_ARGUMENT,
                     "gfe_batch_assemble_solve: x lives on device %d, the context on %d",
                     pa.device, ctx->device);
  double* xd = x;
  if (!xdev) {
    GFE_TRY(B->xbuf.reserve(sizeof(double) * (size_t)std::max<int64_t>(B->nfree_total, 1)));
    xd = B->xbuf.as<double>();
  }
  // autotune once per batch: every shape that can run here on the full solve (a capped one
  // balances the work differently), the fastest kept
  if (B->nt == 0) {
    cudaEvent_t ev[kNumShapes + 1];
    for (auto& e : ev) cudaEventCreate(&e);
    int st = GFE_OK;
    bool ran[kNumShapes] = {false};
    cudaEventRecord(ev[0], ctx->stream);
    for (int s = 0; s < kNumShapes && st == GFE_OK; ++s) {
      if (batch_groups(ctx, B, s) >= 1) {
        st = batch_launch(ctx, B, s, source, rtol, maxit, xd);
        ran[s] = st == GFE_OK;
      }
      cudaEventRecord(ev[s + 1], ctx->stream);
    }
    int best = -1;
    float tbest = 0.f;
    if (st == GFE_OK && cudaEventSynchronize(ev[kNumShapes]) == cudaSuccess) {
      for (int s = 0; s < kNumShapes; ++s) {
        float t = 0.f;
        if (!ran[s] || cudaEventElapsedTime(&t, ev[s], ev[s + 1]) != cudaSuccess) continue;
        if (best < 0 || t < tbest) {
          tbest = t;
          best = s;
        }
      }
    } else if (st == GFE_OK) {
      st = set_error(GFE_ERR_CUDA, "gfe_batch_assemble_solve: autotune failed");
    }
    for (auto& e : ev) cudaEventDestroy(e);
    GFE_TRY(st);
    if (best < 0) return set_error(GFE_ERR_UNSUPPORTED, "gfe_batch_assemble_solve: no launch "
                                   "shape can run on this device");
    B->nt = kShapes[best].nt;
    B->cs = kShapes[best].cs;
    B->large = kShapes[best].large;
  }
  int s = 0;
  while (s < kNumShapes && !(kShapes[s].nt == B->nt && kShapes[s].cs == B->cs &&
                             kShapes[s].large == B->large))
    ++s;
  GFE_TRY(batch_launch(ctx, B, s, source, rtol, maxit, xd));
  // results: per-problem iterations and convergence, x to the caller's host array
  int32_t* hs = (int32_t*)ctx->h_pinned;
  const size_t sbytes = sizeof(int32_t) * 2 * (size_t)B->nproblems;
  std::vector<int32_t> big;
  if (sbytes > 4096) {  // the context's pinned staging block
    big.resize(2 * (size_t)B->nproblems);
    hs = big.data();
  }
  GFE_CUDA_TRY(cudaMemcpyAsync(hs, B->status.ptr, sbytes, cudaMemcpyDeviceToHost, ctx->stream));
  if (!xdev)
    GFE_CUDA_TRY(cudaMemcpyAsync(x, xd, sizeof(double) * (size_t)B->nfree_total,
                                 cudaMemcpyDeviceToHost, ctx->stream));
  GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  int32_t nconv = 0;
  for (int32_t pi = 0; pi < B->nproblems; ++pi) {
    if (iterations) iterations[pi] = hs[pi];
    nconv += hs[B->nproblems + pi];
  }
  if (nconverged) *nconverged = nconv;
  return check_device_error(ctx, "gfe_batch_assemble_solve");
}
