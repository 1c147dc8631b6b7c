// gfe_pmg.cu -- p-multigrid preconditioner for 3-D Q2 diffusion on Cartesian hexahedra (node
// coordinates possibly jittered): the Q2 level is smoothed with damped Jacobi on the assembled
// FP32 matrix (sliced ELL), and its residual goes to the Q1 space of the same cells, which the
// geometric multigrid V-cycle of gfe_mg.cu solves approximately on the lattice operator of the
// uniform grid. Gridap has no multigrid; this is a LinearSolver plug-in preconditioner.
//
// Transfers. A Q1 function is a Q2 function (Q1 is a subspace of Q2 on the same cells, and
// both interpolate in reference coordinates), so the prolongation P: Q1 -> Q2 is exact: the
// Q2 nodes of a cell form a 3x3x3 lattice in reference coordinates, and the nodes of the whole
// grid the (2 n0 + 1) x (2 n1 + 1) x (2 n2 + 1) lattice, on which a Q1 vertex is every other
// point. The value of a Q1 function at a Q2 node is then the trilinear interpolation of its
// vertex values: weight 1 at even lattice positions, 1/2 per odd coordinate. R = P^T sums the
// 27 Q2 nodes around a vertex with weights prod (1 - |delta| / 2). Both are stencils on the Q2
// node lattice, read through a lattice -> free dof map built once from the cell ids.
//
// The coarse operator is the Q1 stiffness of the uniform grid with the problem's kappa (for
// jittered nodes the exact Galerkin product P^T A P is the Q1 stiffness of the jittered cells;
// the uniform one is spectrally equivalent within the jitter's distortion, and the flexible
// CG absorbs the difference). The coarse free dofs are the interior vertices in node order,
// the numbering Gridap's conforming Q2 spaces give vertex dofs when every boundary node is
// Dirichlet; the attach step checks this on the device.
//
// One V-cycle (pre: the sweep from zero fused with the next; post: two sweeps):
//   x = S0(b);  r = b - A x;  b_c = R r;  x_c = MG(b_c);  x += P x_c;  x = S(S(x)).
#include <cmath>

#include "gfe_internal.h"

namespace gfe {
#include "gfe_lattice.cuh"
#include "gfe_sell.cuh"

namespace {

constexpr int kPmgBlock = 256;
constexpr float kPmgOmega = 0.6f;  // damped Jacobi on Q2: max eigenvalue of D^-1 A near 3

struct NodeIdx {
  int v[27 * 3];  // lattice position (0, 1, 2 per direction) of each local Q2 node
};

__device__ __forceinline__ bool stop_p(const int* done) { return done && *done; }

// Q2 node lattice -> free dof (0-based, -1 Dirichlet), and the check that the vertex dofs are
// the interior vertices in node order.
__global__ void k_q2_node_map(int64_t ncells, const int32_t* __restrict__ ids, int n0, int n1,
                              int n2, NodeIdx idx, int32_t* __restrict__ map, int* bad) {
  const int64_t L0 = 2 * (int64_t)n0 + 1, L1 = 2 * (int64_t)n1 + 1;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ncells * 27;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / 27;
    const int a = (int)(t - c * 27);
    const int ci = (int)(c % n0), cj = (int)((c / n0) % n1), ck = (int)(c / ((int64_t)n0 * n1));
    const int px = 2 * ci + idx.v[3 * a], py = 2 * cj + idx.v[3 * a + 1],
              pz = 2 * ck + idx.v[3 * a + 2];
    const int32_t id = ids[t];
    map[px + L0 * (py + L1 * pz)] = id > 0 ? id - 1 : -1;
    if (a < 8) {  // a vertex: (px/2, py/2, pz/2) on the vertex lattice
      const int i = px / 2, j = py / 2, k = pz / 2;
      const bool interior = i > 0 && j > 0 && k > 0 && i < n0 && j < n1 && k < n2;
      const int64_t want = 1 + (i - 1) + (int64_t)(n0 - 1) * ((j - 1) + (int64_t)(n1 - 1) * (k - 1));
      if (interior ? (int64_t)id != want : id > 0) atomicExch(bad, 1);
    }
  }
}

__global__ void k_pmg_kappa(const double* __restrict__ c, int kind, int64_t n0, int64_t c1,
                            int64_t n, float* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[(i % n0) + c1 * (i / n0)] =
        kind == GFE_COEF_CELL ? (float)c[i] : kind == GFE_COEF_CONST ? (float)c[0] : 1.f;
}

struct SellF {
  const int64_t* sptr;
  const int32_t* scol;
  const float* sval;
};

// x1 = x0 + omega D^-1 (b - A x0),  x0 = omega D^-1 b formed on the fly
__global__ void __launch_bounds__(kPmgBlock)
    k_pmg_pre(int64_t n, SellF A, const float* __restrict__ b, const float* __restrict__ dinv,
              float* __restrict__ x1, const int* done) {
  if (stop_p(done)) return;
  const int64_t r = (int64_t)blockIdx.x * kPmgBlock + threadIdx.x;
  if (r >= n) return;
  auto x0 = [&](int32_t c) { return kPmgOmega * __ldg(dinv + c) * __ldg(b + c); };
  const float acc = sell_row_f(r, A.sptr, A.scol, A.sval, x0);
  x1[r] = fmaf(kPmgOmega * __ldg(dinv + r), __ldg(b + r) - acc, x0((int32_t)r));
}

// xo = x + omega D^-1 (b - A x)
__global__ void __launch_bounds__(kPmgBlock)
    k_pmg_smooth(int64_t n, SellF A, const float* __restrict__ x, const float* __restrict__ b,
                 const float* __restrict__ dinv, float* __restrict__ xo, const int* done) {
  if (stop_p(done)) return;
  const int64_t r = (int64_t)blockIdx.x * kPmgBlock + threadIdx.x;
  if (r >= n) return;
  const float acc = sell_row<float, float>(r, A.sptr, A.scol, A.sval, x);
  xo[r] = fmaf(kPmgOmega * __ldg(dinv + r), __ldg(b + r) - acc, __ldg(x + r));
}

// res = b - A x
__global__ void __launch_bounds__(kPmgBlock)
    k_pmg_residual(int64_t n, SellF A, const float* __restrict__ x, const float* __restrict__ b,
                   float* __restrict__ res, const int* done) {
  if (stop_p(done)) return;
  const int64_t r = (int64_t)blockIdx.x * kPmgBlock + threadIdx.x;
  if (r >= n) return;
  res[r] = __ldg(b + r) - sell_row<float, float>(r, A.sptr, A.scol, A.sval, x);
}

// b_c = R r: coarse interior vertex (I, J, K) at Q2 lattice (2I+2, 2J+2, 2K+2), the 27 lattice
// nodes around it with weights prod (1 - |delta| / 2)
__global__ void k_pmg_restrict(int n0, int n1, int n2, const int32_t* __restrict__ map,
                               const float* __restrict__ r, float* __restrict__ bc,
                               const int* done) {
  if (stop_p(done)) return;
  const int m0 = n0 - 1, m1 = n1 - 1, m2 = n2 - 1;
  const int64_t L0 = 2 * (int64_t)n0 + 1, L1 = 2 * (int64_t)n1 + 1;
  const int64_t nc = (int64_t)m0 * m1 * m2;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nc;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int I = (int)(q % m0), J = (int)((q / m0) % m1), K = (int)(q / ((int64_t)m0 * m1));
    const int px = 2 * I + 2, py = 2 * J + 2, pz = 2 * K + 2;
    float s = 0.f;
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
          const int32_t d = __ldg(map + (px + dx) + L0 * ((py + dy) + L1 * (pz + dz)));
          if (d >= 0) {
            const float w = (dx ? 0.5f : 1.f) * (dy ? 0.5f : 1.f) * (dz ? 0.5f : 1.f);
            s = fmaf(w, __ldg(r + d), s);
          }
        }
    bc[q] = s;
  }
}

// x += P x_c at every free Q2 node: per direction the vertex at p/2 (p even) or the two at
// (p -+ 1)/2 with weight 1/2 (p odd); boundary vertices are Dirichlet (zero)
__global__ void k_pmg_prolong(int n0, int n1, int n2, const int32_t* __restrict__ map,
                              const float* __restrict__ xc, float* __restrict__ x,
                              const int* done) {
  if (stop_p(done)) return;
  const int m0 = n0 - 1, m1 = n1 - 1;
  const int64_t L0 = 2 * (int64_t)n0 + 1, L1 = 2 * (int64_t)n1 + 1;
  const int64_t L = L0 * L1 * (2 * (int64_t)n2 + 1);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < L;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t d = __ldg(map + t);
    if (d < 0) continue;
    const int p[3] = {(int)(t % L0), (int)((t / L0) % L1), (int)(t / (L0 * L1))};
    const int nn[3] = {n0, n1, n2};
    int v[3][2];
    float w[3][2];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if ((p[a] & 1) == 0) {
        v[a][0] = p[a] / 2 - 1;  // coarse interior index of vertex p/2
        w[a][0] = 1.f;
        v[a][1] = -1;
        w[a][1] = 0.f;
      } else {
        v[a][0] = (p[a] - 1) / 2 - 1;
        v[a][1] = (p[a] + 1) / 2 - 1;
        w[a][0] = w[a][1] = 0.5f;
      }
#pragma unroll
      for (int e = 0; e < 2; ++e)
        if (v[a][e] < 0 || v[a][e] >= nn[a] - 1) v[a][e] = -1;
    }
    float s = 0.f;
#pragma unroll
    for (int ez = 0; ez < 2; ++ez)
#pragma unroll
      for (int ey = 0; ey < 2; ++ey)
#pragma unroll
        for (int ex = 0; ex < 2; ++ex)
          if (v[0][ex] >= 0 && v[1][ey] >= 0 && v[2][ez] >= 0)
            s = fmaf(w[0][ex] * w[1][ey] * w[2][ez],
                     __ldg(xc + v[0][ex] + (int64_t)m0 * (v[1][ey] + (int64_t)m1 * v[2][ez])), s);
    x[d] += s;
  }
}

}  // namespace

int attach_q2_pmg(gfe_ctx* ctx, gfe_matrix* A, const gfe_problem* p, const double* d_coef) {
  A->pmg_state = 0;
  const int64_t n0 = p->partition[0], n1 = p->partition[1], n2 = p->partition[2];
  if (p->dim != 3 || p->reffe != GFE_REFFE_Q2 || A->nd != 27 || A->cols_per_cell() != 27 ||
      A->nrows != A->ncols || n0 < 2 || n1 < 2 || n2 < 2 || A->ncells != n0 * n1 * n2 ||
      (2 * n0 + 1) * (2 * n1 + 1) * (2 * n2 + 1) > (int64_t)INT32_MAX)
    return GFE_OK;
  A->pmg_node.owner = A->pmg_kap32.owner = A->pmg_flag.owner = ctx;
  const int64_t L = (2 * n0 + 1) * (2 * n1 + 1) * (2 * n2 + 1);
  GFE_TRY(A->pmg_node.reserve(sizeof(int32_t) * (size_t)L));
  GFE_CUDA_TRY(cudaMemsetAsync(A->pmg_node.ptr, 0xFF, sizeof(int32_t) * (size_t)L, ctx->stream));
  GFE_TRY(A->pmg_flag.reserve(sizeof(int) * 4));
  GFE_CUDA_TRY(cudaMemsetAsync(A->pmg_flag.ptr, 0, sizeof(int), ctx->stream));
  const int64_t c1 = (n0 + 3) & ~(int64_t)3;
  GFE_TRY(A->pmg_kap32.reserve(sizeof(float) * (size_t)(c1 * n1 * n2)));
  GFE_CUDA_TRY(cudaMemsetAsync(A->pmg_kap32.ptr, 0, sizeof(float) * (size_t)(c1 * n1 * n2),
                               ctx->stream));
  NodeIdx idx;
  q2_node_lattice(3, idx.v);
  const int64_t nc = A->ncells;
  k_q2_node_map<<<grid_for(nc * 27, 256, (int64_t)ctx->num_sms * 16), 256, 0, ctx->stream>>>(
      nc, A->cell_rows.as<int32_t>(), (int)n0, (int)n1, (int)n2, idx, A->pmg_node.as<int32_t>(),
      A->pmg_flag.as<int>());
  k_pmg_kappa<<<grid_for(nc, 256, (int64_t)ctx->num_sms * 8), 256, 0, ctx->stream>>>(
      d_coef, d_coef ? p->coef_kind : GFE_COEF_ONE, n0, c1, nc, A->pmg_kap32.as<float>());
  ctx->launches += 2;
  GFE_CUDA_TRY(cudaGetLastError());
  // Q1 reference stiffness of the uniform grid: sum over directions d of the 1-D stiffness
  // (+-1/h_d) times the 1-D masses (h/3 same vertex, h/6 other) of the other directions
  double h[3];
  for (int d = 0; d < 3; ++d) h[d] = (p->domain[2 * d + 1] - p->domain[2 * d]) / (double)p->partition[d];
  for (int a = 0; a < 8; ++a)
    for (int b = 0; b < 8; ++b) {
      double v = 0.0;
      for (int d = 0; d < 3; ++d) {
        double t = (((a >> d) & 1) == ((b >> d) & 1) ? 1.0 : -1.0) / h[d];
        for (int e = 0; e < 3; ++e)
          if (e != d) t *= (((a >> e) & 1) == ((b >> e) & 1)) ? h[e] / 3.0 : h[e] / 6.0;
        v += t;
      }
      A->pmg_K[a + 8 * b] = (float)v;
    }
  A->pmg_n[0] = n0;
  A->pmg_n[1] = n1;
  A->pmg_n[2] = n2;
  A->pmg_state = 1;
  return GFE_OK;
}

int pmg_ready(gfe_ctx* ctx, gfe_matrix* A, bool* ok) {
  if (A->pmg_state == 1) {
    int bad = 1;
    GFE_TRY(copy_out(ctx, &bad, A->pmg_flag.ptr, sizeof(int)));
    A->pmg_state = bad ? 0 : 2;
  }
  *ok = A->pmg_state == 2;
  return GFE_OK;
}

struct Q2PMG {
  gfe_ctx* ctx;
  gfe_matrix* A;
  LatticeMG* coarse = nullptr;
  DevBuf buf;
  float *xf = nullptr, *tf = nullptr, *bc = nullptr, *xc = nullptr;
  cudaGraphExec_t exec = nullptr;
  const float* cap_r = nullptr;
  float* cap_z = nullptr;
  const int* cap_done = nullptr;
  long long nodes = 0;
  explicit Q2PMG(gfe_ctx* c, gfe_matrix* a) : ctx(c), A(a), buf(c) {}
  ~Q2PMG() {
    if (exec) cudaGraphExecDestroy(exec);
    if (coarse) mg_destroy(coarse);
  }
};

int pmg_create(gfe_ctx* ctx, gfe_matrix* A, Q2PMG** out) {
  bool ok = false;
  GFE_TRY(pmg_ready(ctx, A, &ok));
  if (!ok || !A->plan_valid)
    return set_error(GFE_ERR_UNSUPPORTED, "p-multigrid: the matrix has no Q2 lattice data");
  Q2PMG* pm = new Q2PMG(ctx, A);
  *out = pm;
  LatticeQ1Op op;
  op.kap = A->pmg_kap32.as<float>();
  op.n0 = (int)A->pmg_n[0];
  op.n1 = (int)A->pmg_n[1];
  op.n2 = (int)A->pmg_n[2];
  op.s1 = op.n0 - 1;
  op.s2 = (op.n0 - 1) * (op.n1 - 1);
  op.c1 = (op.n0 + 3) & ~3;
  op.c2 = op.c1 * op.n1;
  op.p1 = (op.n0 + 1 + 3) & ~3;
  op.p2 = op.p1 * (op.n1 + 1);
  for (int e = 0; e < 64; ++e) op.K[e] = A->pmg_K[e];
  GFE_TRY(mg_create(ctx, op, &pm->coarse));
  const int64_t n = A->nrows;
  const int64_t nc = (int64_t)(op.n0 - 1) * (op.n1 - 1) * (op.n2 - 1);
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  GFE_TRY(pm->buf.reserve(2 * al(sizeof(float) * n) + 2 * al(sizeof(float) * nc)));
  char* p = (char*)pm->buf.ptr;
  pm->xf = (float*)p;
  pm->tf = (float*)(p + al(sizeof(float) * n));
  pm->bc = (float*)(p + 2 * al(sizeof(float) * n));
  pm->xc = (float*)(p + 2 * al(sizeof(float) * n) + al(sizeof(float) * nc));
  return GFE_OK;
}

// one V-cycle: z = M(r)
int pmg_record(Q2PMG* pm, const float* r, float* z, const int* done) {
  gfe_ctx* ctx = pm->ctx;
  gfe_matrix* A = pm->A;
  const int64_t n = A->nrows;
  const SellF sop{A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(),
                  A->sell_val32.as<float>()};
  const float* dinv = A->dinv32.as<float>();
  const unsigned g = grid_for(n, kPmgBlock);
  const int n0 = (int)A->pmg_n[0], n1 = (int)A->pmg_n[1], n2 = (int)A->pmg_n[2];
  const int32_t* map = A->pmg_node.as<int32_t>();
  const int64_t nc = (int64_t)(n0 - 1) * (n1 - 1) * (n2 - 1);
  const int64_t L = (2 * (int64_t)n0 + 1) * (2 * (int64_t)n1 + 1) * (2 * (int64_t)n2 + 1);
  k_pmg_pre<<<g, kPmgBlock, 0, ctx->stream>>>(n, sop, r, dinv, pm->xf, done);
  k_pmg_residual<<<g, kPmgBlock, 0, ctx->stream>>>(n, sop, pm->xf, r, pm->tf, done);
  k_pmg_restrict<<<grid_for(nc, 256, (int64_t)ctx->num_sms * 8), 256, 0, ctx->stream>>>(
      n0, n1, n2, map, pm->tf, pm->bc, done);
  ctx->launches += 3;
  GFE_TRY(mg_record(pm->coarse, pm->bc, pm->xc, done));
  k_pmg_prolong<<<grid_for(L, 256, (int64_t)ctx->num_sms * 8), 256, 0, ctx->stream>>>(
      n0, n1, n2, map, pm->xc, pm->xf, done);
  k_pmg_smooth<<<g, kPmgBlock, 0, ctx->stream>>>(n, sop, pm->xf, r, dinv, pm->tf, done);
  k_pmg_smooth<<<g, kPmgBlock, 0, ctx->stream>>>(n, sop, pm->tf, r, dinv, z, done);
  ctx->launches += 3;
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

int pmg_apply(Q2PMG* pm, const float* r, float* z, const int* done) {
  gfe_ctx* ctx = pm->ctx;
  if (!pm->exec || pm->cap_r != r || pm->cap_z != z || pm->cap_done != done) {
    if (pm->exec) {
      cudaGraphExecDestroy(pm->exec);
      pm->exec = nullptr;
    }
    const long long l0 = ctx->launches;
    cudaGraph_t graph = nullptr;
    GFE_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int st = pmg_record(pm, r, z, done);
    const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    ctx->launches = l0;  // counted when replayed
    if (st != GFE_OK || ce != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return st != GFE_OK ? st
                          : set_error(GFE_ERR_CUDA, "p-multigrid: graph capture failed: %s",
                                      cudaGetErrorString(ce));
    }
    const cudaError_t ie = cudaGraphInstantiate(&pm->exec, graph, 0);
    size_t nodes = 0;
    cudaGraphGetNodes(graph, nullptr, &nodes);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess)
      return set_error(GFE_ERR_CUDA, "p-multigrid: graph instantiate failed: %s",
                       cudaGetErrorString(ie));
    pm->cap_r = r;
    pm->cap_z = z;
    pm->cap_done = done;
    pm->nodes = (long long)nodes;
  }
  timer_begin(ctx, GFE_KT_PRECOND);
  GFE_CUDA_TRY(cudaGraphLaunch(pm->exec, ctx->stream));
  timer_end(ctx);
  ctx->launches += pm->nodes;
  return GFE_OK;
}

void pmg_destroy(Q2PMG* pm) { delete pm; }

// ==== vector P2 elasticity on a simplexified box: two levels, P2 -> P1 ======================
// The P1 space on the same tets is a subspace of P2: P maps a vertex dof to itself and an
// edge-midpoint dof to the mean of its edge's two vertex dofs (component by component), and
// P^T A_P2 P is the P1 elasticity matrix (constant strains, integrated exactly), assembled
// here from the P1 cell matrices. Gridap numbers the vertex dofs of a conforming P2 space
// before the edge dofs, so the coarse dofs are the first ones of the fine numbering (checked).
// The P2 level is smoothed by Chebyshev-accelerated Jacobi of degree 2 on the eigenvalue
// interval [0.1, 1.1] x lambda_max(D^-1 A) (lambda_max from 12 power steps at set-up; point
// Jacobi alone damps poorly: lambda_max is near 6 for P2 elasticity); the coarse system is
// solved approximately by kCoarseIts steps of Jacobi-PCG, all in FP32 and in one CUDA graph.
namespace {

constexpr int kCoarseIts = 30;
__device__ __constant__ int kTetEdge[6][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 3}, {2, 3}};
// local vertices (x fastest) of the 6 tets of a hexahedron, in the box's simplexification
__device__ __constant__ int kHexTet[6][4] = {{0, 1, 2, 6}, {0, 1, 4, 6}, {1, 2, 3, 6},
                                             {1, 3, 6, 7}, {1, 4, 5, 6}, {1, 5, 6, 7}};

__global__ void k_p1_ids(int64_t ncells, const int32_t* __restrict__ p2, int32_t* __restrict__ p1,
                         int* __restrict__ maxv) {
  int m = 0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ncells * 12;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / 12;
    const int l = (int)(t - c * 12), comp = l / 4, node = l % 4;
    const int32_t id = p2[c * 30 + comp * 10 + node];
    p1[t] = id;
    m = max(m, (int)id);
  }
  for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) atomicMax(maxv, m);
}

// every positive edge-node id above the vertex ids
__global__ void k_p2_edges_after(int64_t ncells, const int32_t* __restrict__ p2, int nv,
                                 int* __restrict__ bad) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ncells * 18;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / 18;
    const int l = (int)(t - c * 18), comp = l / 6, e = l % 6;
    const int32_t id = p2[c * 30 + comp * 10 + 4 + e];
    if (id > 0 && id <= nv) atomicExch(bad, 1);
  }
}

// P1 elasticity cell matrices of the simplexified box: K[(c*12 + li + 12 lj)], local dof
// comp*4 + node, column-major; K = |T| (lambda d_k phi_i d_l phi_j + mu (delta_kl grad phi_i .
// grad phi_j + d_l phi_i d_k phi_j)) with constant gradients
__global__ void k_p1_elasticity_cells(int64_t ncells, int n0, int n1, double h0, double h1,
                                      double h2, double x0, double y0, double z0, int coef_kind,
                                      const double* __restrict__ coef, double* __restrict__ K) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const int64_t hex = c / 6;
  const int t = (int)(c - hex * 6);
  const int ci = (int)(hex % n0), cj = (int)((hex / n0) % n1), ck = (int)(hex / ((int64_t)n0 * n1));
  double X[4][3];
  for (int a = 0; a < 4; ++a) {
    const int L = kHexTet[t][a];
    X[a][0] = x0 + (ci + (L & 1)) * h0;
    X[a][1] = y0 + (cj + ((L >> 1) & 1)) * h1;
    X[a][2] = z0 + (ck + (L >> 2)) * h2;
  }
  double J[3][3];
  for (int k = 0; k < 3; ++k)
    for (int l = 0; l < 3; ++l) J[k][l] = X[k + 1][l] - X[0][l];
  // inverse of J (rows: edge vectors): grad phi_{k+1} = column k of J^-1
  const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  const double id = 1.0 / det;
  double Ji[3][3];
  Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
  Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  double g[4][3];  // physical gradients of the 4 barycentric shape functions
  for (int d = 0; d < 3; ++d) {
    g[1][d] = Ji[d][0];
    g[2][d] = Ji[d][1];
    g[3][d] = Ji[d][2];
    g[0][d] = -(g[1][d] + g[2][d] + g[3][d]);
  }
  double lam = 1.0, mu = 1.0;
  if (coef_kind == GFE_COEF_CELL) {
    lam = coef[2 * c];
    mu = coef[2 * c + 1];
  } else if (coef_kind == GFE_COEF_CONST) {
    lam = coef[0];
    mu = coef[1];
  }
  const double vol = fabs(det) / 6.0;
  double* Kc = K + c * 144;
  for (int lj = 0; lj < 12; ++lj) {
    const int l = lj / 4, j = lj % 4;
    for (int li = 0; li < 12; ++li) {
      const int k = li / 4, i = li % 4;
      double v = lam * g[i][k] * g[j][l] + mu * g[i][l] * g[j][k];
      if (k == l) v += mu * (g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2]);
      Kc[li + 12 * lj] = vol * v;
    }
  }
}

// P (fine dof -> up to two coarse dofs, 0-based) from the P2 ids; identical rows are written
// by every tet that holds the dof
__global__ void k_p2_prolong_rows(int64_t ncells, const int32_t* __restrict__ p2,
                                  int32_t* __restrict__ pc) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < ncells * 30;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / 30;
    const int l = (int)(t - c * 30), comp = l / 10, node = l % 10;
    const int32_t d = p2[t];
    if (d <= 0) continue;
    const int32_t* ids = p2 + c * 30 + comp * 10;
    int32_t a = -1, b = -1;
    if (node < 4) {
      a = d - 1;
    } else {
      const int32_t va = ids[kTetEdge[node - 4][0]], vb = ids[kTetEdge[node - 4][1]];
      a = va > 0 ? va - 1 : -1;
      b = vb > 0 ? vb - 1 : -1;
    }
    pc[2 * (int64_t)(d - 1)] = a;
    pc[2 * (int64_t)(d - 1) + 1] = b;
  }
}

// transpose of P: count, fill (slots by atomics), then each coarse row sorted by fine index
__global__ void k_pt_count(int64_t n, const int32_t* __restrict__ pc, int32_t* __restrict__ cnt) {
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < n;
       d += (int64_t)gridDim.x * blockDim.x)
    for (int s = 0; s < 2; ++s)
      if (pc[2 * d + s] >= 0) atomicAdd(cnt + pc[2 * d + s], 1);
}
__global__ void k_pt_fill(int64_t n, const int32_t* __restrict__ pc,
                          const int64_t* __restrict__ ptr, int32_t* __restrict__ fill,
                          int32_t* __restrict__ rows) {
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < n;
       d += (int64_t)gridDim.x * blockDim.x)
    for (int s = 0; s < 2; ++s) {
      const int32_t v = pc[2 * d + s];
      if (v >= 0) rows[ptr[v] + atomicAdd(fill + v, 1)] = (int32_t)d;
    }
}
__global__ void k_pt_sort(int64_t nc, const int64_t* __restrict__ ptr, int32_t* __restrict__ rows) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nc;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = ptr[v], e = ptr[v + 1];
    for (int64_t i = a + 1; i < e; ++i) {
      const int32_t x = rows[i];
      int64_t k = i - 1;
      while (k >= a && rows[k] > x) {
        rows[k + 1] = rows[k];
        --k;
      }
      rows[k + 1] = x;
    }
  }
}

// b_c[v] = sum over the fine dofs d referencing v of w(d, v) r[d] (w = 1 for the vertex's own
// dof, 1/2 for an edge midpoint), in ascending d
__global__ void k_p2_restrict(int64_t nc, const int64_t* __restrict__ ptr,
                              const int32_t* __restrict__ rows, const int32_t* __restrict__ pc,
                              const float* __restrict__ r, float* __restrict__ bc,
                              const int* done) {
  if (stop_p(done)) return;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nc;
       v += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int64_t q = ptr[v]; q < ptr[v + 1]; ++q) {
      const int32_t d = rows[q];
      const float w = pc[2 * (int64_t)d + 1] >= 0 || pc[2 * (int64_t)d] != (int32_t)v ? 0.5f : 1.f;
      s = fmaf(w, __ldg(r + d), s);
    }
    bc[v] = s;
  }
}

// x += P x_c
__global__ void k_p2_prolong(int64_t n, const int32_t* __restrict__ pc,
                             const float* __restrict__ xc, float* __restrict__ x,
                             const int* done) {
  if (stop_p(done)) return;
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < n;
       d += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = pc[2 * d], b = pc[2 * d + 1];
    float s;
    if (b < 0 && a >= 0 && a == (int32_t)d) s = xc[a];
    else s = 0.5f * ((a >= 0 ? xc[a] : 0.f) + (b >= 0 ? xc[b] : 0.f));
    x[d] += s;
  }
}

// Chebyshev-accelerated Jacobi: d = c1 d + c2 D^-1 (b - A x_in), x_out = x_in + d; with
// zero_x the step from x = 0 (d = c2 D^-1 b, no product)
__global__ void __launch_bounds__(kPmgBlock)
    k_cheb(int64_t n, SellF A, const float* __restrict__ xin, const float* __restrict__ b,
           const float* __restrict__ dinv, float* __restrict__ dvec, float* __restrict__ xout,
           float c1, float c2, int zero_x, const int* done) {
  if (stop_p(done)) return;
  const int64_t r = (int64_t)blockIdx.x * kPmgBlock + threadIdx.x;
  if (r >= n) return;
  const float res = zero_x ? __ldg(b + r)
                           : __ldg(b + r) - sell_row<float, float>(r, A.sptr, A.scol, A.sval, xin);
  const float dn = (zero_x ? 0.f : c1 * dvec[r]) + c2 * __ldg(dinv + r) * res;
  dvec[r] = dn;
  xout[r] = (zero_x ? 0.f : __ldg(xin + r)) + dn;
}

// ---- the coarse Jacobi-PCG (FP32 vectors, FP64 reductions), all steps on the device ----
struct ICState {
  double rz, rz_new, pq;
  float alpha, beta;
  int stop;
  unsigned ticket[2];
};

template <int NT>
__device__ __forceinline__ double blk_sum(double v, double* sh) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < NT / 32; ++i) s += sh[i];
  __syncthreads();
  return s;
}

// block partials in block order, reduced by the last block to arrive
__device__ bool ic_last(unsigned* ticket, const double* part, double* out, double* sh) {
  __shared__ bool last;
  __threadfence();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double s = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += kPmgBlock) s += __ldcg(part + i);
  s = blk_sum<kPmgBlock>(s, sh);
  if (threadIdx.x == 0) {
    *out = s;
    *ticket = 0u;
  }
  return true;
}

__global__ void __launch_bounds__(kPmgBlock)
    k_ic_init(int64_t n, const float* __restrict__ b, const float* __restrict__ dinv,
              float* __restrict__ x, float* __restrict__ r, float* __restrict__ p,
              double* part, ICState* S, const int* done) {
  __shared__ double sh[kPmgBlock / 32];
  if (stop_p(done)) return;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kPmgBlock + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kPmgBlock) {
    const float bi = b[i], zi = dinv[i] * bi;
    x[i] = 0.f;
    r[i] = bi;
    p[i] = zi;
    acc += (double)bi * zi;
  }
  acc = blk_sum<kPmgBlock>(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
  double tot;
  if (ic_last(&S->ticket[0], part, &tot, sh) && threadIdx.x == 0) {
    S->rz = tot;
    S->stop = !(tot > 0.0) || !isfinite(tot);
  }
}

__global__ void __launch_bounds__(kPmgBlock)
    k_ic_spmv(int64_t n, SellF A, const float* __restrict__ p, float* __restrict__ q,
              double* part, ICState* S, const int* done) {
  __shared__ double sh[kPmgBlock / 32];
  if (stop_p(done) || S->stop) return;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kPmgBlock + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kPmgBlock) {
    const float qi = sell_row<float, float>(i, A.sptr, A.scol, A.sval, p);
    q[i] = qi;
    acc += (double)p[i] * qi;
  }
  acc = blk_sum<kPmgBlock>(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
  double tot;
  if (ic_last(&S->ticket[1], part, &tot, sh) && threadIdx.x == 0) {
    S->pq = tot;
    if (!(tot > 0.0) || !isfinite(tot)) S->stop = 1;
    else S->alpha = (float)(S->rz / tot);
  }
}

__global__ void __launch_bounds__(kPmgBlock)
    k_ic_update(int64_t n, const float* __restrict__ dinv, float* __restrict__ x,
                float* __restrict__ r, const float* __restrict__ p, const float* __restrict__ q,
                double* part, ICState* S, const int* done) {
  __shared__ double sh[kPmgBlock / 32];
  if (stop_p(done) || S->stop) return;
  const float al = S->alpha;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kPmgBlock + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kPmgBlock) {
    x[i] = fmaf(al, p[i], x[i]);
    const float ri = fmaf(-al, q[i], r[i]);
    r[i] = ri;
    acc += (double)ri * (dinv[i] * ri);
  }
  acc = blk_sum<kPmgBlock>(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
  double tot;
  if (ic_last(&S->ticket[0], part, &tot, sh) && threadIdx.x == 0) {
    if (!isfinite(tot)) {
      S->stop = 1;
    } else {
      S->beta = (float)(tot / S->rz);
      S->rz = tot;
      if (!(tot > 0.0)) S->stop = 1;
    }
  }
}

__global__ void k_ic_dir(int64_t n, const float* __restrict__ dinv, const float* __restrict__ r,
                         float* __restrict__ p, const ICState* S, const int* done) {
  if (stop_p(done) || S->stop) return;
  const float be = S->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = fmaf(be, p[i], dinv[i] * r[i]);
}

// power iteration on D^-1 A: v <- D^-1 A v / ||v||; nrm[k] = ||D^-1 A v_k|| for unit v_k
__global__ void k_pw_init(int64_t n, float* __restrict__ v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t h = (uint32_t)i * 2654435761u;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    v[i] = (float)(h & 0xFFFF) / 65536.f + 0.25f;
  }
}
__global__ void __launch_bounds__(kPmgBlock)
    k_pw_step(int64_t n, SellF A, const float* __restrict__ dinv, const float* __restrict__ v,
              float* __restrict__ w, const double* __restrict__ vnorm, double* part,
              double* wnorm, unsigned* ticket) {
  __shared__ double sh[kPmgBlock / 32];
  const float s = vnorm ? (float)(1.0 / sqrt(*vnorm)) : 1.f;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kPmgBlock + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kPmgBlock) {
    const float wi = s * dinv[i] * sell_row<float, float>(i, A.sptr, A.scol, A.sval, v);
    w[i] = wi;
    acc += (double)wi * wi;
  }
  acc = blk_sum<kPmgBlock>(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
  double tot;
  if (ic_last(ticket, part, &tot, sh) && threadIdx.x == 0) *wnorm = tot;
}

}  // namespace

int attach_p2_pmg(gfe_ctx* ctx, gfe_matrix* A, const gfe_problem* p, const double* d_coef) {
  A->p2mg_state = 0;
  if (p->reffe != GFE_REFFE_P2_TET || p->form != GFE_FORM_ELASTICITY || p->ncomp != 3 ||
      A->nd != 30 || A->cols_per_cell() != 30 || A->nrows != A->ncols ||
      p->geometry != GFE_GEOM_CARTESIAN)
    return GFE_OK;
  A->p2mg_lame.owner = ctx;
  const size_t nl = p->coef_kind == GFE_COEF_CELL ? 2 * (size_t)p->ncells : 2;
  GFE_TRY(A->p2mg_lame.reserve(sizeof(double) * nl));
  if (d_coef && (p->coef_kind == GFE_COEF_CELL || p->coef_kind == GFE_COEF_CONST))
    GFE_CUDA_TRY(cudaMemcpyAsync(A->p2mg_lame.ptr, d_coef, sizeof(double) * nl,
                                 cudaMemcpyDeviceToDevice, ctx->stream));
  A->p2mg_coef_kind = d_coef ? p->coef_kind : GFE_COEF_ONE;
  for (int d = 0; d < 3; ++d) A->p2mg_part[d] = p->partition[d];
  for (int d = 0; d < 6; ++d) A->p2mg_dom[d] = p->domain[d];
  A->p2mg_state = 2;
  return GFE_OK;
}

struct P2PMG {
  gfe_ctx* ctx;
  gfe_matrix* A;
  gfe_matrix* Ac = nullptr;  // P1 coarse matrix
  int64_t n = 0, nc = 0;
  DevBuf buf, pc, ptptr, ptrows;
  float *xf, *tf, *df, *bc, *xc, *rc, *pcv, *qc;
  double* part;
  ICState* S;
  float theta = 1.f, delta = 1.f, sigma = 1.f;
  cudaGraphExec_t exec = nullptr;
  const float* cap_r = nullptr;
  float* cap_z = nullptr;
  const int* cap_done = nullptr;
  long long nodes = 0;
  explicit P2PMG(gfe_ctx* c, gfe_matrix* a) : ctx(c), A(a), buf(c), pc(c), ptptr(c), ptrows(c) {}
  ~P2PMG() {
    if (exec) cudaGraphExecDestroy(exec);
    if (Ac) gfe_matrix_destroy(Ac);
  }
};

int p2mg_create(gfe_ctx* ctx, gfe_matrix* A, P2PMG** out) {
  if (A->p2mg_state != 2 || !A->plan_valid)
    return set_error(GFE_ERR_UNSUPPORTED, "two-level P2: the matrix has no attached data");
  P2PMG* pm = new P2PMG(ctx, A);
  *out = pm;
  const int64_t ncells = A->ncells, n = A->nrows;
  pm->n = n;
  // coarse ids and the vertex-first check
  DevBuf ids1(ctx), flags(ctx);
  GFE_TRY(ids1.reserve(sizeof(int32_t) * (size_t)ncells * 12));
  GFE_TRY(flags.reserve(sizeof(int) * 2));
  GFE_CUDA_TRY(cudaMemsetAsync(flags.ptr, 0, sizeof(int) * 2, ctx->stream));
  const int32_t* p2 = A->cell_rows.as<int32_t>();
  k_p1_ids<<<grid_for(ncells * 12, 256, (int64_t)ctx->num_sms * 16), 256, 0, ctx->stream>>>(
      ncells, p2, ids1.as<int32_t>(), flags.as<int>());
  int hv[2] = {0, 1};
  GFE_TRY(copy_out(ctx, hv, flags.ptr, sizeof(int)));
  const int nv = hv[0];
  k_p2_edges_after<<<grid_for(ncells * 18, 256, (int64_t)ctx->num_sms * 16), 256, 0,
                     ctx->stream>>>(ncells, p2, nv, flags.as<int>() + 1);
  ctx->launches += 2;
  GFE_TRY(copy_out(ctx, hv + 1, flags.as<int>() + 1, sizeof(int)));
  if (nv < 1 || hv[1])
    return set_error(GFE_ERR_UNSUPPORTED, "two-level P2: vertex dofs are not numbered first");
  pm->nc = nv;
  // the coarse P1 matrix: pattern of the P1 ids, cell matrices, numeric loop, FP32 plan
  GFE_TRY(gfe_symbolic_loop_matrix(ctx, ncells, 12, ids1.as<int32_t>(), ids1.as<int32_t>(), nv,
                                   nv, &pm->Ac));
  {
    DevBuf K(ctx);
    GFE_TRY(K.reserve(sizeof(double) * (size_t)ncells * 144));
    double h[3];
    for (int d = 0; d < 3; ++d)
      h[d] = (A->p2mg_dom[2 * d + 1] - A->p2mg_dom[2 * d]) / (double)A->p2mg_part[d];
    k_p1_elasticity_cells<<<(unsigned)((ncells + 127) / 128), 128, 0, ctx->stream>>>(
        ncells, (int)A->p2mg_part[0], (int)A->p2mg_part[1], h[0], h[1], h[2], A->p2mg_dom[0],
        A->p2mg_dom[2], A->p2mg_dom[4], A->p2mg_coef_kind, A->p2mg_lame.as<double>(),
        K.as<double>());
    ctx->launches++;
    GFE_CUDA_TRY(cudaGetLastError());
    GFE_TRY(gfe_numeric_loop_matrix(ctx, pm->Ac, K.as<double>()));
  }
  GFE_TRY(build_solver_plan(ctx, pm->Ac));
  // P and its transpose
  GFE_TRY(pm->pc.reserve(sizeof(int32_t) * 2 * (size_t)n));
  GFE_CUDA_TRY(cudaMemsetAsync(pm->pc.ptr, 0xFF, sizeof(int32_t) * 2 * (size_t)n, ctx->stream));
  k_p2_prolong_rows<<<grid_for(ncells * 30, 256, (int64_t)ctx->num_sms * 16), 256, 0,
                      ctx->stream>>>(ncells, p2, pm->pc.as<int32_t>());
  DevBuf cnt(ctx), fill(ctx);
  GFE_TRY(cnt.reserve(sizeof(int32_t) * (size_t)(nv + 1)));
  GFE_TRY(fill.reserve(sizeof(int32_t) * (size_t)(nv + 1)));
  GFE_CUDA_TRY(cudaMemsetAsync(cnt.ptr, 0, sizeof(int32_t) * (size_t)(nv + 1), ctx->stream));
  GFE_CUDA_TRY(cudaMemsetAsync(fill.ptr, 0, sizeof(int32_t) * (size_t)(nv + 1), ctx->stream));
  const unsigned gn = grid_for(n, 256, (int64_t)ctx->num_sms * 16);
  k_pt_count<<<gn, 256, 0, ctx->stream>>>(n, pm->pc.as<int32_t>(), cnt.as<int32_t>());
  GFE_TRY(pm->ptptr.reserve(sizeof(int64_t) * (size_t)(nv + 1)));
  GFE_TRY(scan_exclusive_i32_to_i64(ctx, cnt.as<int32_t>(), pm->ptptr.as<int64_t>(), nv));
  int64_t total = 0;
  GFE_TRY(copy_out(ctx, &total, pm->ptptr.as<int64_t>() + nv, sizeof(int64_t)));
  GFE_TRY(pm->ptrows.reserve(sizeof(int32_t) * (size_t)(total > 0 ? total : 1)));
  k_pt_fill<<<gn, 256, 0, ctx->stream>>>(n, pm->pc.as<int32_t>(), pm->ptptr.as<int64_t>(),
                                         fill.as<int32_t>(), pm->ptrows.as<int32_t>());
  k_pt_sort<<<grid_for(nv, 256, (int64_t)ctx->num_sms * 16), 256, 0, ctx->stream>>>(
      nv, pm->ptptr.as<int64_t>(), pm->ptrows.as<int32_t>());
  ctx->launches += 4;
  GFE_CUDA_TRY(cudaGetLastError());
  // vectors: fine x, t, d; coarse b, x, r, p, q; partials; coarse-solve state
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t fb = al(sizeof(float) * n), cb = al(sizeof(float) * nv);
  const size_t nparts = (size_t)ctx->num_sms * 8 + 64;
  GFE_TRY(pm->buf.reserve(3 * fb + 5 * cb + al(sizeof(double) * nparts) + al(sizeof(ICState)) +
                          al(sizeof(double) * 4)));
  char* q = (char*)pm->buf.ptr;
  pm->xf = (float*)q; q += fb;
  pm->tf = (float*)q; q += fb;
  pm->df = (float*)q; q += fb;
  pm->bc = (float*)q; q += cb;
  pm->xc = (float*)q; q += cb;
  pm->rc = (float*)q; q += cb;
  pm->pcv = (float*)q; q += cb;
  pm->qc = (float*)q; q += cb;
  pm->part = (double*)q; q += al(sizeof(double) * nparts);
  pm->S = (ICState*)q; q += al(sizeof(ICState));
  double* norms = (double*)q;
  GFE_CUDA_TRY(cudaMemsetAsync(pm->S, 0, sizeof(ICState), ctx->stream));
  // lambda_max(D^-1 A) by 12 power steps (ping-pong between xf and tf)
  const SellF sop{A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(), A->sell_val32.as<float>()};
  const float* dinv = A->dinv32.as<float>();
  const unsigned gp = (unsigned)(ctx->num_sms * 8);
  k_pw_init<<<gn, 256, 0, ctx->stream>>>(n, pm->xf);
  k_pw_step<<<gp, kPmgBlock, 0, ctx->stream>>>(n, sop, dinv, pm->xf, pm->tf, nullptr, pm->part,
                                              norms, &pm->S->ticket[0]);
  float* v = pm->tf;
  float* w = pm->xf;
  for (int it = 0; it < 12; ++it) {
    k_pw_step<<<gp, kPmgBlock, 0, ctx->stream>>>(n, sop, dinv, v, w, norms + (it & 1), pm->part,
                                                norms + ((it + 1) & 1), &pm->S->ticket[0]);
    std::swap(v, w);
  }
  ctx->launches += 14;
  GFE_CUDA_TRY(cudaGetLastError());
  double hn[2] = {0, 0};
  GFE_TRY(copy_out(ctx, hn, norms, sizeof(double) * 2));
  // after the last step: norms[12 & 1 = 0] = ||D^-1 A v_unit||^2
  const double lmax = std::sqrt(hn[0]);
  if (!(lmax > 0.0) || !std::isfinite(lmax))
    return set_error(GFE_ERR_NONFINITE, "two-level P2: eigenvalue estimate failed");
  const double a = 0.1 * lmax, b = 1.1 * lmax;
  pm->theta = (float)(0.5 * (a + b));
  pm->delta = (float)(0.5 * (b - a));
  pm->sigma = pm->theta / pm->delta;
  return GFE_OK;
}

int p2mg_record(P2PMG* pm, const float* r, float* z, const int* done) {
  gfe_ctx* ctx = pm->ctx;
  gfe_matrix* A = pm->A;
  gfe_matrix* Ac = pm->Ac;
  const int64_t n = pm->n, nc = pm->nc;
  const SellF sop{A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(), A->sell_val32.as<float>()};
  const SellF cop{Ac->sell_ptr.as<int64_t>(), Ac->sell_col.as<int32_t>(),
                  Ac->sell_val32.as<float>()};
  const float* dinv = A->dinv32.as<float>();
  const float* dinvc = Ac->dinv32.as<float>();
  const unsigned g = grid_for(n, kPmgBlock), gc = (unsigned)(ctx->num_sms * 8);
  const unsigned gv = grid_for(n, 256, (int64_t)ctx->num_sms * 8);
  const unsigned gcv = grid_for(nc, 256, (int64_t)ctx->num_sms * 8);
  // Chebyshev coefficients of the two steps: rho0 = 1/sigma, rho1 = 1/(2 sigma - rho0)
  const float rho0 = 1.f / pm->sigma, rho1 = 1.f / (2.f * pm->sigma - rho0);
  const float c2_0 = 1.f / pm->theta, c1_1 = rho1 * rho0, c2_1 = 2.f * rho1 / pm->delta;
  // pre-smoothing from zero: xf
  k_cheb<<<g, kPmgBlock, 0, ctx->stream>>>(n, sop, nullptr, r, dinv, pm->df, pm->tf, 0.f, c2_0,
                                           1, done);
  k_cheb<<<g, kPmgBlock, 0, ctx->stream>>>(n, sop, pm->tf, r, dinv, pm->df, pm->xf, c1_1, c2_1,
                                           0, done);
  // residual, restriction
  k_pmg_residual<<<g, kPmgBlock, 0, ctx->stream>>>(n, sop, pm->xf, r, pm->tf, done);
  k_p2_restrict<<<gcv, 256, 0, ctx->stream>>>(nc, pm->ptptr.as<int64_t>(),
                                              pm->ptrows.as<int32_t>(), pm->pc.as<int32_t>(),
                                              pm->tf, pm->bc, done);
  ctx->launches += 4;
  // coarse: kCoarseIts Jacobi-PCG steps from zero
  GFE_CUDA_TRY(cudaMemsetAsync(pm->S, 0, sizeof(ICState), ctx->stream));
  k_ic_init<<<gc, kPmgBlock, 0, ctx->stream>>>(nc, pm->bc, dinvc, pm->xc, pm->rc, pm->pcv,
                                               pm->part, pm->S, done);
  ctx->launches++;
  for (int it = 0; it < kCoarseIts; ++it) {
    k_ic_spmv<<<gc, kPmgBlock, 0, ctx->stream>>>(nc, cop, pm->pcv, pm->qc, pm->part, pm->S, done);
    k_ic_update<<<gc, kPmgBlock, 0, ctx->stream>>>(nc, dinvc, pm->xc, pm->rc, pm->pcv, pm->qc,
                                                   pm->part, pm->S, done);
    k_ic_dir<<<gcv, 256, 0, ctx->stream>>>(nc, dinvc, pm->rc, pm->pcv, pm->S, done);
    ctx->launches += 3;
  }
  // prolongation, post-smoothing from xf (two Chebyshev steps) into z
  k_p2_prolong<<<gv, 256, 0, ctx->stream>>>(n, pm->pc.as<int32_t>(), pm->xc, pm->xf, done);
  k_cheb<<<g, kPmgBlock, 0, ctx->stream>>>(n, sop, pm->xf, r, dinv, pm->df, pm->tf, 0.f, c2_0,
                                           0, done);
  k_cheb<<<g, kPmgBlock, 0, ctx->stream>>>(n, sop, pm->tf, r, dinv, pm->df, z, c1_1, c2_1, 0,
                                           done);
  ctx->launches += 3;
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

int p2mg_apply(P2PMG* pm, const float* r, float* z, const int* done) {
  gfe_ctx* ctx = pm->ctx;
  if (!pm->exec || pm->cap_r != r || pm->cap_z != z || pm->cap_done != done) {
    if (pm->exec) {
      cudaGraphExecDestroy(pm->exec);
      pm->exec = nullptr;
    }
    const long long l0 = ctx->launches;
    cudaGraph_t graph = nullptr;
    GFE_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int st = p2mg_record(pm, r, z, done);
    const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    ctx->launches = l0;
    if (st != GFE_OK || ce != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return st != GFE_OK ? st
                          : set_error(GFE_ERR_CUDA, "two-level P2: graph capture failed: %s",
                                      cudaGetErrorString(ce));
    }
    const cudaError_t ie = cudaGraphInstantiate(&pm->exec, graph, 0);
    size_t nodes = 0;
    cudaGraphGetNodes(graph, nullptr, &nodes);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess)
      return set_error(GFE_ERR_CUDA, "two-level P2: graph instantiate failed: %s",
                       cudaGetErrorString(ie));
    pm->cap_r = r;
    pm->cap_z = z;
    pm->cap_done = done;
    pm->nodes = (long long)nodes;
  }
  timer_begin(ctx, GFE_KT_PRECOND);
  GFE_CUDA_TRY(cudaGraphLaunch(pm->exec, ctx->stream));
  timer_end(ctx);
  ctx->launches += pm->nodes;
  return GFE_OK;
}

void p2mg_destroy(P2PMG* pm) { delete pm; }

}  // namespace gfe
