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
static int pmg_record(Q2PMG* pm, const float* r, float* z, const int* done) {
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

}  // namespace gfe
