// gfe_batch.cu -- many independent Q1 diffusion problems assembled and solved together.
//
// The problems (unit cubes with their own partitions, per-cell kappa, constant source,
// homogeneous Dirichlet on the boundary) are numbered one after the other into one
// block-diagonal system. Every problem's row range is padded to a multiple of the 256-row
// thread block, so each thread block of the solver kernels belongs to exactly one problem:
// the per-problem dot products reduce deterministically (per-block partials, summed in block
// order by the last block of that problem), every problem has its own alpha, beta and
// convergence flag, and the blocks of a converged problem return at once. Padding rows have
// no entries and a zero right-hand side, so they stay zero.
//
// One call assembles all problems (one symbolic pass and one numeric pass over all cells) and
// runs the batched Jacobi-PCG as chunks of iterations replayed from a CUDA graph, with the
// SpMV launch shape (rows per thread block) picked by a small autotuner on first use.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gfe_internal.h"

namespace gfe {
namespace batch {

constexpr int kRows = 256;  // rows per thread block (and padding unit)
constexpr int kBlk = 256;

struct PState {
  double bb, tol2, rz, rr, pq, alpha, beta;
  int iter, done, converged, pad;
  unsigned ticket[3];
  unsigned pad2;
};

__device__ __forceinline__ double bsum(double v, double* sh) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  __syncthreads();
  return s;
}

// last block of problem p reduces its blocks' partials (NV values each) in block order
template <int NV>
__device__ bool last_of_problem(unsigned* ticket, unsigned nblk, const double* partials,
                                int64_t blk0, double* out, double* sh) {
  __shared__ bool last;
  __threadfence();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == nblk - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  for (int v = 0; v < NV; ++v) {
    double s = 0.0;
    for (unsigned i = threadIdx.x; i < nblk; i += blockDim.x)
      s += __ldcg(partials + (blk0 + i) * NV + v);
    s = bsum(s, sh);
    if (threadIdx.x == 0) out[v] = s;
  }
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}

struct Args {
  int64_t nrows;
  const int64_t* sptr;
  const int32_t* scol;
  const double* sval;
  const double* dinv;
  const int32_t* blk_prob;   // thread block -> problem
  const int64_t* prob_blk0;  // problem -> first thread block
  const int32_t* prob_nblk;  // problem -> number of thread blocks
  PState* S;
  double* partials;          // 2 per thread block
  int* ndone;                // problems finished
  int maxit;
};

__device__ __forceinline__ double sell_row64(int64_t r, const int64_t* __restrict__ sptr,
                                             const int32_t* __restrict__ scol,
                                             const double* __restrict__ sval,
                                             const double* __restrict__ x) {
  const int64_t s = r >> 5;
  const int64_t base = __ldg(sptr + s) + (r & 31);
  const int32_t w = (int32_t)((__ldg(sptr + s + 1) - __ldg(sptr + s)) >> 5);
  double acc = 0.0;
  for (int32_t k = 0; k < w; ++k) {
    const int64_t i = base + (int64_t)k * 32;
    acc = fma(__ldcs(sval + i), __ldg(x + __ldcs(scol + i)), acc);
  }
  return acc;
}

// rows of block b: [b*kRows, (b+1)*kRows); ROWS_PER_THREAD = kRows / blockDim
template <int RPT>
__global__ void __launch_bounds__(kBlk) k_b_init(Args a, const double* __restrict__ b,
                                                 double* __restrict__ x, double* __restrict__ r,
                                                 double* __restrict__ p, double rtol2) {
  __shared__ double sh[kBlk / 32];
  const int prob = a.blk_prob[blockIdx.x];
  double rz = 0.0, bb = 0.0;
  for (int t = 0; t < RPT; ++t) {
    const int64_t i = (int64_t)blockIdx.x * kRows + t * (int64_t)blockDim.x + threadIdx.x;
    if (i < a.nrows) {
      const double bi = b[i];
      x[i] = 0.0;
      r[i] = bi;
      const double z = a.dinv[i] * bi;
      p[i] = z;
      rz += bi * z;
      bb += bi * bi;
    }
  }
  rz = bsum(rz, sh);
  bb = bsum(bb, sh);
  if (threadIdx.x == 0) {
    a.partials[2 * blockIdx.x] = rz;
    a.partials[2 * blockIdx.x + 1] = bb;
  }
  double tot[2];
  PState* S = a.S + prob;
  if (last_of_problem<2>(&S->ticket[1], a.prob_nblk[prob], a.partials, a.prob_blk0[prob], tot,
                         sh) &&
      threadIdx.x == 0) {
    S->rz = tot[0];
    S->bb = tot[1];
    S->rr = tot[1];
    S->tol2 = rtol2 * tot[1];
    S->iter = 0;
    S->converged = tot[1] == 0.0;
    S->done = tot[1] == 0.0;
    if (S->done) atomicAdd(a.ndone, 1);
  }
}

template <int RPT>
__global__ void __launch_bounds__(kBlk) k_b_spmv(Args a, const double* __restrict__ p,
                                                 double* __restrict__ q) {
  __shared__ double sh[kBlk / 32];
  const int prob = a.blk_prob[blockIdx.x];
  PState* S = a.S + prob;
  if (S->done) return;
  double d = 0.0;
  for (int t = 0; t < RPT; ++t) {
    const int64_t i = (int64_t)blockIdx.x * kRows + t * (int64_t)blockDim.x + threadIdx.x;
    if (i < a.nrows) {
      const double y = sell_row64(i, a.sptr, a.scol, a.sval, p);
      q[i] = y;
      d += p[i] * y;
    }
  }
  d = bsum(d, sh);
  if (threadIdx.x == 0) a.partials[2 * blockIdx.x] = d;
  double tot[1];
  // one value per block stored at stride 2: reuse the NV=2 reducer's layout with NV=1 via
  // a private ticket; read partials[2*i]
  __shared__ bool last;
  __threadfence();
  if (threadIdx.x == 0) last = atomicAdd(&S->ticket[0], 1u) == (unsigned)a.prob_nblk[prob] - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  double s = 0.0;
  for (int i = threadIdx.x; i < a.prob_nblk[prob]; i += (int)blockDim.x)
    s += __ldcg(a.partials + 2 * (a.prob_blk0[prob] + i));
  s = bsum(s, sh);
  if (threadIdx.x == 0) {
    tot[0] = s;
    S->pq = tot[0];
    S->alpha = tot[0] != 0.0 ? S->rz / tot[0] : 0.0;
    S->ticket[0] = 0u;
  }
}

template <int RPT>
__global__ void __launch_bounds__(kBlk) k_b_update(Args a, double* __restrict__ x,
                                                   double* __restrict__ r,
                                                   const double* __restrict__ p,
                                                   const double* __restrict__ q) {
  __shared__ double sh[kBlk / 32];
  const int prob = a.blk_prob[blockIdx.x];
  PState* S = a.S + prob;
  if (S->done) return;
  const double alpha = S->alpha;
  double rz = 0.0, rr = 0.0;
  for (int t = 0; t < RPT; ++t) {
    const int64_t i = (int64_t)blockIdx.x * kRows + t * (int64_t)blockDim.x + threadIdx.x;
    if (i < a.nrows) {
      x[i] = fma(alpha, p[i], x[i]);
      const double ri = fma(-alpha, q[i], r[i]);
      r[i] = ri;
      rz += ri * (a.dinv[i] * ri);
      rr += ri * ri;
    }
  }
  rz = bsum(rz, sh);
  rr = bsum(rr, sh);
  if (threadIdx.x == 0) {
    a.partials[2 * blockIdx.x] = rz;
    a.partials[2 * blockIdx.x + 1] = rr;
  }
  double tot[2];
  if (last_of_problem<2>(&S->ticket[1], a.prob_nblk[prob], a.partials, a.prob_blk0[prob], tot,
                         sh) &&
      threadIdx.x == 0) {
    S->iter += 1;
    S->rr = tot[1];
    bool fin = false;
    if (!isfinite(tot[0]) || !isfinite(tot[1])) fin = true;
    else if (tot[1] <= S->tol2) {
      fin = true;
      S->converged = 1;
    } else if (S->iter >= a.maxit) fin = true;
    S->beta = S->rz != 0.0 ? tot[0] / S->rz : 0.0;
    S->rz = tot[0];
    if (fin) {
      S->done = 1;
      atomicAdd(a.ndone, 1);
    }
  }
}

// p = D r + beta p; a problem that just finished skips it (its p is no longer used)
template <int RPT>
__global__ void __launch_bounds__(kBlk) k_b_dir(Args a, const double* __restrict__ r,
                                                double* __restrict__ p) {
  const int prob = a.blk_prob[blockIdx.x];
  const PState* S = a.S + prob;
  if (S->done) return;
  const double beta = S->beta;
  for (int t = 0; t < RPT; ++t) {
    const int64_t i = (int64_t)blockIdx.x * kRows + t * (int64_t)blockDim.x + threadIdx.x;
    if (i < a.nrows) p[i] = fma(beta, p[i], a.dinv[i] * r[i]);
  }
}

}  // namespace batch
}  // namespace gfe

struct gfe_batch {
  gfe_ctx* ctx = nullptr;
  int32_t nproblems = 0;
  int64_t nrows = 0, ncells = 0, nfree_total = 0;
  std::vector<int64_t> row0, nfree, cell0, ncell;  // per problem
  gfe_matrix* A = nullptr;
  gfe::DevBuf ids, coef, b, blk_prob, prob_blk0, prob_nblk, state, partials, ndone, vec;
  int rpt = 0;          // tuned rows per thread (0 = not tuned yet)
  double rtol = 1e-8;
  int32_t maxiter = 100000;
  int64_t nnz = 0;
};

namespace gfe {

static int batch_chunk(gfe_ctx* ctx, gfe_batch* B, int rpt, int iters, double* x, double* r,
                       double* p, double* q) {
  using namespace batch;
  Args a;
  a.nrows = B->nrows;
  a.sptr = B->A->sell_ptr.as<int64_t>();
  a.scol = B->A->sell_col.as<int32_t>();
  a.sval = B->A->sell_val64.as<double>();
  a.dinv = B->A->dinv64.as<double>();
  a.blk_prob = B->blk_prob.as<int32_t>();
  a.prob_blk0 = B->prob_blk0.as<int64_t>();
  a.prob_nblk = B->prob_nblk.as<int32_t>();
  a.S = B->state.as<PState>();
  a.partials = B->partials.as<double>();
  a.ndone = B->ndone.as<int>();
  a.maxit = B->maxiter;
  const unsigned g = (unsigned)(B->nrows / kRows);
  const unsigned thr = (unsigned)(kRows / rpt);
  for (int k = 0; k < iters; ++k) {
    if (rpt == 1) {
      k_b_spmv<1><<<g, thr, 0, ctx->stream>>>(a, p, q);
      k_b_update<1><<<g, thr, 0, ctx->stream>>>(a, x, r, p, q);
      k_b_dir<1><<<g, thr, 0, ctx->stream>>>(a, r, p);
    } else {
      k_b_spmv<2><<<g, thr, 0, ctx->stream>>>(a, p, q);
      k_b_update<2><<<g, thr, 0, ctx->stream>>>(a, x, r, p, q);
      k_b_dir<2><<<g, thr, 0, ctx->stream>>>(a, r, p);
    }
  }
  ctx->launches += 3 * iters;
  return GFE_OK;
}

}  // namespace gfe

using namespace gfe;

extern "C" int gfe_batch_create(gfe_ctx* ctx, int32_t nproblems, const int64_t* partitions,
                                const double* kappa, gfe_batch** out) {
  clear_error();
  if (!ctx || nproblems < 1 || !partitions || !kappa || !out)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_batch_create: bad arguments");
  gfe_batch* B = new gfe_batch();
  B->ctx = ctx;
  B->nproblems = nproblems;
  // per-problem numbering: interior nodes in node order (CLagrangian with "boundary")
  std::vector<int32_t> ids;
  std::vector<double> coef;  // kappa / h^2 per cell (see gfe_batch_assemble_solve)
  {
    int64_t tot = 0;
    for (int32_t p = 0; p < nproblems; ++p)
      tot += partitions[3 * p] * partitions[3 * p + 1] * partitions[3 * p + 2];
    if (tot > 0 && tot < ((int64_t)1 << 34)) {
      ids.reserve((size_t)tot * 8);
      coef.reserve((size_t)tot);
    }
  }
  int64_t row = 0, cells = 0;
  for (int32_t p = 0; p < nproblems; ++p) {
    const int64_t nx = partitions[3 * p], ny = partitions[3 * p + 1], nz = partitions[3 * p + 2];
    if (nx < 1 || ny < 1 || nz < 1) {
      delete B;
      return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_batch_create: partition of problem %d",
                       (int)p);
    }
    if (nx != ny || ny != nz) {  // the unit-cell tables assume cubic cells
      delete B;
      return set_error(GFE_ERR_UNSUPPORTED,
                       "gfe_batch_create: problem %d: partition must be (n, n, n)", (int)p);
    }
    const int64_t nf = (nx - 1) * (ny - 1) * (nz - 1);
    B->row0.push_back(row);
    B->nfree.push_back(nf);
    B->cell0.push_back(cells);
    B->ncell.push_back(nx * ny * nz);
    std::vector<int32_t> node_dof((nx + 1) * (ny + 1) * (nz + 1));
    int32_t f = 0, g = 0;
    for (int64_t k = 0; k <= nz; ++k)
      for (int64_t j = 0; j <= ny; ++j)
        for (int64_t i = 0; i <= nx; ++i) {
          const bool bnd = i == 0 || j == 0 || k == 0 || i == nx || j == ny || k == nz;
          node_dof[i + (nx + 1) * (j + (ny + 1) * k)] = bnd ? -(++g) : ++f;
        }
    const double inv_h2 = (double)nx * (double)nx;
    for (int64_t c = 0; c < nx * ny * nz; ++c) coef.push_back(kappa[cells + c] * inv_h2);
    for (int64_t k = 0; k < nz; ++k)
      for (int64_t j = 0; j < ny; ++j)
        for (int64_t i = 0; i < nx; ++i)
          for (int l = 0; l < 8; ++l) {
            const int64_t ii = i + (l & 1), jj = j + ((l >> 1) & 1), kk = k + ((l >> 2) & 1);
            const int32_t d = node_dof[ii + (nx + 1) * (jj + (ny + 1) * kk)];
            ids.push_back(d > 0 ? (int32_t)(d + row) : d);
          }
    row += (nf + batch::kRows - 1) / batch::kRows * batch::kRows;
    cells += nx * ny * nz;
    B->nfree_total += nf;
  }
  if (row > INT32_MAX) {
    delete B;
    return set_error(GFE_ERR_UNSUPPORTED, "gfe_batch_create: too many rows");
  }
  B->nrows = row;
  B->ncells = cells;
  const int64_t nblk = row / batch::kRows;
  std::vector<int32_t> bp(nblk), pnb(nproblems);
  std::vector<int64_t> pb0(nproblems);
  for (int32_t p = 0; p < nproblems; ++p) {
    pb0[p] = B->row0[p] / batch::kRows;
    const int64_t end = p + 1 < nproblems ? B->row0[p + 1] : row;
    pnb[p] = (int32_t)((end - B->row0[p]) / batch::kRows);
    for (int64_t b = pb0[p]; b < pb0[p] + pnb[p]; ++b) bp[b] = p;
  }
  for (DevBuf* d : {&B->ids, &B->coef, &B->b, &B->blk_prob, &B->prob_blk0, &B->prob_nblk,
                    &B->state, &B->partials, &B->ndone, &B->vec})
    d->owner = ctx;
  int st = GFE_OK;
  auto up = [&](DevBuf& d, const void* src, size_t nb) {
    if (st != GFE_OK) return;
    st = d.reserve(nb);
    if (st == GFE_OK &&
        cudaMemcpyAsync(d.ptr, src, nb, cudaMemcpyDefault, ctx->stream) != cudaSuccess)
      st = set_error(GFE_ERR_CUDA, "gfe_batch_create: copy failed");
  };
  up(B->ids, ids.data(), ids.size() * sizeof(int32_t));
  up(B->coef, coef.data(), (size_t)cells * sizeof(double));
  up(B->blk_prob, bp.data(), bp.size() * sizeof(int32_t));
  up(B->prob_blk0, pb0.data(), pb0.size() * sizeof(int64_t));
  up(B->prob_nblk, pnb.data(), pnb.size() * sizeof(int32_t));
  if (st == GFE_OK) st = B->state.reserve(sizeof(batch::PState) * nproblems);
  if (st == GFE_OK) st = B->partials.reserve(sizeof(double) * 2 * (size_t)nblk);
  if (st == GFE_OK) st = B->ndone.reserve(sizeof(int) * 4);
  if (st == GFE_OK) st = B->b.reserve(sizeof(double) * (size_t)row);
  if (st == GFE_OK) st = B->vec.reserve(sizeof(double) * (size_t)row * 3);
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
  if (B->A) gfe_matrix_destroy(B->A);
  delete B;
  return GFE_OK;
}

extern "C" int gfe_batch_info(gfe_batch* B, int64_t* nrows, int64_t* nfree, int64_t* ncells) {
  clear_error();
  if (!B) return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_batch_info: NULL");
  if (nrows) *nrows = B->nrows;
  if (nfree) *nfree = B->nfree_total;
  if (ncells) *ncells = B->ncells;
  return GFE_OK;
}

// Assembles (symbolic + numeric over all problems' cells) and solves every problem with
// Jacobi-PCG to rtol. x (host or device) receives the free-dof solutions of the problems one
// after the other (sum of nfree entries). iterations[nproblems] (optional, host) gets each
// problem's iteration count. Returns the number of problems that converged in *nconverged.
extern "C" int gfe_batch_assemble_solve(gfe_batch* B, double source, double rtol,
                                        int32_t maxiter, double* x, int32_t* iterations,
                                        int32_t* nconverged) {
  gfe::NvtxRange nvtx_range("gfe_batch_assemble_solve");
  clear_error();
  if (!B || !x || !(rtol > 0.0))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_batch_assemble_solve: bad arguments");
  gfe_ctx* ctx = B->ctx;
  using namespace batch;
  // 1. symbolic + numeric assembly of the block-diagonal system (one pass each)
  if (B->A) {
    gfe_matrix_destroy(B->A);
    B->A = nullptr;
  }
  GFE_TRY(gfe_symbolic_loop_matrix(ctx, B->ncells, 8, B->ids.as<int32_t>(), B->ids.as<int32_t>(),
                                   B->nrows, B->nrows, &B->A));
  // Every cell is a cube of side h = 1/n of its problem; its stiffness is kappa h K1 and its
  // load f h^3 F1, with K1, F1 the unit-cube tables. Each problem's equations are divided by
  // h^3 (which changes neither its solution nor its relative residuals): the cells then carry
  // the coefficient kappa / h^2 (precomputed at create) and the load f F1, one Cartesian
  // problem on unit cells for the whole batch.
  gfe_problem pr;
  memset(&pr, 0, sizeof(pr));
  pr.dim = 3;
  pr.reffe = GFE_REFFE_Q1;
  pr.ncomp = 1;
  pr.degree = 2;
  pr.ncells = B->ncells;
  pr.nd = 8;
  pr.cell_dof_ids = B->ids.as<int32_t>();
  pr.nfree = B->nrows;
  pr.geometry = GFE_GEOM_CARTESIAN;
  pr.partition[0] = pr.partition[1] = pr.partition[2] = 1;
  pr.domain[1] = pr.domain[3] = pr.domain[5] = 1.0;
  pr.form = GFE_FORM_DIFFUSION;
  pr.precision = GFE_PREC_FP64;
  pr.coef_kind = GFE_COEF_CELL;
  pr.coef = B->coef.as<double>();
  pr.source_kind = GFE_SRC_CONST;
  pr.source = &source;
  pr.source_len = 1;
  GFE_CUDA_TRY(cudaMemsetAsync(B->b.ptr, 0, sizeof(double) * B->nrows, ctx->stream));
  GFE_TRY(assemble_problem(ctx, &pr, B->A, B->b.as<double>()));
  B->A->plan_valid = false;
  GFE_TRY(build_solver_plan(ctx, B->A));
  B->nnz = B->A->nnz;
  // 2. batched Jacobi-PCG
  B->rtol = rtol;
  B->maxiter = maxiter > 0 ? maxiter : 100000;
  double* xd = B->vec.as<double>();  // x in padded row space
  GFE_TRY(ctx->scratch[SCR_SOLVER].reserve(sizeof(double) * (size_t)B->nrows * 3 + 64));
  double* r = ctx->scratch[SCR_SOLVER].as<double>();
  double* p = r + B->nrows;
  double* q = p + B->nrows;
  GFE_CUDA_TRY(cudaMemsetAsync(B->state.ptr, 0, sizeof(PState) * B->nproblems, ctx->stream));
  GFE_CUDA_TRY(cudaMemsetAsync(B->ndone.ptr, 0, sizeof(int) * 4, ctx->stream));
  Args a;
  a.nrows = B->nrows;
  a.dinv = B->A->dinv64.as<double>();
  a.blk_prob = B->blk_prob.as<int32_t>();
  a.prob_blk0 = B->prob_blk0.as<int64_t>();
  a.prob_nblk = B->prob_nblk.as<int32_t>();
  a.S = B->state.as<PState>();
  a.partials = B->partials.as<double>();
  a.ndone = B->ndone.as<int>();
  a.maxit = B->maxiter;
  const unsigned g = (unsigned)(B->nrows / kRows);
  k_b_init<1><<<g, kRows, 0, ctx->stream>>>(a, B->b.as<double>(), xd, r, p, rtol * rtol);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  // autotune once: rows per thread 1 or 2 (256 or 128 threads per block), timed on two
  // iterations each of the live system; the solve then restarts from x = 0, so every call
  // runs the same arithmetic (repeated calls give identical results)
  int* hdone = (int*)ctx->h_pinned;
  if (B->rpt == 0) {
    cudaEvent_t e0, e1, e2;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&e2);
    cudaEventRecord(e0, ctx->stream);
    GFE_TRY(batch_chunk(ctx, B, 1, 2, xd, r, p, q));
    cudaEventRecord(e1, ctx->stream);
    GFE_TRY(batch_chunk(ctx, B, 2, 2, xd, r, p, q));
    cudaEventRecord(e2, ctx->stream);
    cudaEventSynchronize(e2);
    float t1 = 0, t2 = 0;
    cudaEventElapsedTime(&t1, e0, e1);
    cudaEventElapsedTime(&t2, e1, e2);
    B->rpt = t2 < t1 ? 2 : 1;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    GFE_CUDA_TRY(cudaMemsetAsync(B->state.ptr, 0, sizeof(PState) * B->nproblems, ctx->stream));
    GFE_CUDA_TRY(cudaMemsetAsync(B->ndone.ptr, 0, sizeof(int) * 4, ctx->stream));
    k_b_init<1><<<g, kRows, 0, ctx->stream>>>(a, B->b.as<double>(), xd, r, p, rtol * rtol);
    ctx->launches++;
    GFE_CUDA_TRY(cudaGetLastError());
  }
  // chunks of iterations captured once into a CUDA graph and replayed
  const int chunk = 20;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  GFE_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  batch_chunk(ctx, B, B->rpt, chunk, xd, r, p, q);
  GFE_CUDA_TRY(cudaStreamEndCapture(ctx->stream, &graph));
  GFE_CUDA_TRY(cudaGraphInstantiate(&exec, graph, 0));
  cudaGraphDestroy(graph);
  int st = GFE_OK;
  for (int guard = 0; guard < 1000000; ++guard) {
    if (cudaGraphLaunch(exec, ctx->stream) != cudaSuccess) {
      st = set_error(GFE_ERR_CUDA, "batch: graph launch failed");
      break;
    }
    if (cudaMemcpyAsync(hdone, B->ndone.ptr, sizeof(int), cudaMemcpyDeviceToHost,
                        ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
      st = set_error(GFE_ERR_CUDA, "batch: sync failed");
      break;
    }
    if (*hdone >= B->nproblems) break;
  }
  cudaGraphExecDestroy(exec);
  GFE_TRY(st);
  // 3. results: unpad x into the caller's array, per-problem iterations
  std::vector<PState> hs(B->nproblems);
  GFE_TRY(copy_out(ctx, hs.data(), B->state.ptr, sizeof(PState) * B->nproblems));
  int32_t nconv = 0;
  int64_t off = 0;
  const bool xdev = is_device_ptr(x);
  for (int32_t pi = 0; pi < B->nproblems; ++pi) {
    if (iterations) iterations[pi] = hs[pi].iter;
    nconv += hs[pi].converged;
    GFE_CUDA_TRY(cudaMemcpyAsync(x + off, xd + B->row0[pi], sizeof(double) * B->nfree[pi],
                                 cudaMemcpyDefault, ctx->stream));
    off += B->nfree[pi];
  }
  if (!xdev) GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (nconverged) *nconverged = nconv;
  return check_device_error(ctx, "gfe_batch_assemble_solve");
}
