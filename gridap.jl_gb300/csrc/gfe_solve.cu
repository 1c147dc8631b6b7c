// gfe_solve.cu -- Krylov solvers on the device: FP64 PCG and FP32-inner / FP64-refinement
// PCG, the LinearSolver a Gridap user plugs in through solve!(x, ns, b)
// (Algebra/LinearSolvers.jl:58-129,202-209).
//
// Matrix layout for the solver: a sliced-ELL copy of the CSR with 32-row slices. Slice s
// stores its rows' k-th entries contiguously (entry k of row 32s+l at ptr[s] + 32k + l),
// padded to the slice's widest row. One thread owns one row: every load of values and
// column ids is a full 32-lane coalesced transaction and each row's sum is a chain of FMAs
// in one thread -- no shuffle reductions. On GB300 an FP64 warp instruction costs the same
// whatever the active-lane mask, so thread-per-row also minimises FP64 instruction issue.
//
// Each CG iteration is three kernels (SpMV+dot, update+dots, direction update). Dot products
// reduce deterministically: fixed grids, per-block partials, the last block to finish sums
// the partials in a fixed order and computes the scalar (alpha, beta) on the device. A done
// flag set on the device makes later kernels return immediately, so the host launches
// chunks of iterations and checks convergence once per chunk.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>

#include <cuda.h>  // CUtensorMap (the encoder is looked up at run time)

#include "gfe_internal.h"

namespace gfe {

constexpr int kVecBlock = 256;
constexpr int kSpmvBlock = 256;

struct SolverState {
  double bb;      // ||b||^2 of the system being solved
  double tol2;    // rtol^2 * bb
  double rz;      // r.z
  double rz_prev; // r.z of the previous iteration (reliable updates)
  double rr;      // r.r
  double pq;      // p.Ap
  double alpha, beta;
  double delta2;  // reliable-update threshold (squared); 0 disables
  double rmax2;   // ||r||^2 at the last reliable update
  double rr64;    // true FP64 ||b - A x||^2 at the last reliable update
  int iter, done, converged, maxit;
  int need_update;
  unsigned ticket[4];
  int defer_update;  // flexible CG in the device loop: a due reliable update does not stop it
  int updates;       // reliable updates made by the device loop
};

__device__ __forceinline__ void raise_e(DevError* err, int code, long long index) {
  if (atomicCAS(&err->code, 0, code) == 0) err->index = index;
}

#include "gfe_reduce.cuh"

template <int NT, typename T>
__device__ __forceinline__ double block_sum_t(T v, double* sh) {
  if constexpr (sizeof(T) == 4) return block_sum_f<NT>(v, sh);
  else return block_sum<NT>((double)v, sh);
}

// ---- sliced-ELL plan ----------------------------------------------------------------------
__global__ void k_slice_widths(const int32_t* __restrict__ rowptr, int64_t nrows,
                               int64_t nslices, int64_t* __restrict__ w) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslices) return;
  int32_t m = 0;
  for (int l = 0; l < 32; ++l) {
    const int64_t r = s * 32 + l;
    if (r < nrows) {
      const int32_t n = rowptr[r + 1] - rowptr[r];
      m = n > m ? n : m;
    }
  }
  w[s] = (int64_t)m * 32;
}

__global__ void k_sell_fill(const int32_t* __restrict__ rowptr,
                            const int32_t* __restrict__ colval, const double* __restrict__ val,
                            int64_t nrows, int64_t nslices, const int64_t* __restrict__ sptr,
                            int32_t* __restrict__ scol, double* __restrict__ sv64,
                            float* __restrict__ sv32, double* __restrict__ dinv64,
                            float* __restrict__ dinv32) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nslices * 32) return;
  const int64_t s = r >> 5;
  const int l = (int)(r & 31);
  const int64_t base = sptr[s];
  const int32_t w = (int32_t)((sptr[s + 1] - base) >> 5);
  int32_t start = 0, n = 0;
  if (r < nrows) {
    start = rowptr[r];
    n = rowptr[r + 1] - start;
  }
  double diag = 0.0;
  for (int32_t k = 0; k < w; ++k) {
    const int64_t idx = base + (int64_t)k * 32 + l;
    int32_t c = r < nrows ? (int32_t)r : 0;
    double v = 0.0;
    if (k < n) {
      c = colval[start + k];
      v = val[start + k];
      if (c == r) diag = v;
    }
    scol[idx] = c;
    sv64[idx] = v;
    sv32[idx] = (float)v;
  }
  if (r < nrows) {
    const double d = (diag != 0.0 && isfinite(diag)) ? 1.0 / diag : 1.0;
    dinv64[r] = d;
    dinv32[r] = (float)d;
  }
}

int build_solver_plan(gfe_ctx* ctx, gfe_matrix* A) {
  if (A->plan_valid) return GFE_OK;
  const int64_t nrows = A->nrows;
  const int64_t nslices = (nrows + 31) / 32;
  DevBuf w(ctx);
  GFE_TRY(w.reserve(sizeof(int64_t) * (nslices + 1)));
  GFE_TRY(A->sell_ptr.reserve(sizeof(int64_t) * (nslices + 1)));
  k_slice_widths<<<grid_for(nslices, 256), 256, 0, ctx->stream>>>(A->rowptr.as<int32_t>(), nrows,
                                                                  nslices, w.as<int64_t>());
  ctx->launches++;
  GFE_TRY(scan_exclusive_i64(ctx, w.as<int64_t>(), A->sell_ptr.as<int64_t>(), nslices));
  int64_t total = 0;
  GFE_TRY(copy_out(ctx, &total, A->sell_ptr.as<int64_t>() + nslices, sizeof(int64_t)));
  A->nslices = nslices;
  A->sell_nnz = total;
  GFE_TRY(A->sell_col.reserve(sizeof(int32_t) * (total > 0 ? total : 1)));
  GFE_TRY(A->sell_val64.reserve(sizeof(double) * (total > 0 ? total : 1)));
  GFE_TRY(A->sell_val32.reserve(sizeof(float) * (total > 0 ? total : 1)));
  GFE_TRY(A->dinv64.reserve(sizeof(double) * (nrows > 0 ? nrows : 1)));
  GFE_TRY(A->dinv32.reserve(sizeof(float) * (nrows > 0 ? nrows : 1)));
  k_sell_fill<<<grid_for(nslices * 32, 256), 256, 0, ctx->stream>>>(
      A->rowptr.as<int32_t>(), A->colval.as<int32_t>(), A->val.as<double>(), nrows, nslices,
      A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(), A->sell_val64.as<double>(),
      A->sell_val32.as<float>(), A->dinv64.as<double>(), A->dinv32.as<float>());
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  A->plan_valid = true;
  return GFE_OK;
}

// ---- diagonal (DIA) FP32 copy ---------------------------------------------------------------
__global__ void k_first_row_of_width(const int32_t* __restrict__ rowptr, int64_t n, int32_t w,
                                     unsigned long long* out) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x)
    if (rowptr[r + 1] - rowptr[r] == w) atomicMin(out, (unsigned long long)r);
}

struct DiagSet {
  int32_t off[32];
  int32_t nd;
};

__global__ void k_dia_check(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                            int64_t n, DiagSet o, int* bad) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x)
    for (int32_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
      const int64_t off = (int64_t)col[k] - r;
      bool found = false;
      for (int d = 0; d < o.nd; ++d) found |= (o.off[d] == off);
      if (!found) atomicExch(bad, 1);
    }
}

// thread per row, one pass per diagonal (sorted columns and sorted offsets merge)
__global__ void k_dia_fill(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                           const double* __restrict__ val, int64_t n, DiagSet o,
                           float* __restrict__ dval) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  int32_t k = rowptr[r];
  const int32_t e = rowptr[r + 1];
  for (int d = 0; d < o.nd; ++d) {
    const int64_t c = r + o.off[d];
    float v = 0.f;
    if (k < e && (int64_t)col[k] == c) v = (float)val[k++];
    dval[(int64_t)d * n + r] = v;
  }
}

int build_dia(gfe_ctx* ctx, gfe_matrix* A) {
  if (A->dia_checked) return GFE_OK;
  A->dia_checked = true;
  A->dia_valid = false;
  const int64_t n = A->nrows;
  const int w = A->max_width;
  if (n == 0 || w < 1 || w > 32 || A->nrows != A->ncols) return GFE_OK;
  DevBuf tmp(ctx);
  GFE_TRY(tmp.reserve(64 + sizeof(int32_t) * 64));
  unsigned long long* drow = tmp.as<unsigned long long>();
  int* dbad = (int*)((char*)tmp.ptr + 16);
  const unsigned long long init = ~0ull;
  GFE_CUDA_TRY(cudaMemcpyAsync(drow, &init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
  GFE_CUDA_TRY(cudaMemsetAsync(dbad, 0, sizeof(int), ctx->stream));
  k_first_row_of_width<<<grid_for(n, 256, (int64_t)ctx->num_sms * 8), 256, 0, ctx->stream>>>(
      A->rowptr.as<int32_t>(), n, w, drow);
  ctx->launches++;
  unsigned long long row = 0;
  GFE_TRY(copy_out(ctx, &row, drow, sizeof(row)));
  if (row >= (unsigned long long)n) return GFE_OK;
  int32_t start = 0;
  GFE_TRY(copy_out(ctx, &start, A->rowptr.as<int32_t>() + row, sizeof(int32_t)));
  int32_t cols[32];
  GFE_TRY(copy_out(ctx, cols, A->colval.as<int32_t>() + start, sizeof(int32_t) * w));
  DiagSet o;
  o.nd = w;
  for (int d = 0; d < w; ++d) o.off[d] = cols[d] - (int32_t)row;
  k_dia_check<<<grid_for(n, 256, (int64_t)ctx->num_sms * 8), 256, 0, ctx->stream>>>(
      A->rowptr.as<int32_t>(), A->colval.as<int32_t>(), n, o, dbad);
  ctx->launches++;
  int bad = 0;
  GFE_TRY(copy_out(ctx, &bad, dbad, sizeof(int)));
  if (bad) return GFE_OK;
  GFE_TRY(A->dia_val32.reserve(sizeof(float) * (size_t)n * w));
  k_dia_fill<<<grid_for(n, 256), 256, 0, ctx->stream>>>(
      A->rowptr.as<int32_t>(), A->colval.as<int32_t>(), A->val.as<double>(), n, o,
      A->dia_val32.as<float>());
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  A->dia_ndiag = w;
  for (int d = 0; d < w; ++d) A->dia_off[d] = o.off[d];
  A->dia_valid = true;
  return GFE_OK;
}

// ---- matrix-free lattice operator: attach (at assembly) and validate -------------------------
// Checks that the matrix rows are the interior nodes of the (n0, n1, n2) box in node order:
// every interior corner of every cell carries dof 1 + its interior lattice index, every
// boundary corner a Dirichlet (negative) id.
__global__ void k_lattice_check(const int32_t* __restrict__ ids, int64_t n0, int64_t n1,
                                int64_t n2, int* bad) {
  const int64_t ncells = n0 * n1 * n2;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ci = c % n0, t = c / n0, cj = t % n1, ck = t / n1;
    for (int a = 0; a < 8; ++a) {
      const int64_t i = ci + (a & 1), j = cj + ((a >> 1) & 1), k = ck + (a >> 2);
      const bool interior = i > 0 && j > 0 && k > 0 && i < n0 && j < n1 && k < n2;
      const int32_t id = ids[c * 8 + a];
      const int64_t want = 1 + (i - 1) + (n0 - 1) * ((j - 1) + (n1 - 1) * (k - 1));
      if (interior ? (int64_t)id != want : id >= 0) atomicExch(bad, 1);
    }
  }
}

// kappa in FP32 at the lattice operator's cell layout: rows of n0 cells padded to a
// multiple of 4 (16-byte row strides, as the tensor-map copies of the operator require)
// (cells (i, line), line = j + n1 k: i over x-blocks and threads, lines over y-blocks)
__global__ void k_coef_to_f32(const double* __restrict__ c, int kind, int64_t n0, int64_t c1,
                              int64_t nlines, float* __restrict__ out) {
  const float cst = kind == GFE_COEF_CONST ? (float)c[0] : 1.f;
  for (int64_t l = blockIdx.y; l < nlines; l += gridDim.y)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n0;
         i += (int64_t)gridDim.x * blockDim.x)
      out[i + c1 * l] = kind == GFE_COEF_CELL ? (float)c[i + n0 * l] : cst;
}

int attach_lattice_operator(gfe_ctx* ctx, gfe_matrix* A, const gfe_problem* p,
                            const double* d_coef, const double* Kref) {
  A->mf_state = 0;
  const int64_t n0 = p->partition[0], n1 = p->partition[1], n2 = p->partition[2];
  if (p->dim != 3 || n0 < 2 || n1 < 2 || n2 < 2 || A->nd != 8 || A->cols_per_cell() != 8 ||
      A->ncells != n0 * n1 * n2 || A->nrows != (n0 - 1) * (n1 - 1) * (n2 - 1) ||
      A->nrows != A->ncols)
    return GFE_OK;
  // the operator's 32-bit strides and its (i-tiles, j-tiles, k) grid
  if (n0 * n1 >= ((int64_t)1 << 31) || n2 - 1 > 65535 || (n1 - 1 + 7) / 8 > 65535)
    return GFE_OK;
  const int64_t nc = A->ncells;
  const int64_t c1 = (n0 + 3) & ~(int64_t)3;
  A->mf_kap32.owner = A->mf_flag.owner = ctx;
  GFE_TRY(A->mf_kap32.reserve(sizeof(float) * (size_t)(c1 * n1 * n2)));
  GFE_CUDA_TRY(cudaMemsetAsync(A->mf_kap32.ptr, 0, sizeof(float) * (size_t)(c1 * n1 * n2),
                               ctx->stream));
  GFE_TRY(A->mf_flag.reserve(sizeof(int) * 4));
  GFE_CUDA_TRY(cudaMemsetAsync(A->mf_flag.ptr, 0, sizeof(int), ctx->stream));
  const unsigned g = grid_for(nc, 256, (int64_t)ctx->num_sms * 8);
  const dim3 gc((unsigned)((n0 + 127) / 128), (unsigned)std::min<int64_t>(n1 * n2, 65535));
  k_coef_to_f32<<<gc, 128, 0, ctx->stream>>>(d_coef, d_coef ? p->coef_kind : GFE_COEF_ONE, n0,
                                             c1, n1 * n2, A->mf_kap32.as<float>());
  ctx->launches++;
  // a closed-form lattice pattern of this grid has had its ids checked already
  const bool known = A->cart_lattice && A->cart_n[0] == n0 && A->cart_n[1] == n1 &&
                     A->cart_n[2] == n2;
  if (!known) {
    k_lattice_check<<<g, 256, 0, ctx->stream>>>(A->cell_rows.as<int32_t>(), n0, n1, n2,
                                                A->mf_flag.as<int>());
    ctx->launches++;
  }
  GFE_CUDA_TRY(cudaGetLastError());
  for (int e = 0; e < 64; ++e) A->mf_K[e] = (float)Kref[e];
  A->mf_n[0] = n0;
  A->mf_n[1] = n1;
  A->mf_n[2] = n2;
  A->mf_state = known ? 2 : 1;
  return GFE_OK;
}

// Resolves a pending numbering check (one small device read); true when the lattice
// operator may replace the FP32 matrix.
static int lattice_ready(gfe_ctx* ctx, gfe_matrix* A, bool* ok) {
  if (A->mf_state == 1) {
    int bad = 1;
    GFE_TRY(copy_out(ctx, &bad, A->mf_flag.ptr, sizeof(int)));
    A->mf_state = bad ? 0 : 2;
  }
  *ok = A->mf_state == 2;
  return GFE_OK;
}

// ---- SpMV ---------------------------------------------------------------------------------
#include "gfe_sell.cuh"

// SpMV operators (thread per row). row_index() is the row of the calling thread (or -1) and
// blocks() the grid that covers all rows with kSpmvBlock threads per block.
__device__ __forceinline__ int64_t linear_row() {
  return (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
}

template <typename T>
struct SellOp {
  const int64_t* sptr;
  const int32_t* scol;
  const T* sval;
  __device__ __forceinline__ T row(int64_t r, const T* __restrict__ x) const {
    return sell_row<T, T>(r, sptr, scol, sval, x);
  }
  __device__ __forceinline__ int64_t row_index() const { return linear_row(); }
  unsigned blocks(int64_t n) const { return grid_for(n, kSpmvBlock); }
  dim3 grid(int64_t n) const { return dim3(blocks(n)); }
};

struct DiagOffsets {
  int32_t off[32];
  int32_t nd;
};

// Diagonal storage: val[d*n + r] = A(r, r + off[d]) (0 where absent). Every load of values
// and of x is a coalesced stream; no column ids are read.
template <typename T>
struct DiaOp {
  const T* val;
  int64_t n;
  DiagOffsets o;
  __device__ __forceinline__ T row(int64_t r, const T* __restrict__ x) const {
    T acc = (T)0;
#pragma unroll 9
    for (int d = 0; d < o.nd; ++d) {
      const int64_t c = r + o.off[d];
      if ((uint64_t)c < (uint64_t)n) acc = fma(__ldcs(val + (int64_t)d * n + r), __ldg(x + c), acc);
    }
    return acc;
  }
  __device__ __forceinline__ int64_t row_index() const { return linear_row(); }
  unsigned blocks(int64_t nr) const { return grid_for(nr, kSpmvBlock); }
  dim3 grid(int64_t nr) const { return dim3(blocks(nr)); }
};

#include "gfe_lattice.cuh"

template <typename TV, typename TX, typename TY>
__global__ void __launch_bounds__(kSpmvBlock)
    k_spmv(int64_t nrows, const int64_t* __restrict__ sptr, const int32_t* __restrict__ scol,
           const TV* __restrict__ sval, const TX* __restrict__ x, TY* __restrict__ y) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  y[r] = (TY)sell_row<TV, TX>(r, sptr, scol, sval, x);
}

int spmv64(gfe_ctx* ctx, gfe_matrix* A, const double* d_x, double* d_y) {
  GFE_TRY(build_solver_plan(ctx, A));
  k_spmv<double, double, double><<<grid_for(A->nrows, kSpmvBlock), kSpmvBlock, 0, ctx->stream>>>(
      A->nrows, A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(),
      A->sell_val64.as<double>(), d_x, d_y);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

// q = A p with the lattice operator; partial p.q (and p.r for flexible CG), last-block alpha.
// PAD: p, q (and r) in the zero-halo padded layout (LatticeQ1Op::pad_index): every
// neighbour load is unconditional and q is written at the padded index. Otherwise the rows
// are the dof numbering and neighbours outside the interior read as 0.
template <bool FCG, bool PAD>
__global__ void __launch_bounds__(kSpmvBlock)
    k_lattice_spmv(LatticeQ1Op op, const float* __restrict__ p, float* __restrict__ q,
                   const float* __restrict__ rr, double* __restrict__ partials, SolverState* S) {
  __shared__ double sh[kSpmvBlock / 32];
  if (S->done) return;
  float d1 = 0.f, d2 = 0.f;
  lattice_tile<FCG, PAD>(op, (int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z, p, q, rr, d1,
                         d2);
  const double s1 = block_sum_f<kSpmvBlock>(d1, sh);
  double s2 = 0.0;
  if (FCG) s2 = block_sum_f<kSpmvBlock>(d2, sh);
  const unsigned bl = block_linear();
  if (threadIdx.x == 0) {
    if (FCG) {
      partials[2 * bl] = s1;
      partials[2 * bl + 1] = s2;
    } else {
      partials[bl] = s1;
    }
  }
  double tot[2];
  if (FCG) {
    if (last_block_reduce<kSpmvBlock, 2>(&S->ticket[0], partials, grid_blocks(), tot, sh) &&
        threadIdx.x == 0) {
      S->pq = tot[0];
      S->alpha = tot[0] != 0.0 ? tot[1] / tot[0] : 0.0;
    }
  } else if (last_block_reduce<kSpmvBlock, 1>(&S->ticket[0], partials, grid_blocks(), tot, sh) &&
             threadIdx.x == 0) {
    S->pq = tot[0];
    S->alpha = tot[0] != 0.0 ? S->rz / tot[0] : 0.0;
  }
}

// The flexible CG's direction update folded into its SpMV on the lattice operator: p = z +
// beta p, and q = A p formed as A z + beta q (A p_new = A z + beta A p_old, q holding A p_old),
// so that the stencil reads z and every other vector only at the thread's own row; partials
// of p.q and p.r and the last-block alpha = (p.r) / (p.q) as k_lattice_spmv<true, false>.
// beta (S->beta) is formed by the preconditioner's last kernel; beta = 0 (a first direction)
// reads neither p nor q.
__global__ void __launch_bounds__(kSpmvBlock)
    k_lattice_spmv_dir(LatticeQ1Op op, const float* __restrict__ z, float* __restrict__ p,
                       float* __restrict__ q, const float* __restrict__ r,
                       double* __restrict__ partials, SolverState* S) {
  __shared__ double sh[kSpmvBlock / 32];
  if (S->done) return;
  const float beta = (float)S->beta;
  const bool keep = beta != 0.f;
  float d1 = 0.f, d2 = 0.f;
  auto epi = [&](int64_t row, float zc, float acc) {
    const float pn = keep ? fmaf(beta, p[row], zc) : zc;
    const float qn = keep ? fmaf(beta, q[row], acc) : acc;
    p[row] = pn;
    q[row] = qn;
    d1 = fmaf(pn, qn, d1);
    d2 = fmaf(pn, __ldg(r + row), d2);
  };
  lattice_rows<false>(op, (int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z, z, epi);
  const double s1 = block_sum_f<kSpmvBlock>(d1, sh);
  const double s2 = block_sum_f<kSpmvBlock>(d2, sh);
  const unsigned bl = block_linear();
  if (threadIdx.x == 0) {
    partials[2 * bl] = s1;
    partials[2 * bl + 1] = s2;
  }
  double tot[2];
  if (last_block_reduce<kSpmvBlock, 2>(&S->ticket[0], partials, grid_blocks(), tot, sh) &&
      threadIdx.x == 0) {
    S->pq = tot[0];
    S->alpha = tot[0] != 0.0 ? tot[1] / tot[0] : 0.0;
  }
}

// ---- lattice SpMV with the tile staged by the tensor-memory accelerator ---------------------
// The same rows and arithmetic as k_lattice_spmv<false, true>, but the block's halo of p
// (34 x 10 x (kLatK + 2) padded nodes) and of kappa (33 x 9 x (kLatK + 1) cells) arrive in
// shared memory through two cp.async.bulk.tensor copies issued by one thread, completing on
// an mbarrier; the k-march then reads its planes from shared memory instead of waiting on L1/L2
// for 13 loads per row. Boxes are 36 floats wide (16-byte rows); their x origin, 32 bx, is a
// multiple of 4 floats. Boxes past the arrays' ends read zeros.
// The TMA tiles march over kTmaK planes: smaller tiles than the register kernel's, so that
// the 128^3 grid (2048 blocks) spreads evenly over the SMs at six resident blocks each.
constexpr int kTmaK = 4;
constexpr int kTmaX = 36, kTmaPY = 10, kTmaPZ = kTmaK + 2, kTmaKY = 9, kTmaKZ = kTmaK + 1;
constexpr unsigned long long kTmaWaitNs = 1000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long gtimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// bounded wait on phase `phase` of an mbarrier (false after limit_ns)
__device__ __forceinline__ bool tma_bar_wait(uint32_t bar, uint32_t phase,
                                             unsigned long long limit_ns = kTmaWaitNs) {
  const unsigned long long t0 = gtimer_ns();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
    if (gtimer_ns() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];"
      :
      : "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

__global__ void __launch_bounds__(kSpmvBlock, 6)
    k_lattice_spmv_tma(const __grid_constant__ CUtensorMap tmap_p,
                       const __grid_constant__ CUtensorMap tmap_k, LatticeQ1Op op,
                       float* __restrict__ q, double* __restrict__ partials, SolverState* S,
                       DevError* err, unsigned long long first_wait_ns) {
  __shared__ alignas(128) float sp[kTmaPZ][kTmaPY][kTmaX];
  __shared__ alignas(128) float sk[kTmaKZ][kTmaKY][kTmaX];
  __shared__ alignas(8) uint64_t bar;
  __shared__ double sh[kSpmvBlock / 32];
  if (S->done) return;
  const int bx = (int)blockIdx.x, by = (int)blockIdx.y, k0 = (int)blockIdx.z * kTmaK;
  const uint32_t b = smem_u32(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b),
                 "r"((uint32_t)(sizeof(sp) + sizeof(sk)))
                 : "memory");
    tma_load_3d(smem_u32(&sp[0][0][0]), &tmap_p, 32 * bx, 8 * by, k0, b);
    tma_load_3d(smem_u32(&sk[0][0][0]), &tmap_k, 32 * bx, 8 * by, k0, b);
  }
  // one thread polls the barrier (the others wait at bar.sync without taking issue slots)
  __shared__ int landed;
  if (threadIdx.x == 0) {
    // first_wait_ns == 0 gives up without polling (the timeout path, exercised by tests)
    landed = first_wait_ns > 0 && tma_bar_wait(b, 0, first_wait_ns) ? 1 : 0;
    if (!landed) {
      // the copies did not land in time: report, then wait (bounded again, kTmaWaitNs) for
      // them to land before the block leaves its shared memory, and skip the tile; if that
      // wait runs out too the copies may still be in flight, and the status tells the caller
      // to discard the context
      raise_e(err, GFE_ERR_TIMEOUT, (long long)block_linear());
      tma_bar_wait(b, 0);
      S->done = 1;
    }
  }
  __syncthreads();
  float d1 = 0.f;
  if (landed) {
    const int m0 = op.n0 - 1, m1 = op.n1 - 1, m2 = op.n2 - 1;
    const int lane = (int)(threadIdx.x & 31), wy = (int)(threadIdx.x >> 5);
    const int i = 32 * bx + lane, j = 8 * by + wy;
    if (i < m0 && j < m1) {
      float xa[9], xb[9], xc[9], ka[4], kb[4];
      auto xplane = [&](int t, float* xv) {  // plane k0 + t - 1 (t = 0 .. kTmaK + 1)
#pragma unroll
        for (int dy = 0; dy < 3; ++dy)
#pragma unroll
          for (int dx = 0; dx < 3; ++dx) xv[dx + 3 * dy] = sp[t][wy + dy][lane + dx];
      };
      auto kplane = [&](int t, float* kv) {  // cell layer k0 + t
#pragma unroll
        for (int cy = 0; cy < 2; ++cy)
#pragma unroll
          for (int cx = 0; cx < 2; ++cx) kv[cx + 2 * cy] = sk[t][wy + cy][lane + cx];
      };
      xplane(0, xa);
      xplane(1, xb);
      kplane(0, ka);
      const int64_t col = op.pad_index(i, j, 0);
#pragma unroll
      for (int t = 0; t < kTmaK; ++t) {
        const int k = k0 + t;
        if (k < m2) {
          xplane(t + 2, xc);
          kplane(t + 1, kb);
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
                for (int lc = 0; lc < 8; ++lc) {
                  const int ix = cx + (lc & 1), iy = cy + ((lc >> 1) & 1), iz = cz + (lc >> 2);
                  const float xv = iz == 0 ? xa[ix + 3 * iy] : iz == 1 ? xb[ix + 3 * iy]
                                                                       : xc[ix + 3 * iy];
                  s = fmaf(op.K[lr + 8 * lc], xv, s);
                }
                acc = fmaf(cz == 0 ? ka[cx + 2 * cy] : kb[cx + 2 * cy], s, acc);
              }
          q[col + (int64_t)op.p2 * k] = acc;
          d1 = fmaf(xb[4], acc, d1);
        }
#pragma unroll
        for (int e = 0; e < 9; ++e) {
          xa[e] = xb[e];
          xb[e] = xc[e];
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) ka[e] = kb[e];
      }
    }
  }
  const double s1 = block_sum_f<kSpmvBlock>(d1, sh);
  if (threadIdx.x == 0) partials[block_linear()] = s1;
  double tot[1];
  if (last_block_reduce<kSpmvBlock, 1>(&S->ticket[0], partials, grid_blocks(), tot, sh) &&
      threadIdx.x == 0) {
    S->pq = tot[0];
    S->alpha = tot[0] != 0.0 ? S->rz / tot[0] : 0.0;
  }
}

// cuTensorMapEncodeTiled from the driver, looked up once (no link-time dependency).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn tensor_map_encoder() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult qr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &qr) == cudaSuccess &&
        qr == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
    else
      (void)cudaGetLastError();
  }
  return fn;
}

// Tensor maps of the padded p vector (p1, m1 + 2, m2 + 2) and of kappa (c1, n1, n2) with the
// boxes of k_lattice_spmv_tma. False when the encoder is unavailable or refuses.
static bool lattice_tensor_maps(const LatticeQ1Op& op, const float* p, CUtensorMap* tp,
                                CUtensorMap* tk) {
  EncodeTiledFn enc = tensor_map_encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(p) & 15) || (reinterpret_cast<uintptr_t>(op.kap) & 15))
    return false;
  const cuuint32_t ones[3] = {1, 1, 1};
  const cuuint64_t pd[3] = {(cuuint64_t)op.p1, (cuuint64_t)op.n1 + 1, (cuuint64_t)op.n2 + 1};
  const cuuint64_t ps[2] = {(cuuint64_t)op.p1 * 4, (cuuint64_t)op.p2 * 4};
  const cuuint32_t pb[3] = {kTmaX, kTmaPY, kTmaPZ};
  const cuuint64_t kd[3] = {(cuuint64_t)op.c1, (cuuint64_t)op.n1, (cuuint64_t)op.n2};
  const cuuint64_t ks[2] = {(cuuint64_t)op.c1 * 4, (cuuint64_t)op.c2 * 4};
  const cuuint32_t kb[3] = {kTmaX, kTmaKY, kTmaKZ};
  if (enc(tp, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(p), pd, ps, pb, ones,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  if (enc(tk, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(op.kap), kd, ks, kb, ones,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  return true;
}

static LatticeQ1Op lattice_op(const gfe_matrix* A) {
  LatticeQ1Op op;
  op.kap = A->mf_kap32.as<float>();
  op.n0 = (int)A->mf_n[0];
  op.n1 = (int)A->mf_n[1];
  op.n2 = (int)A->mf_n[2];
  op.s1 = op.n0 - 1;
  op.s2 = (op.n0 - 1) * (op.n1 - 1);
  op.c1 = (op.n0 + 3) & ~3;  // 16-byte row strides (tensor-map copies)
  op.c2 = op.c1 * op.n1;
  op.p1 = (op.n0 + 1 + 3) & ~3;
  op.p2 = op.p1 * (op.n1 + 1);
  for (int e = 0; e < 64; ++e) op.K[e] = A->mf_K[e];
  return op;
}

// ---- dof layout <-> zero-halo padded lattice layout (mixed CG with the lattice operator) ----
__device__ __forceinline__ int64_t dof_to_pad(const LatticeQ1Op& op, int64_t r) {
  const unsigned m0 = (unsigned)(op.n0 - 1), m1 = (unsigned)(op.n1 - 1);
  const unsigned ru = (unsigned)r;
  const unsigned i = ru % m0, t = ru / m0;
  return op.pad_index((int)i, (int)(t % m1), (int)(t / m1));
}

// out[pad(r)] = in[r] (FP32), halo untouched (zero)
__global__ void k_to_pad(LatticeQ1Op op, int64_t n, const float* __restrict__ in,
                         float* __restrict__ out) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x)
    out[dof_to_pad(op, r)] = in[r];
}

// CG start from x = 0 in the padded layout: r = rhs, p = D r; partials of r.z, r.r
__global__ void __launch_bounds__(kVecBlock)
    k_cg_init_pad(LatticeQ1Op op, int64_t n, const double* __restrict__ rhs,
                  float* __restrict__ r, float* __restrict__ p, const float* __restrict__ dinv,
                  double* __restrict__ partials, SolverState* S, double rtol2) {
  __shared__ double sh[kVecBlock / 32];
  double rz = 0.0, rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = dof_to_pad(op, i);
    const float ri = (float)rhs[i];
    r[j] = ri;
    const float zi = dinv[j] * ri;
    p[j] = zi;
    rz += (double)ri * (double)zi;
    rr += (double)ri * (double)ri;
  }
  rz = block_sum<kVecBlock>(rz, sh);
  rr = block_sum<kVecBlock>(rr, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = rz;
    partials[2 * blockIdx.x + 1] = rr;
  }
  double tot[2];
  if (last_block_reduce<kVecBlock, 2>(&S->ticket[1], partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0) {
    S->rz = tot[0];
    S->rr = tot[1];
    S->bb = tot[1];
    S->tol2 = rtol2 * tot[1];
    S->iter = 0;
    S->converged = 0;
    S->done = (tot[1] == 0.0) ? 1 : 0;
    if (tot[1] == 0.0) S->converged = 1;
  }
}

// x64 += x32 (padded), x32 = 0
__global__ void k_merge_pad(LatticeQ1Op op, int64_t n, double* __restrict__ x64,
                            float* __restrict__ x32) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = dof_to_pad(op, i);
    x64[i] += (double)x32[j];
    x32[j] = 0.f;
  }
}

// ---- CG kernels (T: vector/matrix type; dot products accumulate in double) ----------------
// q = A p and partial p.q; the last block computes alpha = rz / pq.
template <typename T, class Op>
__global__ void __launch_bounds__(kSpmvBlock)
    k_cg_spmv_dot(int64_t n, Op op, const T* __restrict__ p, T* __restrict__ q,
                  double* __restrict__ partials, SolverState* S) {
  __shared__ double sh[kSpmvBlock / 32];
  if (S->done) return;
  const int64_t r = op.row_index();
  T dt = (T)0;
  if (r >= 0 && r < n) {
    const T y = op.row(r, p);
    q[r] = y;
    dt = p[r] * y;
  }
  const double d = block_sum_t<kSpmvBlock, T>(dt, sh);
  if (threadIdx.x == 0) partials[block_linear()] = d;
  double tot[1];
  if (last_block_reduce<kSpmvBlock, 1>(&S->ticket[0], partials, grid_blocks(), tot, sh) &&
      threadIdx.x == 0) {
    S->pq = tot[0];
    S->alpha = tot[0] != 0.0 ? S->rz / tot[0] : 0.0;
  }
}

// x += alpha p; r -= alpha q; partial r.z (z = dinv r) and r.r; the last block decides.
template <typename T>
__global__ void __launch_bounds__(kVecBlock)
    k_cg_update(int64_t n, T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                const T* __restrict__ q, const T* __restrict__ dinv,
                double* __restrict__ partials, SolverState* S) {
  __shared__ double sh[kVecBlock / 32];
  if (S->done) return;
  const T alpha = (T)S->alpha;
  // per-thread partial sums in T (a thread covers ~n / (grid*block) entries); FP64 from the
  // block sum on, so FP32 vectors cost no FP64 issue slots per element
  T rz_t = (T)0, rr_t = (T)0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    const T ri = fma(-alpha, q[i], r[i]);
    r[i] = ri;
    rz_t = fma(ri, dinv[i] * ri, rz_t);
    rr_t = fma(ri, ri, rr_t);
  }
  double rz = block_sum<kVecBlock>((double)rz_t, sh);
  double rr = block_sum<kVecBlock>((double)rr_t, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = rz;
    partials[2 * blockIdx.x + 1] = rr;
  }
  double tot[2];
  if (last_block_reduce<kVecBlock, 2>(&S->ticket[1], partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0) {
    S->iter += 1;
    S->rr = tot[1];
    if (!isfinite(tot[1]) || !isfinite(tot[0])) {
      S->done = 1;
      S->converged = 0;
    } else if (tot[1] <= S->tol2) {
      S->done = 1;
      S->converged = 1;
    } else if (S->iter >= S->maxit) {
      S->done = 1;
    } else if (S->delta2 > 0.0 && tot[1] < S->delta2 * S->rmax2) {
      S->done = 1;  // hand over to the host for an FP64 reliable update
      S->need_update = 1;
    }
    S->beta = S->rz != 0.0 ? tot[0] / S->rz : 0.0;
    S->rz_prev = S->rz;
    S->rz = tot[0];
  }
}

template <typename T>
__global__ void __launch_bounds__(kVecBlock)
    k_cg_direction(int64_t n, T* __restrict__ p, const T* __restrict__ r,
                   const T* __restrict__ dinv, const SolverState* S) {
  if (S->done) return;
  const T beta = (T)S->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = fma(beta, p[i], dinv[i] * r[i]);
}

// FP32 update / direction with 16-byte vector accesses (all bases 16-byte aligned); the
// scalar tail covers n % 4 entries. Same arithmetic per entry as the scalar kernels.
__device__ __forceinline__ void upd1(float alpha, float& x, float& r, float p, float q, float d,
                                     float& rz, float& rr) {
  x = fmaf(alpha, p, x);
  r = fmaf(-alpha, q, r);
  rz = fmaf(r, d * r, rz);
  rr = fmaf(r, r, rr);
}

__global__ void __launch_bounds__(kVecBlock)
    k_cg_update4(int64_t n, float* __restrict__ x, float* __restrict__ r,
                 const float* __restrict__ p, const float* __restrict__ q,
                 const float* __restrict__ dinv, double* __restrict__ partials, SolverState* S) {
  __shared__ double sh[kVecBlock / 32];
  if (S->done) return;
  const float alpha = (float)S->alpha;
  float rz_t = 0.f, rr_t = 0.f;
  const int64_t n4 = n >> 2;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  // two float4 groups per trip so that ten 16-byte loads are in flight per thread
  for (int64_t i0 = tid; i0 < n4; i0 += 2 * nth) {
    float4 xv[2], rv[2], pv[2], qv[2], dv[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int64_t i = i0 + u * nth;
      if (i < n4) {
        xv[u] = reinterpret_cast<float4*>(x)[i];
        rv[u] = reinterpret_cast<float4*>(r)[i];
        pv[u] = __ldg(reinterpret_cast<const float4*>(p) + i);  // p, r, x stay L2-resident
        qv[u] = __ldcs(reinterpret_cast<const float4*>(q) + i);  // q is rewritten next
        dv[u] = __ldg(reinterpret_cast<const float4*>(dinv) + i);
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int64_t i = i0 + u * nth;
      if (i < n4) {
        upd1(alpha, xv[u].x, rv[u].x, pv[u].x, qv[u].x, dv[u].x, rz_t, rr_t);
        upd1(alpha, xv[u].y, rv[u].y, pv[u].y, qv[u].y, dv[u].y, rz_t, rr_t);
        upd1(alpha, xv[u].z, rv[u].z, pv[u].z, qv[u].z, dv[u].z, rz_t, rr_t);
        upd1(alpha, xv[u].w, rv[u].w, pv[u].w, qv[u].w, dv[u].w, rz_t, rr_t);
        reinterpret_cast<float4*>(x)[i] = xv[u];
        reinterpret_cast<float4*>(r)[i] = rv[u];
      }
    }
  }
  for (int64_t i = 4 * n4 + tid; i < n; i += nth) upd1(alpha, x[i], r[i], p[i], q[i], dinv[i], rz_t, rr_t);
  double rz = block_sum_f<kVecBlock>(rz_t, sh);
  double rr = block_sum_f<kVecBlock>(rr_t, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = rz;
    partials[2 * blockIdx.x + 1] = rr;
  }
  double tot[2];
  if (last_block_reduce<kVecBlock, 2>(&S->ticket[1], partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0) {
    S->iter += 1;
    S->rr = tot[1];
    if (!isfinite(tot[1]) || !isfinite(tot[0])) {
      S->done = 1;
      S->converged = 0;
    } else if (tot[1] <= S->tol2) {
      S->done = 1;
      S->converged = 1;
    } else if (S->iter >= S->maxit) {
      S->done = 1;
    } else if (S->delta2 > 0.0 && tot[1] < S->delta2 * S->rmax2) {
      S->done = 1;
      S->need_update = 1;
    }
    S->beta = S->rz != 0.0 ? tot[0] / S->rz : 0.0;
    S->rz_prev = S->rz;
    S->rz = tot[0];
  }
}

__global__ void __launch_bounds__(kVecBlock)
    k_cg_direction4(int64_t n, float* __restrict__ p, const float* __restrict__ r,
                    const float* __restrict__ dinv, const SolverState* S) {
  if (S->done) return;
  const float beta = (float)S->beta;
  const int64_t n4 = n >> 2;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < n4; i += nth) {
    float4 pv = reinterpret_cast<float4*>(p)[i];
    const float4 rv = __ldg(reinterpret_cast<const float4*>(r) + i);
    const float4 dv = __ldg(reinterpret_cast<const float4*>(dinv) + i);
    pv.x = fmaf(beta, pv.x, dv.x * rv.x);
    pv.y = fmaf(beta, pv.y, dv.y * rv.y);
    pv.z = fmaf(beta, pv.z, dv.z * rv.z);
    pv.w = fmaf(beta, pv.w, dv.w * rv.w);
    reinterpret_cast<float4*>(p)[i] = pv;
  }
  for (int64_t i = 4 * n4 + tid; i < n; i += nth) p[i] = fmaf(beta, p[i], dinv[i] * r[i]);
}

// CG start from x = 0: r = s*rhs (T), z = dinv r, p = z; partials of r.z and r.r.
template <typename T, typename TR>
__global__ void __launch_bounds__(kVecBlock)
    k_cg_init(int64_t n, const TR* __restrict__ rhs, double scale, T* __restrict__ x,
              T* __restrict__ r, T* __restrict__ p, const T* __restrict__ dinv,
              double* __restrict__ partials, SolverState* S, double rtol2) {
  __shared__ double sh[kVecBlock / 32];
  double rz = 0.0, rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T ri = (T)((double)rhs[i] * scale);
    x[i] = (T)0;
    r[i] = ri;
    const T zi = dinv ? dinv[i] * ri : ri;  // no diagonal: z = r (the caller preconditions)
    p[i] = zi;
    rz += (double)ri * (double)zi;
    rr += (double)ri * (double)ri;
  }
  rz = block_sum<kVecBlock>(rz, sh);
  rr = block_sum<kVecBlock>(rr, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = rz;
    partials[2 * blockIdx.x + 1] = rr;
  }
  double tot[2];
  if (last_block_reduce<kVecBlock, 2>(&S->ticket[1], partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0) {
    S->rz = tot[0];
    S->rr = tot[1];
    S->bb = tot[1];
    S->tol2 = rtol2 * tot[1];
    S->iter = 0;
    S->converged = 0;
    S->done = (tot[1] == 0.0) ? 1 : 0;
    if (tot[1] == 0.0) S->converged = 1;
  }
}

// FP64 residual of the refinement loop: r = b - A x (A in FP64), partial r.r.
__global__ void __launch_bounds__(kSpmvBlock)
    k_residual64(int64_t n, const int64_t* __restrict__ sptr, const int32_t* __restrict__ scol,
                 const double* __restrict__ sval, const double* __restrict__ x,
                 const double* __restrict__ b, double* __restrict__ r,
                 double* __restrict__ partials, double* out_rr, unsigned* ticket) {
  __shared__ double sh[kSpmvBlock / 32];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double d = 0.0;
  if (i < n) {
    const double ri = b[i] - sell_row<double, double>(i, sptr, scol, sval, x);
    r[i] = ri;
    d = ri * ri;
  }
  d = block_sum<kSpmvBlock>(d, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = d;
  double tot[1];
  if (last_block_reduce<kSpmvBlock, 1>(ticket, partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0)
    *out_rr = tot[0];
}

// The same residual from the CSR arrays, for solvers that need no sliced-ELL copy: LANES
// threads per row (strided over the row's entries, then a shuffle sum), rows of a warp
// advancing together so that every shuffle has the whole warp.
template <int LANES>
__global__ void __launch_bounds__(kSpmvBlock)
    k_residual64_csr(int64_t n, const int32_t* __restrict__ rowptr,
                     const int32_t* __restrict__ colval, const double* __restrict__ val,
                     const double* __restrict__ x, const double* __restrict__ b,
                     double* __restrict__ r, double* __restrict__ partials, double* out_rr,
                     unsigned* ticket) {
  constexpr int kRowsPerWarp = 32 / LANES;
  __shared__ double sh[kSpmvBlock / 32];
  const int lane = threadIdx.x & (LANES - 1);
  const int sub = (threadIdx.x & 31) / LANES;
  const int64_t warp = ((int64_t)blockIdx.x * kSpmvBlock + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * kSpmvBlock) >> 5;
  double d = 0.0;
  for (int64_t w0 = warp * kRowsPerWarp; w0 < n; w0 += nwarps * kRowsPerWarp) {
    const int64_t i = w0 + sub;
    double s = 0.0;
    if (i < n) {
      const int32_t e = __ldg(rowptr + i + 1);
      for (int32_t k = __ldg(rowptr + i) + lane; k < e; k += LANES)
        s = fma(__ldcs(val + k), __ldg(x + __ldcs(colval + k)), s);
    }
#pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (i < n && lane == 0) {
      const double ri = b[i] - s;
      r[i] = ri;
      d += ri * ri;
    }
  }
  d = block_sum<kSpmvBlock>(d, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = d;
  double tot[1];
  if (last_block_reduce<kSpmvBlock, 1>(ticket, partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0)
    *out_rr = tot[0];
}

// The same FP64 residual for a matrix with the closed-form lattice pattern of a 3-D
// Cartesian Q1 grid (rows = interior nodes in node order, each row's columns its interior
// neighbours among the 27 in (dz, dy, dx) order): the column ids follow from the row's
// position, so only the values stream from memory (8 instead of 12 bytes per entry). A warp
// takes 32 consecutive rows of one x-line, whose values are one contiguous slice: it copies
// the slice into shared memory with coalesced loads, then each lane forms its row from there
// with the neighbours' x. Persistent grid; x-lines dealt to warps in a fixed order, so the
// reduction is deterministic.
// ZF: the matrix's face-class entries (neighbours along one axis) are exact zeros (the
// class-sum values of cubic cells): their products are skipped, 21 FP64 FMAs per interior row
// instead of 27, the same sum
template <bool ZF>
__global__ void __launch_bounds__(kSpmvBlock)
    k_residual64_lattice(int m0, int m1, int m2, const int32_t* __restrict__ rowptr,
                         const double* __restrict__ val, const double* __restrict__ x,
                         const double* __restrict__ b, double* __restrict__ r,
                         float* __restrict__ r32, double* __restrict__ partials, double* out_rr,
                         unsigned* ticket) {
  extern __shared__ double stage_all[];
  __shared__ double sh[kSpmvBlock / 32];
  const int lane = (int)(threadIdx.x & 31), wib = (int)(threadIdx.x >> 5);
  double* stage = stage_all + wib * (32 * 27);
  const int tx = (m0 + 31) / 32;
  const int64_t ntask = (int64_t)tx * m1 * m2;
  const int64_t nwarps = (int64_t)gridDim.x * (kSpmvBlock / 32);
  const int64_t sy = m0, sz = (int64_t)m0 * m1;
  double d = 0.0;
  for (int64_t task = (int64_t)blockIdx.x * (kSpmvBlock / 32) + wib; task < ntask;
       task += nwarps) {
    const int64_t line = task / tx;
    const int i = (int)(task - line * tx) * 32 + lane;
    const int k = (int)(line / m1), j = (int)(line - (int64_t)k * m1);
    const bool act = i < m0;
    const int64_t row = (int64_t)(act ? i : m0 - 1) + sy * j + sz * k;
    int32_t rp = 0, rpn = 0;
    if (act) {
      rp = __ldg(rowptr + row);
      rpn = __ldg(rowptr + row + 1);
    }
    const int32_t rp0 = __shfl_sync(0xffffffffu, rp, 0);
    int32_t rend = rpn;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
      rend = max(rend, __shfl_xor_sync(0xffffffffu, rend, off));
    for (int q = lane; q < rend - rp0; q += 32) stage[q] = __ldcs(val + rp0 + q);
    __syncwarp();
    if (act) {
      const bool okx[3] = {i > 0, true, i < m0 - 1};
      const bool oky[3] = {j > 0, true, j < m1 - 1};
      const bool okz[3] = {k > 0, true, k < m2 - 1};
      int pos = rp - rp0;
      double s = 0.0;
#pragma unroll
      for (int dz = 0; dz < 3; ++dz)
#pragma unroll
        for (int dy = 0; dy < 3; ++dy)
#pragma unroll
          for (int dx = 0; dx < 3; ++dx)
            if (okz[dz] && oky[dy] && okx[dx]) {
              const int axes = (dx != 1) + (dy != 1) + (dz != 1);
              if (!ZF || axes != 1)
                s = fma(stage[pos], __ldg(x + row + (dx - 1) + sy * (dy - 1) + sz * (dz - 1)),
                        s);
              ++pos;
            }
      const double ri = b[row] - s;
      if (r32)  // the FP32 residual the inner iterations restart from
        r32[row] = (float)ri;
      else if (r)
        r[row] = ri;
      d = fma(ri, ri, d);
    }
    __syncwarp();
  }
  d = block_sum<kSpmvBlock>(d, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = d;
  double tot[1];
  if (last_block_reduce<kSpmvBlock, 1>(ticket, partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0)
    *out_rr = tot[0];
}

// x64 += s * d32
__global__ void k_refine_update(int64_t n, double* __restrict__ x, const float* __restrict__ d,
                                double s) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] += s * (double)d[i];
}

__global__ void k_dot_self(int64_t n, const double* __restrict__ v, double* __restrict__ partials,
                           double* out, unsigned* ticket) {
  __shared__ double sh[kVecBlock / 32];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s += v[i] * v[i];
  s = block_sum<kVecBlock>(s, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
  double tot[1];
  if (last_block_reduce<kVecBlock, 1>(ticket, partials, gridDim.x, tot, sh) && threadIdx.x == 0)
    *out = tot[0];
}

// ---- reliable updates of the mixed-precision CG ---------------------------------------------
// x64 += x32; x32 = 0
__global__ void k_merge(int64_t n, double* __restrict__ x64, float* __restrict__ x32) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    x64[i] += (double)x32[i];
    x32[i] = 0.f;
  }
}

// After r64 = b - A64 x64: stop if converged; else r32 = r64, rz = r.Dr, rp = r.p, and the
// last block sets c = rp/rz (to re-orthogonalise p against the new r) and beta = rz/rz_prev.
__global__ void __launch_bounds__(kVecBlock)
    k_restart32(int64_t n, const double* __restrict__ r64, float* __restrict__ r32,
                const float* __restrict__ p, const float* __restrict__ dinv,
                double* __restrict__ partials, SolverState* S) {
  __shared__ double sh[kVecBlock / 32];
  if (S->rr64 <= S->tol2) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      S->converged = 1;
      S->done = 1;
      S->need_update = 0;
    }
    return;
  }
  double rz = 0.0, rp = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float ri = (float)r64[i];
    r32[i] = ri;
    rz += (double)ri * (double)(dinv[i] * ri);
    rp += (double)ri * (double)p[i];
  }
  rz = block_sum<kVecBlock>(rz, sh);
  rp = block_sum<kVecBlock>(rp, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = rz;
    partials[2 * blockIdx.x + 1] = rp;
  }
  double tot[2];
  if (last_block_reduce<kVecBlock, 2>(&S->ticket[1], partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0) {
    S->alpha = tot[0] != 0.0 ? tot[1] / tot[0] : 0.0;  // c (reused field)
    S->beta = S->rz_prev != 0.0 ? tot[0] / S->rz_prev : 0.0;
    S->rz = tot[0];
    S->rmax2 = S->rr64;
    S->rr = S->rr64;
    S->need_update = 0;
    S->converged = 0;
    S->done = (S->iter >= S->maxit || !isfinite(tot[0])) ? 1 : 0;
  }
}

// k_restart32 for the padded layout: r32[pad(i)] = r64[i], dots r.Dr and r.p over the rows
__global__ void __launch_bounds__(kVecBlock)
    k_restart32_pad(LatticeQ1Op op, int64_t n, const double* __restrict__ r64,
                    float* __restrict__ r32, const float* __restrict__ p,
                    const float* __restrict__ dinv, double* __restrict__ partials,
                    SolverState* S) {
  __shared__ double sh[kVecBlock / 32];
  if (S->rr64 <= S->tol2) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      S->converged = 1;
      S->done = 1;
      S->need_update = 0;
    }
    return;
  }
  double rz = 0.0, rp = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = dof_to_pad(op, i);
    const float ri = (float)r64[i];
    r32[j] = ri;
    rz += (double)ri * (double)(dinv[j] * ri);
    rp += (double)ri * (double)p[j];
  }
  rz = block_sum<kVecBlock>(rz, sh);
  rp = block_sum<kVecBlock>(rp, sh);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = rz;
    partials[2 * blockIdx.x + 1] = rp;
  }
  double tot[2];
  if (last_block_reduce<kVecBlock, 2>(&S->ticket[1], partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0) {
    S->alpha = tot[0] != 0.0 ? tot[1] / tot[0] : 0.0;  // c (reused field)
    S->beta = S->rz_prev != 0.0 ? tot[0] / S->rz_prev : 0.0;
    S->rz = tot[0];
    S->rmax2 = S->rr64;
    S->rr = S->rr64;
    S->need_update = 0;
    S->converged = 0;
    S->done = (S->iter >= S->maxit || !isfinite(tot[0])) ? 1 : 0;
  }
}

// p = beta (p - c z) + z with z = D r (c in S->alpha)
__global__ void k_restart_dir(int64_t n, float* __restrict__ p, const float* __restrict__ r,
                              const float* __restrict__ dinv, const SolverState* S) {
  if (S->done) return;
  const float c = (float)S->alpha, beta = (float)S->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float z = dinv[i] * r[i];
    p[i] = fma(beta, p[i] - c * z, z);
  }
}

__global__ void k_set_reliable(SolverState* S, double delta2) {
  S->delta2 = delta2;
  S->rmax2 = S->bb;
  S->rr64 = S->bb;
}

// ---- flexible CG (FCG(1)) with a variable preconditioner --------------------------------------
//   x += a p; r -= a q; z = M(r); beta = -(z.q)/(p.q); p = z + beta p; q = A p; a = (p.r)/(p.q)
// (Notay's truncated flexible CG with one previous direction). FP32 vectors; x and the true
// residual in FP64 through reliable updates, as the mixed CG.

// The conditions of the device-driven loop's WHILE node (repeat while not done) and IF node
// (the reliable update is due), set by the kernels that decide them; on = 0 outside that graph.
struct LoopConds {
  cudaGraphConditionalHandle w, i;
  int on;
};
__device__ __forceinline__ void set_conds(const LoopConds& c, const SolverState* S) {
  if (!c.on) return;
  cudaGraphSetConditional(c.i, S->need_update && !S->done ? 1u : 0u);
  cudaGraphSetConditional(c.w, S->done ? 0u : 1u);
}

// After an update with the FP32 residual rr: count the iteration, then stop (not finite,
// converged, maxit) or ask for a reliable update (residual dropped by delta; with
// defer_update, in the device loop, also at convergence, which the FP64 residual confirms)
__device__ __forceinline__ void fcg_decide(SolverState* S, double rr) {
  S->iter += 1;
  S->rr = rr;
  if (!isfinite(rr)) {
    S->done = 1;
  } else if (rr <= S->tol2) {
    if (S->defer_update) {
      S->need_update = 1;
    } else {
      S->done = 1;
      S->converged = 1;
    }
  } else if (S->iter >= S->maxit) {
    S->done = 1;
  } else if (S->delta2 > 0.0 && rr < S->delta2 * S->rmax2) {
    S->need_update = 1;
    if (!S->defer_update) S->done = 1;
  }
}
__global__ void __launch_bounds__(kVecBlock)
    k_fcg_update(int64_t n, float* __restrict__ x, float* __restrict__ r,
                 const float* __restrict__ p, const float* __restrict__ q,
                 double* __restrict__ partials, SolverState* S, LoopConds c) {
  __shared__ double sh[kVecBlock / 32];
  if (S->done) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_conds(c, S);
    return;
  }
  const float a = (float)S->alpha;
  float rr_t = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = fmaf(a, p[i], x[i]);
    const float ri = fmaf(-a, q[i], r[i]);
    r[i] = ri;
    rr_t = fmaf(ri, ri, rr_t);
  }
  const double rr = block_sum<kVecBlock>((double)rr_t, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = rr;
  double tot[1];
  if (last_block_reduce<kVecBlock, 1>(&S->ticket[1], partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0) {
    fcg_decide(S, tot[0]);
    set_conds(c, S);
  }
}

__global__ void k_jacobi_apply(int64_t n, const float* __restrict__ r,
                               const float* __restrict__ dinv, float* __restrict__ z,
                               const SolverState* S) {
  if (S && S->done) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    z[i] = dinv[i] * r[i];
}

// beta = -(z.q) / (p.q)
__global__ void __launch_bounds__(kVecBlock)
    k_fcg_beta(int64_t n, const float* __restrict__ z, const float* __restrict__ q,
               double* __restrict__ partials, SolverState* S) {
  __shared__ double sh[kVecBlock / 32];
  if (S->done) return;
  float t = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    t = fmaf(z[i], q[i], t);
  const double d = block_sum<kVecBlock>((double)t, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = d;
  double tot[1];
  if (last_block_reduce<kVecBlock, 1>(&S->ticket[3], partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0)
    S->beta = S->pq != 0.0 ? -tot[0] / S->pq : 0.0;
}

__global__ void k_fcg_dir(int64_t n, float* __restrict__ p, const float* __restrict__ z,
                          const SolverState* S) {
  if (S->done) return;
  const float beta = (float)S->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = fmaf(beta, p[i], z[i]);
}

// q = A p, partials of p.q and p.r; alpha = (p.r)/(p.q)
template <class Op>
__global__ void __launch_bounds__(kSpmvBlock)
    k_fcg_spmv(int64_t n, Op op, const float* __restrict__ p, float* __restrict__ q,
               const float* __restrict__ r, double* __restrict__ partials, SolverState* S) {
  __shared__ double sh[kSpmvBlock / 32];
  if (S->done) return;
  const int64_t i = op.row_index();
  float pq = 0.f, pr = 0.f;
  if (i >= 0 && i < n) {
    const float y = op.row(i, p);
    q[i] = y;
    pq = p[i] * y;
    pr = p[i] * r[i];
  }
  const double dpq = block_sum_f<kSpmvBlock>(pq, sh);
  const double dpr = block_sum_f<kSpmvBlock>(pr, sh);
  if (threadIdx.x == 0) {
    partials[2 * block_linear()] = dpq;
    partials[2 * block_linear() + 1] = dpr;
  }
  double tot[2];
  if (last_block_reduce<kSpmvBlock, 2>(&S->ticket[0], partials, grid_blocks(), tot, sh) &&
      threadIdx.x == 0) {
    S->pq = tot[0];
    S->alpha = tot[0] != 0.0 ? tot[1] / tot[0] : 0.0;
  }
}

// r32 = (float) r64 after a reliable update (no orthogonalisation needed: FCG takes alpha from
// p.r and beta from z.q with the current vectors); stop when the FP64 residual meets rtol.
// (r64 null: the FP64 residual kernel wrote r32 itself)
__global__ void k_fcg_restart(int64_t n, const double* __restrict__ r64, float* __restrict__ r32,
                              SolverState* S, LoopConds c) {
  const bool conv = S->rr64 <= S->tol2;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r64 && i < n && !conv;
       i += (int64_t)gridDim.x * blockDim.x)
    r32[i] = (float)r64[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    S->need_update = 0;
    S->updates += 1;
    if (conv) {
      S->converged = 1;
      S->done = 1;
    } else {
      S->rmax2 = S->rr64;
      S->rr = S->rr64;
      S->converged = 0;
      S->done = S->iter >= S->maxit ? 1 : 0;
    }
    set_conds(c, S);
  }
}

// The same three FCG vector steps over float4 groups (16-byte aligned vectors), two groups in
// flight per thread per trip; a scalar tail covers n % 4 entries. Same arithmetic per entry.
__global__ void __launch_bounds__(kVecBlock)
    k_fcg_update4(int64_t n, float* __restrict__ x, float* __restrict__ r,
                  const float* __restrict__ p, const float* __restrict__ q,
                  double* __restrict__ partials, SolverState* S, LoopConds c) {
  __shared__ double sh[kVecBlock / 32];
  if (S->done) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_conds(c, S);
    return;
  }
  const float a = (float)S->alpha;
  float rr_t = 0.f;
  const int64_t n4 = n >> 2;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = tid; i0 < n4; i0 += 2 * nth) {
    float4 xv[2], rv[2], pv[2], qv[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int64_t i = i0 + u * nth;
      if (i < n4) {
        xv[u] = reinterpret_cast<float4*>(x)[i];
        rv[u] = reinterpret_cast<float4*>(r)[i];
        pv[u] = __ldg(reinterpret_cast<const float4*>(p) + i);
        qv[u] = __ldg(reinterpret_cast<const float4*>(q) + i);
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int64_t i = i0 + u * nth;
      if (i < n4) {
        float* xs = &xv[u].x;
        float* rs = &rv[u].x;
        const float* ps = &pv[u].x;
        const float* qs = &qv[u].x;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          xs[c] = fmaf(a, ps[c], xs[c]);
          rs[c] = fmaf(-a, qs[c], rs[c]);
          rr_t = fmaf(rs[c], rs[c], rr_t);
        }
        reinterpret_cast<float4*>(x)[i] = xv[u];
        reinterpret_cast<float4*>(r)[i] = rv[u];
      }
    }
  }
  for (int64_t i = 4 * n4 + tid; i < n; i += nth) {
    x[i] = fmaf(a, p[i], x[i]);
    const float ri = fmaf(-a, q[i], r[i]);
    r[i] = ri;
    rr_t = fmaf(ri, ri, rr_t);
  }
  const double rr = block_sum<kVecBlock>((double)rr_t, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = rr;
  double tot[1];
  if (last_block_reduce<kVecBlock, 1>(&S->ticket[1], partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0) {
    fcg_decide(S, tot[0]);
    set_conds(c, S);
  }
}

__global__ void __launch_bounds__(kVecBlock)
    k_fcg_beta4(int64_t n, const float* __restrict__ z, const float* __restrict__ q,
                double* __restrict__ partials, SolverState* S) {
  __shared__ double sh[kVecBlock / 32];
  if (S->done) return;
  float t = 0.f;
  const int64_t n4 = n >> 2;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = tid; i0 < n4; i0 += 2 * nth) {
    float4 zv[2], qv[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int64_t i = i0 + u * nth;
      if (i < n4) {
        zv[u] = __ldg(reinterpret_cast<const float4*>(z) + i);
        qv[u] = __ldg(reinterpret_cast<const float4*>(q) + i);
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (i0 + u * nth < n4) {
        t = fmaf(zv[u].x, qv[u].x, t);
        t = fmaf(zv[u].y, qv[u].y, t);
        t = fmaf(zv[u].z, qv[u].z, t);
        t = fmaf(zv[u].w, qv[u].w, t);
      }
  }
  for (int64_t i = 4 * n4 + tid; i < n; i += nth) t = fmaf(z[i], q[i], t);
  const double d = block_sum<kVecBlock>((double)t, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = d;
  double tot[1];
  if (last_block_reduce<kVecBlock, 1>(&S->ticket[3], partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0)
    S->beta = S->pq != 0.0 ? -tot[0] / S->pq : 0.0;
}

__global__ void __launch_bounds__(kVecBlock)
    k_fcg_dir4(int64_t n, float* __restrict__ p, const float* __restrict__ z,
               const SolverState* S) {
  if (S->done) return;
  const float beta = (float)S->beta;
  const int64_t n4 = n >> 2;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = tid; i0 < n4; i0 += 2 * nth) {
    float4 pv[2], zv[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int64_t i = i0 + u * nth;
      if (i < n4) {
        pv[u] = reinterpret_cast<float4*>(p)[i];
        zv[u] = __ldg(reinterpret_cast<const float4*>(z) + i);
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int64_t i = i0 + u * nth;
      if (i < n4) {
        pv[u].x = fmaf(beta, pv[u].x, zv[u].x);
        pv[u].y = fmaf(beta, pv[u].y, zv[u].y);
        pv[u].z = fmaf(beta, pv[u].z, zv[u].z);
        pv[u].w = fmaf(beta, pv[u].w, zv[u].w);
        reinterpret_cast<float4*>(p)[i] = pv[u];
      }
    }
  }
  for (int64_t i = 4 * n4 + tid; i < n; i += nth) p[i] = fmaf(beta, p[i], z[i]);
}

// FCG start from x = 0 over float4 groups (16-byte aligned b, x, r): x = 0, r = (float) b,
// and ||b||^2 in FP64 (the relative residual's denominator; it also sets the stopping
// threshold and the starting r.r); z = r is left to the caller's preconditioner
__global__ void __launch_bounds__(kVecBlock)
    k_fcg_init4(int64_t n, const double* __restrict__ b, float* __restrict__ x,
                float* __restrict__ r, double* __restrict__ partials, SolverState* S,
                double rtol2) {
  __shared__ double sh[kVecBlock / 32];
  double bb_t = 0.0;
  const int64_t n4 = n >> 2;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < n4; i += nth) {
    const double2 b0 = __ldg(reinterpret_cast<const double2*>(b) + 2 * i);
    const double2 b1 = __ldg(reinterpret_cast<const double2*>(b) + 2 * i + 1);
    const float4 rv = make_float4((float)b0.x, (float)b0.y, (float)b1.x, (float)b1.y);
    reinterpret_cast<float4*>(r)[i] = rv;
    reinterpret_cast<float4*>(x)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    bb_t = fma(b0.x, b0.x, bb_t);
    bb_t = fma(b0.y, b0.y, bb_t);
    bb_t = fma(b1.x, b1.x, bb_t);
    bb_t = fma(b1.y, b1.y, bb_t);
  }
  for (int64_t i = 4 * n4 + tid; i < n; i += nth) {
    const double bi = b[i];
    r[i] = (float)bi;
    x[i] = 0.f;
    bb_t = fma(bi, bi, bb_t);
  }
  const double bb = block_sum<kVecBlock>(bb_t, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = bb;
  double tot[1];
  if (last_block_reduce<kVecBlock, 1>(&S->ticket[1], partials, gridDim.x, tot, sh) &&
      threadIdx.x == 0) {
    S->rz = tot[0];
    S->rr = tot[0];
    S->bb = tot[0];
    S->tol2 = rtol2 * tot[0];
    S->iter = 0;
    S->converged = 0;
    S->done = (tot[0] == 0.0) ? 1 : 0;
    if (tot[0] == 0.0) S->converged = 1;
  }
}

// x64 += x32; x32 = 0 over float4 groups (16-byte aligned x64 and x32)
__global__ void k_merge4(int64_t n, double* __restrict__ x64, float* __restrict__ x32) {
  const int64_t n4 = n >> 2;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < n4; i += nth) {
    const float4 d = reinterpret_cast<const float4*>(x32)[i];
    double2 a0 = reinterpret_cast<double2*>(x64)[2 * i];
    double2 a1 = reinterpret_cast<double2*>(x64)[2 * i + 1];
    a0.x += (double)d.x;
    a0.y += (double)d.y;
    a1.x += (double)d.z;
    a1.y += (double)d.w;
    reinterpret_cast<double2*>(x64)[2 * i] = a0;
    reinterpret_cast<double2*>(x64)[2 * i + 1] = a1;
    reinterpret_cast<float4*>(x32)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  for (int64_t i = 4 * n4 + tid; i < n; i += nth) {
    x64[i] += (double)x32[i];
    x32[i] = 0.f;
  }
}

// the flexible CG's settings in the zeroed state, after its start (which sets ||b||^2)
__global__ void k_fcg_setup(SolverState* S, double delta2, int maxit, int defer) {
  S->delta2 = delta2;
  S->rmax2 = S->bb;
  S->rr64 = S->bb;
  S->maxit = maxit;
  S->defer_update = defer;
}

// ---- host drivers -------------------------------------------------------------------------
// ||r|| / ||b|| from the squares: not finite when either is (a NaN in b must not read as a
// zero residual), 0 for b = 0
static double rel_residual(double rr, double bb) {
  if (!std::isfinite(rr) || !std::isfinite(bb)) return std::numeric_limits<double>::quiet_NaN();
  return bb > 0.0 ? std::sqrt(rr / bb) : 0.0;
}

struct SolverWork {
  SolverState* S;      // device
  SolverState* hS;     // pinned host mirror
  double* partials;    // device
  unsigned* tickets;   // device (inside S)
};

// (stage_err: the device error word comes along, for the caller's check after this wait)
static int read_state(gfe_ctx* ctx, SolverWork& w, bool flush = true, bool stage_err = false) {
  GFE_CUDA_TRY(cudaMemcpyAsync(w.hS, w.S, sizeof(SolverState), cudaMemcpyDeviceToHost,
                               ctx->stream));
  if (stage_err) GFE_TRY(stage_device_error(ctx));
  GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return flush ? timer_flush(ctx) : GFE_OK;
}

// Runs PCG on A (values of type T) for rhs*scale from x=0 until done; returns iterations.
// Launches chunks of CG iterations until the device sets `done`.
template <typename T, class Op>
static int iterate(gfe_ctx* ctx, gfe_matrix* A, const Op& op, const T* dinv, T* x, T* r, T* p,
                   T* q, int check_every, SolverWork& w, int64_t nvec = -1) {
  // n: length of the vectors (the rows, or the padded lattice size)
  const int64_t n = nvec >= 0 ? nvec : A->nrows;
  const dim3 gs = op.grid(n);
  // FP32 vectors with 16-byte aligned bases take the 4-wide update kernels. Four blocks per
  // SM with two 16-byte groups in flight per thread keep enough bytes in flight to stream at
  // HBM rate, while the per-block reduction cost (barriers, fence, ticket) stays small.
  bool vec4 = false;
  if constexpr (sizeof(T) == 4) {
    vec4 = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(r) |
             reinterpret_cast<uintptr_t>(p) | reinterpret_cast<uintptr_t>(q) |
             reinterpret_cast<uintptr_t>(dinv)) & 15) == 0;
  }
  const unsigned gv = vec4 ? (unsigned)std::max<int64_t>(
                                 1, std::min<int64_t>((n + 1023) / 1024, ctx->num_sms * 4))
                           : (unsigned)(ctx->num_sms * 4);
  // Without kernel timing a chunk of iterations is captured once into a CUDA graph (cached in
  // the context while its launch parameters match) and replayed. With timing on, every
  // iteration is launched directly with CUDA events around the SpMV; launches after the
  // converged iteration (they return at once) are dropped from the timing.
  // the lattice operator's halos arrive by tensor-map copies where the encoder is available
  CUtensorMap tmap_p, tmap_k;
  bool tma = false;
  if constexpr (std::is_same<Op, LatticeQ1Op>::value) {
    tma = lattice_tensor_maps(op, reinterpret_cast<const float*>(p), &tmap_p, &tmap_k);
    // six resident blocks of 15 KB each: prefer shared memory over L1 for this kernel
    if (tma)
      GFE_CUDA_TRY(cudaFuncSetAttribute(k_lattice_spmv_tma,
                                        cudaFuncAttributePreferredSharedMemoryCarveout,
                                        (int)cudaSharedmemCarveoutMaxShared));
  }
  auto launch_spmv = [&]() {
    if constexpr (std::is_same<Op, LatticeQ1Op>::value) {
      if (tma)
        k_lattice_spmv_tma<<<op.grid_k(kTmaK), kSpmvBlock, 0, ctx->stream>>>(
            tmap_p, tmap_k, op, q, w.partials, w.S, ctx->d_err, ctx->first_wait_ns);
      else
        k_lattice_spmv<false, true><<<gs, kSpmvBlock, 0, ctx->stream>>>(op, p, q, nullptr,
                                                                        w.partials, w.S);
    } else
      k_cg_spmv_dot<T, Op><<<gs, kSpmvBlock, 0, ctx->stream>>>(n, op, p, q, w.partials, w.S);
  };
  auto launch_vec = [&](unsigned g) {
    if constexpr (sizeof(T) == 4) {
      if (vec4) {
        k_cg_update4<<<g, kVecBlock, 0, ctx->stream>>>(n, x, r, p, q, dinv, w.partials, w.S);
        k_cg_direction4<<<g, kVecBlock, 0, ctx->stream>>>(n, p, r, dinv, w.S);
        return;
      }
    }
    k_cg_update<T><<<g, kVecBlock, 0, ctx->stream>>>(n, x, r, p, q, dinv, w.partials, w.S);
    k_cg_direction<T><<<g, kVecBlock, 0, ctx->stream>>>(n, p, r, dinv, w.S);
  };
  const bool timing = ctx->timer.enabled;
  const int kind = sizeof(T) == 4 ? GFE_KT_SPMV32 : GFE_KT_SPMV64;
  cudaGraphExec_t exec = nullptr;
  if (!timing) {
    uint64_t key = 1469598103934665603ull;  // FNV-1a over what the launches depend on
    auto mix = [&key](const void* ptr, size_t nb) {
      const unsigned char* c = static_cast<const unsigned char*>(ptr);
      for (size_t i = 0; i < nb; ++i) key = (key ^ c[i]) * 1099511628211ull;
    };
    const void* ptrs[] = {x, r, p, q, dinv, w.partials, w.S};
    mix(ptrs, sizeof(ptrs));
    mix(&op, sizeof(Op));
    mix(&n, sizeof(n));
    mix(&check_every, sizeof(check_every));
    mix(&gv, sizeof(gv));
    mix(&vec4, sizeof(vec4));
    mix(&tma, sizeof(tma));
    mix(&ctx->first_wait_ns, sizeof(ctx->first_wait_ns));
    const int tsize = (int)sizeof(T);
    mix(&tsize, sizeof(tsize));
    if (ctx->cg_exec && ctx->cg_key == key) exec = ctx->cg_exec;
    if (!exec) {
      if (ctx->cg_exec) {
        cudaGraphExecDestroy(ctx->cg_exec);
        ctx->cg_exec = nullptr;
      }
      cudaGraph_t graph = nullptr;
      GFE_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      for (int k = 0; k < check_every; ++k) {
        launch_spmv();
        launch_vec(gv);
      }
      const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
      if (ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return set_error(GFE_ERR_CUDA, "solve: graph capture failed: %s",
                         cudaGetErrorString(ce));
      }
      const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ie != cudaSuccess)
        return set_error(GFE_ERR_CUDA, "solve: graph instantiate failed: %s",
                         cudaGetErrorString(ie));
      ctx->cg_exec = exec;
      ctx->cg_key = key;
    }
  }
  int st = GFE_OK;
  for (;;) {
    const int iter0 = w.hS->iter;
    if (exec) {
      const cudaError_t le = cudaGraphLaunch(exec, ctx->stream);
      if (le != cudaSuccess) {
        st = set_error(GFE_ERR_CUDA, "solve: graph launch: %s", cudaGetErrorString(le));
        break;
      }
      ctx->launches += 3 * check_every;
    } else {
      for (int k = 0; k < check_every; ++k) {
        timer_begin(ctx, kind);
        launch_spmv();
        timer_end(ctx);
        timer_begin(ctx, GFE_KT_VECTOR);
        launch_vec(gv);
        timer_end(ctx);
        ctx->launches += 3;
      }
      const cudaError_t le = cudaGetLastError();
      if (le != cudaSuccess) {
        st = set_error(GFE_ERR_CUDA, "solve: launch: %s", cudaGetErrorString(le));
        break;
      }
    }
    st = read_state(ctx, w, false);
    if (st != GFE_OK) break;
    if (timing) timer_drop_last(ctx, 2 * (check_every - (w.hS->iter - iter0)));
    st = timer_flush(ctx);
    if (st != GFE_OK || w.hS->done) break;
  }
  return st;
}

template <typename T>
static int run_pcg(gfe_ctx* ctx, gfe_matrix* A, const T* sval, const T* dinv, const void* rhs,
                   bool rhs_is_double, double scale, T* x, T* r, T* p, T* q, double rtol,
                   int maxit, int check_every, SolverWork& w, int* iters, int* converged) {
  const int64_t n = A->nrows;
  const unsigned gv = (unsigned)(ctx->num_sms * 4);
  GFE_CUDA_TRY(cudaMemsetAsync(w.S, 0, sizeof(SolverState), ctx->stream));
  int maxit_field = maxit;
  GFE_CUDA_TRY(cudaMemcpyAsync(&w.S->maxit, &maxit_field, sizeof(int), cudaMemcpyHostToDevice,
                               ctx->stream));
  if (rhs_is_double)
    k_cg_init<T, double><<<gv, kVecBlock, 0, ctx->stream>>>(
        n, (const double*)rhs, scale, x, r, p, dinv, w.partials, w.S, rtol * rtol);
  else
    k_cg_init<T, float><<<gv, kVecBlock, 0, ctx->stream>>>(n, (const float*)rhs, scale, x, r, p,
                                                          dinv, w.partials, w.S, rtol * rtol);
  ctx->launches++;
  w.hS->iter = 0;
  SellOp<T> op{A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(), sval};
  GFE_TRY((iterate<T, SellOp<T>>(ctx, A, op, dinv, x, r, p, q, check_every, w)));
  const int done_iters = w.hS->iter;
  *iters = done_iters;
  *converged = w.hS->converged;
  return GFE_OK;
}

__global__ void k_axpy64(int64_t n, double* __restrict__ x, const double* __restrict__ d) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] += d[i];
}

struct GuessStats {
  double rr, bb;
  unsigned ticket[2];
};

// Solve from the values in d_x (a restart): r0 = b - A x0 in FP64, the chosen solver runs on
// A d = r0 from d = 0 with its tolerance scaled so that ||r0 - A d|| <= rtol ||b||, then
// x = x0 + d and the report's relative residual is recomputed on x against b.
static int solve_from_guess(gfe_ctx* ctx, gfe_matrix* A, gfe_learned_pc* pc, bool fcg,
                            const gfe_solver_opts* o, const double* d_b, double* d_x,
                            gfe_solve_report* rep) {
  GFE_TRY(build_solver_plan(ctx, A));
  const int64_t n = A->nrows;
  const unsigned gs = grid_for(n, kSpmvBlock);
  const unsigned gv = (unsigned)(ctx->num_sms * 4);
  const size_t n8 = sizeof(double) * (size_t)(n > 0 ? n : 1);
  DevBuf tmp(ctx);
  const size_t np = (size_t)std::max<unsigned>(gs, gv) + 64;
  GFE_TRY(tmp.reserve(2 * n8 + sizeof(double) * np + 256));
  double* r0 = tmp.as<double>();
  double* d = r0 + (n > 0 ? n : 1);
  double* partials = d + (n > 0 ? n : 1);
  GuessStats* st = reinterpret_cast<GuessStats*>(partials + np);
  GuessStats h;
  auto residual = [&](const double* x) -> int {
    GFE_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(GuessStats), ctx->stream));
    k_residual64<<<gs, kSpmvBlock, 0, ctx->stream>>>(
        n, A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(), A->sell_val64.as<double>(), x,
        d_b, r0, partials, &st->rr, &st->ticket[0]);
    k_dot_self<<<gv, kVecBlock, 0, ctx->stream>>>(n, d_b, partials, &st->bb, &st->ticket[1]);
    ctx->launches += 2;
    GFE_CUDA_TRY(cudaGetLastError());
    return copy_out(ctx, &h, st, sizeof(GuessStats));
  };
  GFE_TRY(residual(d_x));
  memset(rep, 0, sizeof(*rep));
  if (!std::isfinite(h.rr)) {
    rep->status = GFE_ERR_NONFINITE;
    return set_error(GFE_ERR_NONFINITE, "solve: the initial guess gives a non-finite residual");
  }
  if (h.bb == 0.0 || h.rr <= o->rtol * o->rtol * h.bb) {
    if (h.bb == 0.0) GFE_CUDA_TRY(cudaMemsetAsync(d_x, 0, n8, ctx->stream));
    rep->converged = 1;
    rep->relres = rel_residual(h.rr, h.bb);
    return GFE_OK;
  }
  gfe_solver_opts o2 = *o;
  o2.initial_guess = 0;
  o2.rtol = o->rtol * std::sqrt(h.bb / h.rr);
  GFE_TRY(fcg ? solve_fcg(ctx, A, pc, &o2, r0, d, rep) : solve(ctx, A, &o2, r0, d, rep));
  k_axpy64<<<gv, kVecBlock, 0, ctx->stream>>>(n, d_x, d);
  ctx->launches++;
  GFE_TRY(residual(d_x));
  rep->relres = rel_residual(h.rr, h.bb);
  rep->converged = std::isfinite(rep->relres) && rep->relres <= o->rtol * (1.0 + 1e-6);
  return GFE_OK;
}

int solve(gfe_ctx* ctx, gfe_matrix* A, const gfe_solver_opts* o, const double* d_b,
          double* d_x, gfe_solve_report* rep) {
  if (A->nrows != A->ncols)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "solve: matrix is not square");
  if (o->initial_guess) return solve_from_guess(ctx, A, nullptr, false, o, d_b, d_x, rep);
  GFE_TRY(build_solver_plan(ctx, A));
  const int64_t n = A->nrows;
  const int check_every = o->check_every > 0 ? o->check_every : 25;
  const int maxit = o->maxiter > 0 ? o->maxiter : 100000;
  // work vectors: FP64 r, p, q (CG) or FP64 r + FP32 x, r, p, q (IR)
  const size_t n8 = sizeof(double) * (size_t)(n > 0 ? n : 1);
  // FP32 vectors at a stride padded to 64 entries: every base 16-byte aligned (4-wide kernels)
  const int64_t npad = (n + 63) & ~(int64_t)63;
  GFE_TRY(ctx->scratch[SCR_SOLVER].reserve(n8 * 3 + 64));
  GFE_TRY(ctx->scratch[SCR_SOLVER2].reserve(sizeof(float) * (size_t)(npad > 0 ? npad : 64) * 4 +
                                            256));
  bool lattice = false;
  GFE_TRY(lattice_ready(ctx, A, &lattice));
  size_t nblk = grid_for(n, kSpmvBlock);
  // mixed CG on the lattice operator keeps its FP32 vectors (and D^-1) in the zero-halo padded
  // lattice layout, stride nlat
  const bool pad_layout = lattice && o->method == GFE_SOLVER_MIXED_CG;
  const int64_t nlat = pad_layout ? ((lattice_op(A).padded_size() + 63) & ~(int64_t)63) : 0;
  if (pad_layout)
    GFE_TRY(ctx->scratch[SCR_SOLVER2].reserve(sizeof(float) * (size_t)nlat * 5 + 256));
  if (lattice) nblk = std::max<size_t>(nblk, lattice_op(A).blocks(n));
  const size_t npart = nblk * 2 + (size_t)ctx->num_sms * 16 + 64;
  GFE_TRY(ctx->scratch[SCR_REDUCE].reserve(sizeof(SolverState) + sizeof(double) * npart + 256));
  SolverWork w;
  w.S = ctx->scratch[SCR_REDUCE].as<SolverState>();
  w.partials = (double*)((char*)ctx->scratch[SCR_REDUCE].ptr + 256);
  w.hS = (SolverState*)ctx->h_pinned;
  // a grown scratch buffer holds garbage, and a launch cut short by a timed-out wait can
  // leave a ticket part-counted: the reduction tickets must start at zero for every method
  // (the final residual below reduces through them too)
  GFE_CUDA_TRY(cudaMemsetAsync(w.S, 0, sizeof(SolverState), ctx->stream));
  // The precondition switch: Jacobi uses 1/diag, none uses ones (same kernels).
  const bool jac = o->precond == GFE_PC_JACOBI;
  if (!jac && o->precond != GFE_PC_NONE)
    return set_error(GFE_ERR_UNSUPPORTED, "solve: unknown preconditioner %d", o->precond);
  double* v64 = ctx->scratch[SCR_SOLVER].as<double>();
  const double* dinv64 = A->dinv64.as<double>();
  const float* dinv32 = A->dinv32.as<float>();
  DevBuf ones(ctx);
  if (!jac) {
    GFE_TRY(ones.reserve(n8 + sizeof(float) * n + 64));
    std::vector<double> h1(n, 1.0);
    std::vector<float> h1f(n, 1.0f);
    GFE_CUDA_TRY(cudaMemcpyAsync(ones.ptr, h1.data(), n8, cudaMemcpyHostToDevice, ctx->stream));
    GFE_CUDA_TRY(cudaMemcpyAsync((char*)ones.ptr + n8, h1f.data(), sizeof(float) * n,
                                 cudaMemcpyHostToDevice, ctx->stream));
    GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    dinv64 = ones.as<double>();
    dinv32 = (const float*)((char*)ones.ptr + n8);
  }
  rep->iterations = 0;
  rep->refinements = 0;
  rep->converged = 0;
  rep->status = GFE_OK;
  rep->relres = 0.0;

  if (o->method == GFE_SOLVER_CG) {
    double* r = v64;
    double* p = v64 + n;
    double* q = v64 + 2 * n;
    int it = 0, conv = 0;
    GFE_TRY(run_pcg<double>(ctx, A, A->sell_val64.as<double>(), dinv64, d_b, true, 1.0, d_x, r,
                            p, q, o->rtol, maxit, check_every, w, &it, &conv));
    rep->iterations = it;
  } else if (o->method == GFE_SOLVER_MIXED_CG) {
    // FP32 PCG with FP64 reliable updates: whenever the FP32 recursive residual has dropped
    // by delta since the last update (or meets rtol), x64 absorbs the FP32 correction, the
    // true residual b - A x64 is formed in FP64 and replaces the FP32 one, and the search
    // direction is re-orthogonalised against it and continued (no restart).
    double* r64 = v64;
    const LatticeQ1Op lop = lattice ? lattice_op(A) : LatticeQ1Op{};
    const int64_t nv = pad_layout ? nlat : npad;  // FP32 vector stride
    float* f = (float*)ctx->scratch[SCR_SOLVER2].ptr;
    float* x32 = f;
    float* r32 = f + nv;
    float* p32 = f + 2 * nv;
    float* q32 = f + 3 * nv;
    const float* dinv_in = dinv32;  // D^-1 in the layout of the FP32 vectors
    const unsigned gv = (unsigned)(ctx->num_sms * 4);
    const double delta = o->inner_rtol > 0 ? o->inner_rtol : 0.01;
    GFE_CUDA_TRY(cudaMemsetAsync(d_x, 0, n8, ctx->stream));
    GFE_CUDA_TRY(cudaMemsetAsync(w.S, 0, sizeof(SolverState), ctx->stream));
    int maxit_field = maxit;
    GFE_CUDA_TRY(cudaMemcpyAsync(&w.S->maxit, &maxit_field, sizeof(int), cudaMemcpyHostToDevice,
                                 ctx->stream));
    if (pad_layout) {
      // zero halo (x, r, p, q, D^-1), D^-1 scattered to the padded layout
      float* dpad = f + 4 * nv;
      GFE_CUDA_TRY(cudaMemsetAsync(f, 0, sizeof(float) * (size_t)nv * 5, ctx->stream));
      k_to_pad<<<gv, kVecBlock, 0, ctx->stream>>>(lop, n, dinv32, dpad);
      k_cg_init_pad<<<gv, kVecBlock, 0, ctx->stream>>>(lop, n, d_b, r32, p32, dpad, w.partials,
                                                       w.S, o->rtol * o->rtol);
      dinv_in = dpad;
      ctx->launches += 2;
    } else {
      k_cg_init<float, double><<<gv, kVecBlock, 0, ctx->stream>>>(
          n, d_b, 1.0, x32, r32, p32, dinv32, w.partials, w.S, o->rtol * o->rtol);
      ctx->launches++;
    }
    k_set_reliable<<<1, 1, 0, ctx->stream>>>(w.S, delta * delta);
    ctx->launches++;
    w.hS->iter = 0;
    int updates = 0;
    if (!lattice) GFE_TRY(build_dia(ctx, A));
    auto merge = [&]() {
      if (pad_layout)
        k_merge_pad<<<gv, kVecBlock, 0, ctx->stream>>>(lop, n, d_x, x32);
      else
        k_merge<<<gv, kVecBlock, 0, ctx->stream>>>(n, d_x, x32);
      ctx->launches++;
    };
    for (;;) {
      if (pad_layout) {
        GFE_TRY((iterate<float, LatticeQ1Op>(ctx, A, lop, dinv_in, x32, r32, p32, q32,
                                             check_every, w, nv)));
      } else if (A->dia_valid) {
        DiaOp<float> op{A->dia_val32.as<float>(), n, {}};
        for (int d = 0; d < A->dia_ndiag; ++d) op.o.off[d] = A->dia_off[d];
        op.o.nd = A->dia_ndiag;
        GFE_TRY((iterate<float, DiaOp<float>>(ctx, A, op, dinv32, x32, r32, p32, q32,
                                              check_every, w)));
      } else {
        SellOp<float> op{A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(),
                         A->sell_val32.as<float>()};
        GFE_TRY((iterate<float, SellOp<float>>(ctx, A, op, dinv32, x32, r32, p32, q32,
                                               check_every, w)));
      }
      if (w.hS->iter >= maxit || !std::isfinite(w.hS->rr)) {
        if (std::isfinite(w.hS->rr)) merge();  // keep the FP32 correction made so far
        break;
      }
      // reliable update
      merge();
      timer_begin(ctx, GFE_KT_RESIDUAL64);
      k_residual64<<<grid_for(n, kSpmvBlock), kSpmvBlock, 0, ctx->stream>>>(
          n, A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(), A->sell_val64.as<double>(),
          d_x, d_b, r64, w.partials, &w.S->rr64, &w.S->ticket[2]);
      timer_end(ctx);
      if (pad_layout)
        k_restart32_pad<<<gv, kVecBlock, 0, ctx->stream>>>(lop, n, r64, r32, p32, dinv_in,
                                                           w.partials, w.S);
      else
        k_restart32<<<gv, kVecBlock, 0, ctx->stream>>>(n, r64, r32, p32, dinv32, w.partials,
                                                       w.S);
      k_restart_dir<<<gv, kVecBlock, 0, ctx->stream>>>(pad_layout ? nv : n, p32, r32, dinv_in,
                                                       w.S);
      ctx->launches += 3;
      ++updates;
      GFE_CUDA_TRY(cudaGetLastError());
      GFE_TRY(read_state(ctx, w));
      if (w.hS->converged || w.hS->done) break;
      if (updates > 1000) break;
    }
    rep->iterations = w.hS->iter;
    rep->refinements = updates;
    rep->operator_format = lattice ? 2 : A->dia_valid ? 1 : 0;
    rep->ndiag = lattice ? 27 : A->dia_valid ? A->dia_ndiag : 0;
  } else if (o->method == GFE_SOLVER_IR_CG) {
    double* r64 = v64;  // FP64 residual
    float* f = (float*)ctx->scratch[SCR_SOLVER2].ptr;
    float* x32 = f;
    float* r32 = f + npad;
    float* p32 = f + 2 * npad;
    float* q32 = f + 3 * npad;
    const unsigned gv = (unsigned)(ctx->num_sms * 4);
    double* rr_dev = &w.S->rr;
    // x = 0, r = b, ||b||^2
    GFE_CUDA_TRY(cudaMemsetAsync(d_x, 0, n8, ctx->stream));
    GFE_CUDA_TRY(cudaMemcpyAsync(r64, d_b, n8, cudaMemcpyDeviceToDevice, ctx->stream));
    GFE_CUDA_TRY(cudaMemsetAsync(w.S, 0, sizeof(SolverState), ctx->stream));
    k_dot_self<<<gv, kVecBlock, 0, ctx->stream>>>(n, d_b, w.partials, rr_dev, &w.S->ticket[2]);
    ctx->launches++;
    GFE_TRY(read_state(ctx, w));
    const double bb = w.hS->rr;
    const double tol2 = o->rtol * o->rtol * bb;
    double rr = bb;
    const double inner = o->inner_rtol > 0 ? o->inner_rtol : 1e-4;
    int total = 0, outer = 0;
    while (rr > tol2 && total < maxit && bb > 0.0) {
      const double s = 1.0 / std::sqrt(rr);
      int it = 0, conv = 0;
      GFE_TRY(run_pcg<float>(ctx, A, A->sell_val32.as<float>(), dinv32, r64, true, s, x32, r32,
                             p32, q32, inner, maxit - total, check_every, w, &it, &conv));
      total += it;
      ++outer;
      k_refine_update<<<gv, kVecBlock, 0, ctx->stream>>>(n, d_x, x32, 1.0 / s);
      timer_begin(ctx, GFE_KT_RESIDUAL64);
      k_residual64<<<grid_for(n, kSpmvBlock), kSpmvBlock, 0, ctx->stream>>>(
          n, A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(), A->sell_val64.as<double>(),
          d_x, d_b, r64, w.partials, rr_dev, &w.S->ticket[2]);
      timer_end(ctx);
      ctx->launches += 2;
      GFE_CUDA_TRY(cudaGetLastError());
      GFE_TRY(read_state(ctx, w));
      rr = w.hS->rr;
      if (!std::isfinite(rr)) break;
      if (outer > 200) break;
    }
    rep->iterations = total;
    rep->refinements = outer;
  } else if (o->method == GFE_SOLVER_BICGSTAB) {
    int it = 0;
    GFE_TRY(bicgstab(ctx, A, dinv64, d_b, d_x, o->rtol, maxit, &it));
    rep->iterations = it;
  } else {
    return set_error(GFE_ERR_UNSUPPORTED, "solve: unknown method %d", o->method);
  }
  // true FP64 residual of the returned x
  {
    double* r = v64;
    const unsigned gs = grid_for(n, kSpmvBlock);
    k_residual64<<<gs, kSpmvBlock, 0, ctx->stream>>>(
        n, A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(), A->sell_val64.as<double>(), d_x,
        d_b, r, w.partials, &w.S->rr, &w.S->ticket[2]);
    const unsigned gv = (unsigned)(ctx->num_sms * 4);
    k_dot_self<<<gv, kVecBlock, 0, ctx->stream>>>(n, d_b, w.partials, &w.S->bb,
                                                  &w.S->ticket[3]);
    ctx->launches += 2;
    GFE_CUDA_TRY(cudaGetLastError());
    GFE_TRY(read_state(ctx, w));
    const double bb = w.hS->bb;
    rep->relres = rel_residual(w.hS->rr, bb);
    rep->converged = std::isfinite(rep->relres) && rep->relres <= o->rtol * (1.0 + 1e-6);
    if (!std::isfinite(rep->relres)) rep->status = GFE_ERR_NONFINITE;
  }
  return GFE_OK;
}


// The flexible CG's device loop on the lattice multigrid, kept in the context between solves:
// the hierarchy (refreshed from the new kappa by each solve's start) while the fine operator's
// array and dimensions stay the same, and the instantiated loop graph, start included, while
// every buffer it reads and every setting its start takes is the same (the key). Steps that rebuild the same matrix over the same buffers (the
// stream-ordered pool returns them in the same order) skip the graph build.
struct FcgLoopCache {
  LatticeMG* mg = nullptr;
  LatticeQ1Op fine{};
  cudaGraphExec_t exec = nullptr;
  std::vector<uintptr_t> key;
  long long start_launches = 0, body_launches = 0, if_launches = 0;
  ~FcgLoopCache() {
    if (exec) cudaGraphExecDestroy(exec);
    if (mg) mg_destroy(mg);
  }
};

void fcg_cache_release(gfe_ctx* ctx) {
  delete ctx->fcg_cache;
  ctx->fcg_cache = nullptr;
}

static bool same_lattice_op(const LatticeQ1Op& a, const LatticeQ1Op& b) {
  if (a.kap != b.kap || a.n0 != b.n0 || a.n1 != b.n1 || a.n2 != b.n2 || a.s1 != b.s1 ||
      a.s2 != b.s2 || a.c1 != b.c1 || a.c2 != b.c2 || a.p1 != b.p1 || a.p2 != b.p2)
    return false;
  for (int e = 0; e < 64; ++e)
    if (a.K[e] != b.K[e]) return false;
  return true;
}

// Flexible CG with the learned block preconditioner (pc != nullptr) or Jacobi, FP32 vectors
// with FP64 reliable updates. Falls back to Jacobi when the learned preconditioner stagnates
// (the FP32 residual fails to halve over `check_every` iterations twice in a row).
int solve_fcg(gfe_ctx* ctx, gfe_matrix* A, gfe_learned_pc* pc, const gfe_solver_opts* o,
              const double* d_b, double* d_x, gfe_solve_report* rep) {
  if (A->nrows != A->ncols) return set_error(GFE_ERR_INVALID_ARGUMENT, "fcg: not square");
  if (o->initial_guess) return solve_from_guess(ctx, A, pc, true, o, d_b, d_x, rep);
  bool lattice = false;
  GFE_TRY(lattice_ready(ctx, A, &lattice));
  // the multigrid FCG on the lattice operator needs neither the sliced-ELL copy nor its
  // diagonal: its FP64 residuals read the CSR arrays
  const bool csr_residual = lattice && pc == nullptr && o->precond == GFE_PC_MG;
  if (!csr_residual) GFE_TRY(build_solver_plan(ctx, A));
  const int64_t n = A->nrows;
  int check_every = o->check_every > 0 ? o->check_every : 10;
  const int maxit = o->maxiter > 0 ? o->maxiter : 100000;
  const size_t n8 = sizeof(double) * (size_t)(n > 0 ? n : 1);
  const int64_t npad = (n + 63) & ~(int64_t)63;
  GFE_TRY(ctx->scratch[SCR_SOLVER].reserve(n8 * 3 + 64));
  GFE_TRY(ctx->scratch[SCR_SOLVER2].reserve(sizeof(float) * (size_t)(npad > 0 ? npad : 64) * 5 +
                                            256));
  if (!lattice) GFE_TRY(build_dia(ctx, A));
  size_t nblk = grid_for(n, kSpmvBlock);
  if (lattice) nblk = std::max<size_t>(nblk, lattice_op(A).blocks(n));
  const size_t npart = nblk * 2 + (size_t)ctx->num_sms * 16 + 64;
  GFE_TRY(ctx->scratch[SCR_REDUCE].reserve(sizeof(SolverState) + sizeof(double) * npart + 256));
  SolverWork w;
  w.S = ctx->scratch[SCR_REDUCE].as<SolverState>();
  w.partials = (double*)((char*)ctx->scratch[SCR_REDUCE].ptr + 256);
  w.hS = (SolverState*)ctx->h_pinned;
  double* r64 = ctx->scratch[SCR_SOLVER].as<double>();
  float* f = (float*)ctx->scratch[SCR_SOLVER2].ptr;
  float *x32 = f, *r32 = f + npad, *p32 = f + 2 * npad, *q32 = f + 3 * npad,
        *z32 = f + 4 * npad;
  const float* dinv32 = csr_residual ? nullptr : A->dinv32.as<float>();
  const unsigned gv = (unsigned)(ctx->num_sms * 4), gs = grid_for(n, kSpmvBlock);
  // the FP32 vectors sit at multiples of 64 entries from a 256-byte aligned base: the float4
  // kernels apply
  const bool vec4 = (reinterpret_cast<uintptr_t>(f) & 15) == 0;
  // (conds: the device loop's condition handles, when captured into it)
  auto fcg_update = [&](LoopConds conds) {
    if (vec4)
      k_fcg_update4<<<gv, kVecBlock, 0, ctx->stream>>>(n, x32, r32, p32, q32, w.partials, w.S,
                                                       conds);
    else
      k_fcg_update<<<gv, kVecBlock, 0, ctx->stream>>>(n, x32, r32, p32, q32, w.partials, w.S,
                                                      conds);
  };
  // with the multigrid V-cycle on the lattice operator, beta comes from the cycle's last sweep
  // and the direction update runs inside the SpMV (k_lattice_spmv_dir)
  bool fuse_dir = false;
  MgDot mgdot;
  auto fcg_beta_dir = [&]() {
    if (fuse_dir) return;
    if (vec4) {
      k_fcg_beta4<<<gv, kVecBlock, 0, ctx->stream>>>(n, z32, q32, w.partials, w.S);
      k_fcg_dir4<<<gv, kVecBlock, 0, ctx->stream>>>(n, p32, z32, w.S);
    } else {
      k_fcg_beta<<<gv, kVecBlock, 0, ctx->stream>>>(n, z32, q32, w.partials, w.S);
      k_fcg_dir<<<gv, kVecBlock, 0, ctx->stream>>>(n, p32, z32, w.S);
    }
  };
  // r64 = b - A x64 in FP64, r64.r64 into *rr; on the lattice pattern the residual goes
  // straight to r32 for a restart (restart true) and is not stored otherwise
  const size_t lat_smem = sizeof(double) * 32 * 27 * (kSpmvBlock / 32);
  if (A->cart_lattice) {
    GFE_CUDA_TRY(cudaFuncSetAttribute(k_residual64_lattice<true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)lat_smem));
    GFE_CUDA_TRY(cudaFuncSetAttribute(k_residual64_lattice<false>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)lat_smem));
  }
  auto residual64 = [&](double* rr, bool restart) {
    if (A->cart_lattice)
      (A->zf_values ? k_residual64_lattice<true> : k_residual64_lattice<false>)
          <<<(unsigned)(ctx->num_sms * 4), kSpmvBlock, lat_smem, ctx->stream>>>(
              (int)A->cart_n[0] - 1, (int)A->cart_n[1] - 1, (int)A->cart_n[2] - 1,
              A->rowptr.as<int32_t>(), A->val.as<double>(), d_x, d_b, nullptr,
              restart ? r32 : nullptr, w.partials, rr, &w.S->ticket[2]);
    else if (csr_residual)
      k_residual64_csr<4><<<(unsigned)(ctx->num_sms * 8), kSpmvBlock, 0, ctx->stream>>>(
          n, A->rowptr.as<int32_t>(), A->colval.as<int32_t>(), A->val.as<double>(), d_x, d_b,
          r64, w.partials, rr, &w.S->ticket[2]);
    else
      k_residual64<<<gs, kSpmvBlock, 0, ctx->stream>>>(
          n, A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(), A->sell_val64.as<double>(),
          d_x, d_b, r64, w.partials, rr, &w.S->ticket[2]);
  };
  // the restart's source of r32 (none on the lattice pattern: the residual wrote it)
  const double* restart_src = A->cart_lattice ? nullptr : r64;
  // reliable updates: after the FP32 residual has dropped by delta (0.1; 1e-4 with the
  // multigrid preconditioner, which gains about a decade per iteration: two FP64 residuals
  // reach 1e-8 at 128^3, with the same iterations and error as 1e-3's three)
  const double delta = o->inner_rtol > 0 ? o->inner_rtol
                                         : (o->precond == GFE_PC_MG ? 1e-4 : 0.1);
  bool learned = pc != nullptr;
  // the preconditioner in use: the V-cycle (its fine-level smoother learned when pc is
  // given), the learned block preconditioner alone, or Jacobi (also after a fallback)
  bool use_mg = o->precond == GFE_PC_MG;
  DiaOp<float> dop{A->dia_val32.as<float>(), n, {}};
  for (int d = 0; d < A->dia_ndiag; ++d) dop.o.off[d] = A->dia_off[d];
  dop.o.nd = A->dia_ndiag;
  SellOp<float> sop{A->sell_ptr.as<int64_t>(), A->sell_col.as<int32_t>(),
                    A->sell_val32.as<float>()};
  const LatticeQ1Op lop = lattice ? lattice_op(A) : LatticeQ1Op{};
  auto spmv = [&]() {
    timer_begin(ctx, GFE_KT_SPMV32);
    if (lattice && fuse_dir)
      k_lattice_spmv_dir<<<lop.grid(n), kSpmvBlock, 0, ctx->stream>>>(lop, z32, p32, q32, r32,
                                                                      w.partials, w.S);
    else if (lattice)
      k_lattice_spmv<true, false><<<lop.grid(n), kSpmvBlock, 0, ctx->stream>>>(
          lop, p32, q32, r32, w.partials, w.S);
    else if (A->dia_valid)
      k_fcg_spmv<DiaOp<float>><<<gs, kSpmvBlock, 0, ctx->stream>>>(n, dop, p32, q32, r32,
                                                                  w.partials, w.S);
    else
      k_fcg_spmv<SellOp<float>><<<gs, kSpmvBlock, 0, ctx->stream>>>(n, sop, p32, q32, r32,
                                                                   w.partials, w.S);
    timer_end(ctx);
    ctx->launches++;
  };
  // geometric multigrid V-cycle on the lattice operator (GFE_PC_MG without a learned pc)
  LatticeMG* mg = nullptr;
  bool mg_cached = false;  // owned by the context's cache
  struct MgRelease {
    LatticeMG** p;
    const bool* cached;
    ~MgRelease() {
      if (*p && !*cached) mg_destroy(*p);
    }
  } mg_release{&mg, &mg_cached};
  // p-multigrid for Q2 matrices without the Q1 lattice form
  Q2PMG* pmg = nullptr;
  P2PMG* p2mg = nullptr;
  struct PmgRelease {
    Q2PMG** p;
    P2PMG** q;
    ~PmgRelease() {
      if (*p) pmg_destroy(*p);
      if (*q) p2mg_destroy(*q);
    }
  } pmg_release{&pmg, &p2mg};
  // the lattice hierarchy and loop graph may come from (and go to) the context's cache
  const bool cacheable = lattice && use_mg && !learned && !ctx->timer.enabled;
  bool refresh = false;  // the cached hierarchy's coarse kappa and D^-1 are re-formed
  if (use_mg) {
    bool q2 = false;
    if (!lattice) GFE_TRY(pmg_ready(ctx, A, &q2));
    const bool p2 = !lattice && !q2 && A->p2mg_state == 2;
    if (!lattice && !q2 && !p2)
      return set_error(GFE_ERR_UNSUPPORTED,
                       "solve: the multigrid preconditioner needs the lattice operator "
                       "(uniform Cartesian Q1, 3-D, interior-node numbering), a 3-D "
                       "Cartesian Q2 matrix whose vertex dofs are the interior vertices, or "
                       "vector P2 elasticity on a simplexified box");
    if (learned && !lattice)
      return set_error(GFE_ERR_UNSUPPORTED, "solve: the learned smoother is for Q1 lattices");
    if (lattice && cacheable) {
      FcgLoopCache*& C = ctx->fcg_cache;
      if (C && C->mg && same_lattice_op(C->fine, lop)) {
        refresh = true;  // kappa may have new values: with the solve's start
      } else {
        fcg_cache_release(ctx);
        C = new FcgLoopCache();
        GFE_TRY(mg_create(ctx, lop, &C->mg));
        C->fine = lop;
      }
      mg = C->mg;
      mg_cached = true;
    } else if (lattice) {
      GFE_TRY(mg_create(ctx, lop, &mg));
      if (learned) GFE_TRY(mg_set_learned(mg, pc));
    } else if (q2) {
      GFE_TRY(pmg_create(ctx, A, &pmg));
    } else {
      GFE_TRY(p2mg_create(ctx, A, &p2mg));
    }
    // a V-cycle iteration is expensive: look at the state after every one
    if (o->check_every <= 0) check_every = 1;
    if (mg && mg_fuses_dot(mg)) {
      fuse_dir = true;
      mgdot.v = q32;
      mgdot.partials = w.partials;
      mgdot.ticket = &w.S->ticket[3];
      mgdot.den = &w.S->pq;
      mgdot.out = &w.S->beta;
    }
  }
  // launches of fcg_beta_dir
  const int beta_dir_launches = fuse_dir ? 0 : 2;
  // Without kernel timing and without the learned preconditioner's stagnation check, the
  // iterations run as one device-driven loop: a CUDA graph whose WHILE node repeats [update,
  // preconditioner, beta, direction, SpMV] until the state's done flag is set (converged,
  // reliable update due, maxit reached or non-finite), so that the host waits only where the
  // loop stops. The preconditioner's launches are then recorded into that graph, and issued
  // directly outside it, instead of replaying a graph of their own.
  bool device_loop = !ctx->timer.enabled && !learned;
  auto precond = [&]() -> int {
    if (use_mg && pmg) return device_loop ? pmg_record(pmg, r32, z32, &w.S->done)
                                          : pmg_apply(pmg, r32, z32, &w.S->done);
    if (use_mg && p2mg) return device_loop ? p2mg_record(p2mg, r32, z32, &w.S->done)
                                           : p2mg_apply(p2mg, r32, z32, &w.S->done);
    const MgDot* dot = fuse_dir ? &mgdot : nullptr;
    if (use_mg) return device_loop ? mg_record(mg, r32, z32, &w.S->done, dot)
                                   : mg_apply(mg, r32, z32, &w.S->done, dot);
    if (learned) return learned_apply(ctx, pc, r32, z32, &w.S->done);
    k_jacobi_apply<<<gv, kVecBlock, 0, ctx->stream>>>(n, r32, dinv32, z32, w.S);
    ctx->launches++;
    return GFE_OK;
  };
  auto merge = [&]() {
    if (vec4 && (reinterpret_cast<uintptr_t>(d_x) & 15) == 0)
      k_merge4<<<gv, kVecBlock, 0, ctx->stream>>>(n, d_x, x32);
    else
      k_merge<<<gv, kVecBlock, 0, ctx->stream>>>(n, d_x, x32);
  };
  // b and x64 are the caller's buffers: the float4 kernels where they are 16-byte aligned
  const bool vec4_bx = vec4 && ((reinterpret_cast<uintptr_t>(d_b) |
                                 reinterpret_cast<uintptr_t>(d_x)) & 15) == 0;
  // the float4 start forms ||b||^2 in FP64 itself
  const bool bb_from_init = vec4_bx && !dinv32;
  // The start: the hierarchy's refresh, x = 0, r = b, the zeroed state and its settings
  // (defer: the device loop's reliable updates), ||b||^2 in FP64 for the relative residual.
  // z = M r, p = z, q = A p and alpha follow, as the device loop's first iteration or ahead of
  // the host-driven one. *launches: the kernels it launched.
  auto start = [&](bool defer, long long* launches) -> int {
    *launches = 0;
    if (refresh) {
      const long long l0 = ctx->launches;
      GFE_TRY(mg_refresh(mg, lop));
      *launches += ctx->launches - l0;
      ctx->launches = l0;
    }
    GFE_CUDA_TRY(cudaMemsetAsync(d_x, 0, n8, ctx->stream));
    GFE_CUDA_TRY(cudaMemsetAsync(w.S, 0, sizeof(SolverState), ctx->stream));
    if (bb_from_init) {
      k_fcg_init4<<<gv, kVecBlock, 0, ctx->stream>>>(n, d_b, x32, r32, w.partials, w.S,
                                                     o->rtol * o->rtol);
    } else {
      k_cg_init<float, double><<<gv, kVecBlock, 0, ctx->stream>>>(
          n, d_b, 1.0, x32, r32, p32, dinv32, w.partials, w.S, o->rtol * o->rtol);
      k_dot_self<<<gv, kVecBlock, 0, ctx->stream>>>(n, d_b, w.partials, &w.S->bb,
                                                    &w.S->ticket[1]);
      *launches += 1;
    }
    k_fcg_setup<<<1, 1, 0, ctx->stream>>>(w.S, delta * delta, maxit, defer ? 1 : 0);
    *launches += 2;
    // the device loop's first iteration takes beta = 0 (p.q is); the unfused direction update
    // still reads p
    if (defer && !fuse_dir)
      GFE_CUDA_TRY(cudaMemsetAsync(p32, 0, sizeof(float) * n, ctx->stream));
    GFE_CUDA_TRY(cudaGetLastError());
    return GFE_OK;
  };
  struct LoopExec {
    cudaGraphExec_t e = nullptr;
    bool cached = false;  // owned by the context's cache
    ~LoopExec() {
      if (e && !cached) cudaGraphExecDestroy(e);
    }
  } loop;
  long long start_launches = 0, body_launches = 0, if_launches = 0;
  // everything the loop graph reads, by address, and the settings its start takes
  std::vector<uintptr_t> key;
  if (device_loop && mg_cached) {
    const double rtol2 = o->rtol * o->rtol, delta2 = delta * delta;
    uint64_t rb, db;
    std::memcpy(&rb, &rtol2, 8);
    std::memcpy(&db, &delta2, 8);
    key = {(uintptr_t)n, (uintptr_t)d_x, (uintptr_t)d_b, (uintptr_t)A->rowptr.ptr,
           (uintptr_t)A->val.ptr, (uintptr_t)f, (uintptr_t)r64, (uintptr_t)w.S,
           (uintptr_t)w.partials, (uintptr_t)mg,
           (uintptr_t)(vec4 ? 1 : 0) | (vec4_bx ? 2 : 0) | (fuse_dir ? 4 : 0) |
               (refresh ? 8 : 0),
           (uintptr_t)gv, (uintptr_t)lat_smem, (uintptr_t)A->cart_n[0],
           (uintptr_t)A->cart_n[1], (uintptr_t)A->cart_n[2], (uintptr_t)A->cart_lattice,
           (uintptr_t)A->zf_values, (uintptr_t)rb, (uintptr_t)db, (uintptr_t)maxit};
    FcgLoopCache* C = ctx->fcg_cache;
    if (C && C->exec && C->key == key) {
      loop.e = C->exec;
      loop.cached = true;
      start_launches = C->start_launches;
      body_launches = C->body_launches;
      if_launches = C->if_launches;
    }
  }
  if (device_loop && !loop.e) {
    // [start] WHILE (not done) { preconditioner; beta; direction; SpMV; update; IF (reliable
    // update due) { x64 += x32; r64 = b - A x64; r32 = r64 or stop } }: the update and the
    // restart set the two conditions, and the reliable updates run inside the loop too, so
    // that the host waits once per solve. The start is captured into the graph, the WHILE node
    // added after it, and the bodies captured into the nodes' graphs (the IF body on a second
    // stream, its node added at the end of the loop body's capture).
    cudaGraph_t g = nullptr;
    bool ok = cudaGraphCreate(&g, 0) == cudaSuccess;
    cudaGraphConditionalHandle h{}, hif{};
    cudaGraphNodeParams np = {};
    cudaGraphNode_t node;
    ok = ok && cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) ==
                   cudaSuccess;
    // the start, then the WHILE node after it
    if (ok && cudaStreamBeginCaptureToGraph(ctx->stream, g, nullptr, nullptr, 0,
                                            cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const int sst = start(true, &start_launches);
      cudaStreamCaptureStatus cs;
      cudaGraph_t cg = nullptr;
      const cudaGraphNode_t* deps = nullptr;
      const cudaGraphEdgeData* ed = nullptr;
      size_t nd = 0;
      ok = sst == GFE_OK && cudaStreamGetCaptureInfo(ctx->stream, &cs, nullptr, &cg, &deps, &ed,
                                               &nd) == cudaSuccess;
      np.type = cudaGraphNodeTypeConditional;
      np.conditional.handle = h;
      np.conditional.type = cudaGraphCondTypeWhile;
      np.conditional.size = 1;
      ok = ok && cudaGraphAddNode(&node, cg, deps, ed, nd, &np) == cudaSuccess;
      ok = ok && cudaStreamUpdateCaptureDependencies(ctx->stream, &node, nullptr, 1,
                                                     cudaStreamSetCaptureDependencies) ==
                     cudaSuccess;
      cudaGraph_t top = nullptr;
      ok = cudaStreamEndCapture(ctx->stream, &top) == cudaSuccess && ok;
    } else {
      ok = false;
    }
    cudaGraph_t body = ok ? np.conditional.phGraph_out[0] : nullptr;
    ok = ok && cudaGraphConditionalHandleCreate(&hif, body, 0, 0) == cudaSuccess;
    const LoopConds conds{h, hif, 1};
    cudaStream_t s2 = nullptr;
    ok = ok && cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking) == cudaSuccess;
    if (ok && cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0,
                                            cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const long long l0 = ctx->launches;
      const int st = precond();
      fcg_beta_dir();
      spmv();
      fcg_update(conds);
      // precond and SpMV count their launches; + beta and direction (unless fused), update
      body_launches = ctx->launches - l0 + beta_dir_launches + 1;
      ctx->launches = l0;
      // the IF node after the captured work
      cudaStreamCaptureStatus cs;
      cudaGraph_t cg = nullptr;
      const cudaGraphNode_t* deps = nullptr;
      const cudaGraphEdgeData* ed = nullptr;
      size_t nd = 0;
      cudaGraphNodeParams ip = {};
      cudaGraphNode_t ifnode = nullptr;
      bool okif = cudaStreamGetCaptureInfo(ctx->stream, &cs, nullptr, &cg, &deps, &ed, &nd) ==
                  cudaSuccess;
      ip.type = cudaGraphNodeTypeConditional;
      ip.conditional.handle = hif;
      ip.conditional.type = cudaGraphCondTypeIf;
      ip.conditional.size = 1;
      okif = okif && cudaGraphAddNode(&ifnode, cg, deps, ed, nd, &ip) == cudaSuccess;
      if (okif && cudaStreamBeginCaptureToGraph(s2, ip.conditional.phGraph_out[0], nullptr,
                                                nullptr, 0,
                                                cudaStreamCaptureModeThreadLocal) ==
                      cudaSuccess) {
        cudaStream_t main = ctx->stream;
        ctx->stream = s2;  // the reliable update's launches go to the IF body
        merge();
        residual64(&w.S->rr64, true);
        k_fcg_restart<<<gv, kVecBlock, 0, ctx->stream>>>(n, restart_src, r32, w.S, conds);
        if_launches = 3;
        ctx->stream = main;
        cudaGraph_t ifb = nullptr;
        okif = cudaStreamEndCapture(s2, &ifb) == cudaSuccess;
      } else {
        okif = false;
      }
      okif = okif && cudaStreamUpdateCaptureDependencies(ctx->stream, &ifnode, nullptr, 1,
                                                         cudaStreamSetCaptureDependencies) ==
                         cudaSuccess;
      cudaGraph_t bodyg = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &bodyg);
      if (st != GFE_OK) {
        if (g) cudaGraphDestroy(g);
        if (s2) cudaStreamDestroy(s2);
        return st;
      }
      ok = okif && ce == cudaSuccess && cudaGraphInstantiate(&loop.e, g, 0) == cudaSuccess;
    } else {
      ok = false;
    }
    if (s2) cudaStreamDestroy(s2);
    if (g) cudaGraphDestroy(g);
    if (!ok) {
      // conditional graphs unavailable: the host-driven loop below (direct launches)
      (void)cudaGetLastError();
      if (loop.e) cudaGraphExecDestroy(loop.e);
      loop.e = nullptr;
    } else if (mg_cached) {  // hand the graph to the cache
      FcgLoopCache* C = ctx->fcg_cache;
      if (C->exec) cudaGraphExecDestroy(C->exec);
      C->exec = loop.e;
      C->key = key;
      C->start_launches = start_launches;
      C->body_launches = body_launches;
      C->if_launches = if_launches;
      loop.cached = true;
    }
  }
  int updates = 0, slow = 0, fallback = 0;
  bool fresh = false;  // the loop ended on a reliable update: x64 and rr64 are current
  if (loop.e) {
    // the whole solve, reliable updates included, on the device: one wait
    GFE_CUDA_TRY(cudaGraphLaunch(loop.e, ctx->stream));
    GFE_TRY(read_state(ctx, w, true, true));
    updates = w.hS->updates;
    fresh = w.hS->converged != 0;  // only the loop's reliable update declares convergence
    ctx->launches += start_launches + (long long)w.hS->iter * body_launches +
                     (long long)updates * if_launches;
  } else {
    // host-driven loop (kernel timing, the learned preconditioner, no conditional graphs)
    long long sl = 0;
    GFE_TRY(start(false, &sl));
    ctx->launches += sl;
    GFE_TRY(precond());
    // p = z (the fused SpMV forms it: beta is 0 while p.q is)
    if (!fuse_dir)
      GFE_CUDA_TRY(cudaMemcpyAsync(p32, z32, sizeof(float) * n, cudaMemcpyDeviceToDevice,
                                   ctx->stream));
    spmv();
    GFE_TRY(read_state(ctx, w));
  }
  double rr_chunk = w.hS->rr;
  while (!loop.e && !w.hS->done) {
    for (int k = 0; k < check_every; ++k) {
      timer_begin(ctx, GFE_KT_VECTOR);
      fcg_update(LoopConds{});
      timer_end(ctx);
      ctx->launches++;
      GFE_TRY(precond());
      if (!fuse_dir) {
        timer_begin(ctx, GFE_KT_VECTOR);
        fcg_beta_dir();
        timer_end(ctx);
      }
      ctx->launches += beta_dir_launches;
      spmv();
    }
    GFE_CUDA_TRY(cudaGetLastError());
    GFE_TRY(read_state(ctx, w));
    if (w.hS->done && (w.hS->need_update || w.hS->converged)) {
      // reliable update: x64 += x32, r64 = b - A64 x64, r32 = r64 (or stop)
      merge();
      timer_begin(ctx, GFE_KT_RESIDUAL64);
      residual64(&w.S->rr64, true);
      timer_end(ctx);
      k_fcg_restart<<<gv, kVecBlock, 0, ctx->stream>>>(n, restart_src, r32, w.S, LoopConds{});
      ctx->launches += 3;
      ++updates;
      GFE_TRY(read_state(ctx, w));
      if (w.hS->converged || w.hS->done) {
        fresh = true;
        break;
      }
      // z, p restart from the new residual direction (keeps FCG's beta well defined)
      GFE_TRY(precond());
      fcg_beta_dir();
      ctx->launches += beta_dir_launches;
      spmv();
      rr_chunk = w.hS->rr;
      continue;
    }
    if (w.hS->done) break;
    // stagnation check of the learned preconditioner (alone, or as the V-cycle's smoother)
    if (learned) {
      // less than a 4x residual drop per 10 iterations, scaled to the chunk's length
      slow = (w.hS->rr > std::pow(0.25, check_every / 10.0) * rr_chunk) ? slow + 1 : 0;
      if (slow >= 2) {
        learned = false;  // Jacobi from here on
        use_mg = false;
        fallback = 1;
      }
    }
    rr_chunk = w.hS->rr;
  }
  // any FP32 correction not yet absorbed (none when the loop ended on a reliable update)
  if (!fresh) {
    merge();
    ctx->launches++;
  }
  rep->iterations = w.hS->iter;
  rep->refinements = updates;
  rep->operator_format = A->dia_valid ? 1 : 0;
  rep->ndiag = A->dia_valid ? A->dia_ndiag : 0;
  rep->fallback = fallback;
  // true FP64 residual (the reliable update's when it ended the loop: x has not moved since)
  if (!fresh) {
    residual64(&w.S->rr, false);
    ctx->launches++;
  }
  GFE_CUDA_TRY(cudaGetLastError());
  if (!(loop.e && fresh)) GFE_TRY(read_state(ctx, w, true, true));
  const double bb = w.hS->bb;
  const double rr = fresh ? w.hS->rr64 : w.hS->rr;
  rep->relres = rel_residual(rr, bb);
  rep->converged = std::isfinite(rep->relres) && rep->relres <= o->rtol * (1.0 + 1e-6);
  rep->status = std::isfinite(rep->relres) ? GFE_OK : GFE_ERR_NONFINITE;
  return GFE_OK;
}

}  // namespace gfe
