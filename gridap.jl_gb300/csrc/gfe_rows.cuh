// gfe_rows.cuh -- the row-gather assembly kernel shared by the element families.
//
// Every matrix row is owned by one thread, which walks the row's cell references (sorted by
// cell) and accumulates each contribution at its precomputed position in the row, so each
// stored value receives Gridap's additions in Gridap's order (ascending cells), with no
// atomics and no colouring. A block of R rows then writes its contiguous CSR slice with
// coalesced stores. Cell values come from a source functor with
//   load_tables(smem), m(tables, cell, li, lj, nd), v(tables, cell, li)  and  ntab.
#pragma once
#include <type_traits>

#include "gfe_internal.h"

namespace gfe {
namespace {
__device__ __forceinline__ void raise_err(DevError* err, int code, long long index) {
  if (atomicCAS(&err->code, 0, code) == 0) err->index = index;
}

struct RowArgs {
  int64_t nrows;
  int nd;       // local rows per cell (leading dimension of the column-major cell matrices)
  int ndc = 0;  // local columns per cell; 0 means nd
  __host__ __device__ int cols() const { return ndc > 0 ? ndc : nd; }
  const int32_t* rowptr;
  const int32_t* colval;
  const int64_t* ref_ptr;
  const int32_t* refs;
  const int32_t* cell_cols;  // column ids per cell (Gridap convention)
  const void* refpos;        // per (reference, local column) position in the row
  double* val;               // may be null (vector only)
  double* b;                 // may be null (matrix only)
  DevError* err;
  const double* uD = nullptr;  // Dirichlet values for the lift (null: u_D = 0)
  int64_t ndiri = 0;
};

// ---- cell value sources -------------------------------------------------------------------
// FP32 stored cell arrays (the tensor-core element kernels' output), accumulated in FP64.
struct StoredCellsF32 {
  const float* mat;
  const float* vec;
  int64_t cs, es, vcs, ves;
  int ntab;
  __device__ void load_tables(double*) const {}
  __device__ __forceinline__ int64_t cell(int64_t c) const { return c; }
  __device__ __forceinline__ double m(const double*, int64_t cell, int li, int lj, int nd) const {
    return (double)__ldg(mat + cell * cs + (int64_t)(li + lj * nd) * es);
  }
  __device__ __forceinline__ double v(const double*, int64_t cell, int li) const {
    return (double)__ldg(vec + cell * vcs + (int64_t)li * ves);
  }
};

// FP32 cell matrices in 16-cell tiles (the tensor-core P2 kernels' layout): entry e = li +
// lj*nd of cell c at mat[((c / 16) * nd*nd + e) * 16 + c % 16], so the 16 cells of a tile are
// contiguous per entry. No cell vectors.
struct TiledCellsF32 {
  const float* mat;
  int ntab;
  __device__ void load_tables(double*) const {}
  __device__ __forceinline__ int64_t cell(int64_t c) const { return c; }
  __device__ __forceinline__ double m(const double*, int64_t cell, int li, int lj, int nd) const {
    return (double)__ldg(mat + (((cell >> 4) * nd * nd + li + lj * nd) << 4) + (cell & 15));
  }
  __device__ __forceinline__ double v(const double*, int64_t, int) const { return 0.0; }
};

// Stored cell arrays. Entry (cell, li, lj) at mat[cell*cs + (li + lj*nd)*es].
struct StoredCells {
  const double* mat;
  const double* vec;
  int64_t cs, es;    // cell stride, entry stride of mat
  int64_t vcs, ves;  // same for vec
  int ntab;          // no tables
  __device__ void load_tables(double*) const {}
  __device__ __forceinline__ int64_t cell(int64_t c) const { return c; }
  __device__ __forceinline__ double m(const double*, int64_t cell, int li, int lj, int nd) const {
    return __ldg(mat + cell * cs + (int64_t)(li + lj * nd) * es);
  }
  __device__ __forceinline__ double v(const double*, int64_t cell, int li) const {
    return __ldg(vec + cell * vcs + (int64_t)li * ves);
  }
};


// acc + m(...): a source may provide madd(tables, cell data, li, lj, nd, acc) that forms the
// sum with one fused multiply-add (FP64 issue bounds the fused-integral gathers)
template <class S, class = void>
struct has_madd : std::false_type {};
template <class S>
struct has_madd<S, std::void_t<decltype(&S::madd)>> : std::true_type {};

template <class Src, class CC>
__device__ __forceinline__ double src_madd(const Src& src, const double* tab, const CC& cc,
                                           int li, int lj, int nd, double acc) {
  if constexpr (has_madd<Src>::value)
    return src.madd(tab, cc, li, lj, nd, acc);
  else
    return acc + src.m(tab, cc, li, lj, nd);
}

// ---- the row-gather kernel ----------------------------------------------------------------
template <int MAXW, int R, class Src, typename PosT>
__global__ void __launch_bounds__(R) k_assemble_rows(RowArgs a, Src src) {
  extern __shared__ double smem[];
  double* acc = smem;                 // acc[k*R + t]
  double* tab = smem + MAXW * R;      // source tables
  __shared__ int32_t lrp[R + 1];      // block-relative row starts
  const int t = threadIdx.x;
  const int64_t r0 = (int64_t)blockIdx.x * R;
  const int64_t r = r0 + t;
  src.load_tables(tab);

  int32_t start = 0, n = 0;
  if (r < a.nrows) {
    start = a.rowptr[r];
    n = a.rowptr[r + 1] - start;
  }
  const int64_t rend = (r0 + R < a.nrows) ? r0 + R : a.nrows;
  const int32_t bstart = a.rowptr[r0 < a.nrows ? r0 : a.nrows];
  lrp[t] = (r < a.nrows ? start : a.rowptr[rend]) - bstart;
  if (t == 0) lrp[R] = a.rowptr[rend] - bstart;
  if (a.val)
    for (int k = 0; k < n; ++k) acc[k * R + t] = 0.0;
  __syncthreads();

  double bacc = 0.0;
  if (r < a.nrows) {
    const PosT* refpos = static_cast<const PosT*>(a.refpos);
    for (int64_t q = a.ref_ptr[r]; q < a.ref_ptr[r + 1]; ++q) {
      const int32_t e = a.refs[q];
      const int64_t cell = e / a.nd;
      const int li = e - (int)(cell * a.nd);
      if (a.val) {
        const int ndc = a.cols();
        const auto cc = src.cell(cell);  // per-cell data (coefficients) loaded once per ref
        const PosT* pp = refpos + q * ndc;
        auto add = [&](int lj, PosT p) {
          if (p == (PosT)~(PosT)0) return;  // Dirichlet column
          if (p >= n) {
            raise_err(a.err, GFE_ERR_INVALID_ARGUMENT, r);
            return;
          }
          acc[p * R + t] = src_madd(src, tab, cc, li, lj, a.nd, acc[p * R + t]);
        };
        if (sizeof(PosT) == 1 && (ndc & 3) == 0) {
          // byte positions four at a time (the reference's row of the table is 4-aligned)
          const uint32_t* pw = reinterpret_cast<const uint32_t*>(pp);
          for (int w4 = 0; w4 < (ndc >> 2); ++w4) {
            const uint32_t word = __ldg(pw + w4);
#pragma unroll
            for (int bb = 0; bb < 4; ++bb) add(4 * w4 + bb, (PosT)((word >> (8 * bb)) & 0xffu));
          }
        } else {
          for (int lj = 0; lj < ndc; ++lj) add(lj, __ldg(pp + lj));
        }
      }
      if (a.b) bacc += src.v(tab, cell, li);
    }
    if (a.b) a.b[r] = bacc;
  }
  if (!a.val) return;
  __syncthreads();
  // coalesced write-out of the block's CSR slice
  const int32_t total = lrp[R];
  double* out = a.val + bstart;
  for (int32_t l = t; l < total; l += R) {
    int lo = 0, hi = R;  // largest row t' with lrp[t'] <= l
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (lrp[mid] <= l) lo = mid; else hi = mid;
    }
    out[l] = acc[(l - lrp[lo]) * R + lo];
  }
}

template <int MAXW, int R, class Src>
static int launch_rows(gfe_ctx* ctx, const RowArgs& a, const Src& src, int pos_bytes) {
  const size_t smem = sizeof(double) * ((size_t)MAXW * R + (size_t)src.ntab);
  auto kern = pos_bytes == 1 ? k_assemble_rows<MAXW, R, Src, uint8_t>
                             : k_assemble_rows<MAXW, R, Src, uint16_t>;
  if (smem > 48 * 1024)
    GFE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  timer_begin(ctx, GFE_KT_ASSEMBLE);
  kern<<<grid_for(a.nrows, R), R, smem, ctx->stream>>>(a, src);
  timer_end(ctx);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

// Maximum row width of a matrix (device reduction over rowptr differences).
__global__ void k_max_width(const int32_t* __restrict__ rowptr, int64_t n, int32_t* out) {
  int32_t m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t w = rowptr[i + 1] - rowptr[i];
    m = w > m ? w : m;
  }
  for (int off = 16; off > 0; off >>= 1) {
    const int32_t o = __shfl_down_sync(0xffffffffu, m, off);
    m = o > m ? o : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

static int max_row_width(gfe_ctx* ctx, gfe_matrix* A, int* out) {
  GFE_TRY(ctx->scratch[SCR_REDUCE].reserve(256));
  int32_t* d = ctx->scratch[SCR_REDUCE].as<int32_t>();
  GFE_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(int32_t), ctx->stream));
  k_max_width<<<grid_for(A->nrows, 256, (int64_t)ctx->num_sms * 8), 256, 0, ctx->stream>>>(
      A->rowptr.as<int32_t>(), A->nrows, d);
  ctx->launches++;
  int32_t h = 0;
  GFE_TRY(copy_out(ctx, &h, d, sizeof(int32_t)));
  *out = h;
  return GFE_OK;
}

// Warp-per-row variant for elements with many dofs per cell (nd >= 16: Q2, P2, vector
// spaces). A warp owns one row; its lanes take the local columns of one reference at a time
// (lane lj, then lj + 32, ...), so the references -- and hence the additions into every
// stored value -- are still processed in ascending cell order, exactly as in the
// thread-per-row kernel. Distinct local columns of one cell land on distinct positions, so
// the lanes of a step never collide. Each warp keeps its row in MAXW doubles of shared
// memory; 8 warps per block.
constexpr int kRowWarps = 8;

template <int MAXW, class Src, typename PosT>
__global__ void __launch_bounds__(32 * kRowWarps)
    k_assemble_rows_warp(RowArgs a, Src src) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double* acc = smem + wib * MAXW;
  double* tab = smem + kRowWarps * MAXW;
  src.load_tables(tab);
  __syncthreads();
  const int64_t r = (int64_t)blockIdx.x * kRowWarps + wib;
  if (r >= a.nrows) return;
  int32_t start = 0, n = 0;
  if (a.val) {
    start = a.rowptr[r];
    n = a.rowptr[r + 1] - start;
    for (int k = lane; k < n; k += 32) acc[k] = 0.0;
    __syncwarp();
  }
  const PosT* refpos = static_cast<const PosT*>(a.refpos);
  double bacc = 0.0;
  for (int64_t q = a.ref_ptr[r]; q < a.ref_ptr[r + 1]; ++q) {
    const int32_t e = a.refs[q];
    const int64_t cell = e / a.nd;
    const int li = e - (int)(cell * a.nd);
    if (a.val) {
      const auto cc = src.cell(cell);
      const int ndc = a.cols();
      for (int lj = lane; lj < ndc; lj += 32) {
        const PosT pp = __ldg(refpos + q * ndc + lj);
        if (pp == (PosT)~(PosT)0) continue;  // Dirichlet column
        if (pp >= n) {
          raise_err(a.err, GFE_ERR_INVALID_ARGUMENT, r);
          continue;
        }
        acc[pp] = src_madd(src, tab, cc, li, lj, a.nd, acc[pp]);
      }
      __syncwarp();
    }
    if (a.b && lane == 0) bacc += src.v(tab, cell, li);
  }
  if (a.b && lane == 0) a.b[r] = bacc;
  if (!a.val) return;
  double* out = a.val + start;
  for (int k = lane; k < n; k += 32) out[k] = acc[k];
}

template <int MAXW, class Src>
static int launch_rows_warp(gfe_ctx* ctx, const RowArgs& a, const Src& src, int pos_bytes) {
  const size_t smem = sizeof(double) * ((size_t)MAXW * kRowWarps + (size_t)src.ntab);
  auto kern = pos_bytes == 1 ? k_assemble_rows_warp<MAXW, Src, uint8_t>
                             : k_assemble_rows_warp<MAXW, Src, uint16_t>;
  if (smem > 48 * 1024)
    GFE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  timer_begin(ctx, GFE_KT_ASSEMBLE);
  kern<<<grid_for(a.nrows, kRowWarps), 32 * kRowWarps, smem, ctx->stream>>>(a, src);
  timer_end(ctx);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

// Dirichlet lift (AttachDirichletMap, CellData/AttachDirichlet.jl:59-110): every cell's
// vector entry li receives -sum_j K_cell[li][j] u_D[j] over the cell's Dirichlet columns j;
// b[r] += those contributions of the row's references, in cell order.
template <class Src>
__global__ void k_dirichlet_lift(RowArgs a, Src src) {
  extern __shared__ double tab[];
  src.load_tables(tab);
  __syncthreads();
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.nrows) return;
  double acc = 0.0;
  bool any = false;
  for (int64_t q = a.ref_ptr[r]; q < a.ref_ptr[r + 1]; ++q) {
    const int32_t e = a.refs[q];
    const int64_t cell = e / a.nd;
    const int li = e - (int)(cell * a.nd);
    const int ndc = a.cols();
    const int32_t* ids = a.cell_cols + cell * ndc;
    double l = 0.0;
    bool has = false;
    const auto cc = src.cell(cell);
    for (int lj = 0; lj < ndc; ++lj) {
      const int32_t col = __ldg(ids + lj);
      if (col >= 0) continue;
      const int64_t k = -(int64_t)col - 1;
      if (k >= a.ndiri) {
        raise_err(a.err, GFE_ERR_INVALID_ARGUMENT, r);
        continue;
      }
      has = true;
      l -= src.m(tab, cc, li, lj, a.nd) * __ldg(a.uD + k);
    }
    if (has) {
      acc += l;
      any = true;
    }
  }
  if (any) a.b[r] += acc;
}

template <class Src>
static int dirichlet_lift(gfe_ctx* ctx, const RowArgs& a, const Src& src) {
  k_dirichlet_lift<Src><<<grid_for(a.nrows, 128), 128, sizeof(double) * src.ntab,
                          ctx->stream>>>(a, src);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

template <class Src>
static int run_rows_main(gfe_ctx* ctx, const RowArgs& a, const Src& src, int maxw, int pb);

// The row gather, followed by the Dirichlet lift when the call carries Dirichlet values.
template <class Src>
static int run_rows(gfe_ctx* ctx, const RowArgs& a, const Src& src, int maxw, int pb) {
  GFE_TRY(run_rows_main(ctx, a, src, maxw, pb));
  if (a.uD && a.b && a.val && a.cell_cols) GFE_TRY(dirichlet_lift(ctx, a, src));
  return GFE_OK;
}

template <class Src>
static int run_rows_main(gfe_ctx* ctx, const RowArgs& a, const Src& src, int maxw, int pb) {
  if (a.cols() >= 16 && a.val) {
    if (maxw <= 128) return launch_rows_warp<128>(ctx, a, src, pb);
    if (maxw <= 256) return launch_rows_warp<256>(ctx, a, src, pb);
    if (maxw <= 512) return launch_rows_warp<512>(ctx, a, src, pb);
    if (maxw <= 1024) return launch_rows_warp<1024>(ctx, a, src, pb);
    return set_error(GFE_ERR_ROW_TOO_WIDE, "assembly: row width %d exceeds 1024", maxw);
  }
  if (maxw <= 16) return launch_rows<16, 128>(ctx, a, src, pb);
  if (maxw <= 32) return launch_rows<32, 128>(ctx, a, src, pb);
  if (maxw <= 64) return launch_rows<64, 128>(ctx, a, src, pb);
  if (maxw <= 128) return launch_rows<128, 64>(ctx, a, src, pb);
  if (maxw <= 256) return launch_rows<256, 32>(ctx, a, src, pb);
  if (maxw <= 512) return launch_rows<512, 16>(ctx, a, src, pb);
  return set_error(GFE_ERR_ROW_TOO_WIDE, "assembly: row width %d exceeds 512", maxw);
}

static RowArgs row_args(gfe_ctx* ctx, gfe_matrix* A, double* b, bool with_matrix) {
  RowArgs a;
  a.nrows = A->nrows;
  a.nd = A->nd;
  a.ndc = A->cols_per_cell();
  a.rowptr = A->rowptr.as<int32_t>();
  a.colval = A->colval.as<int32_t>();
  a.ref_ptr = A->ref_ptr.as<int64_t>();
  a.refs = A->refs.as<int32_t>();
  a.cell_cols = A->col_ids();
  a.refpos = A->refpos.ptr;
  a.val = with_matrix ? A->val.as<double>() : nullptr;
  a.b = b;
  a.err = ctx->d_err;
  a.uD = ctx->lift_uD;
  a.ndiri = ctx->lift_ndiri;
  return a;
}

// Vector-only gather: b[r] (+)= the row's cell contributions in cell order.
template <class Src, bool ADD>
__global__ void k_vector_rows(RowArgs a, Src src) {
  extern __shared__ double tab[];
  src.load_tables(tab);
  __syncthreads();
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.nrows) return;
  double acc = 0.0;
  for (int64_t q = a.ref_ptr[r]; q < a.ref_ptr[r + 1]; ++q) {
    const int32_t e = a.refs[q];
    const int64_t cell = e / a.nd;
    acc += src.v(tab, cell, e - (int)(cell * a.nd));
  }
  if (ADD) a.b[r] += acc; else a.b[r] = acc;
}

template <class Src, bool ADD = false>
static int vector_only_rows(gfe_ctx* ctx, const RowArgs& a, const Src& src) {
  k_vector_rows<Src, ADD><<<grid_for(a.nrows, 256), 256, sizeof(double) * src.ntab,
                            ctx->stream>>>(a, src);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

}  // namespace
}  // namespace gfe
