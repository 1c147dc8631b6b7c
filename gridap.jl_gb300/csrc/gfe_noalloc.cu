// gfe_noalloc.cu -- an FP64 Jacobi-PCG solve that allocates no device memory.
//
// Some callers cannot call cudaMalloc: applications that hand all device memory to their
// own pool or arena at start-up (a Julia CUDA.jl memory pool, a simulation code with a fixed
// memory budget) and must not have a library allocate behind their back while they run.
// gfe_cg_solve_noalloc serves them: the caller passes the matrix (CSR) and the vectors in
// device memory, and the solver's work vectors and reduction words live in one file-scope
// static __device__ array of fixed size, which every GPU that loads the library holds until
// the process exits.
//
// Limits and rules:
//   - at most kMaxRows rows (2^19 = 524,288): 4 FP64 vectors + reduction words, ~16 MB;
//   - every call shares the array; the state words that must start at zero are cleared at
//     the start of each call, and calls that overlap on the GPU (different streams, threads
//     or processes sharing a context) race on it;
//   - the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current); make that first call
//     before any stream capture.
#include <mutex>

#include "gfe_internal.h"

namespace gfe {
namespace noalloc {

constexpr int64_t kMaxRows = int64_t(1) << 19;
constexpr int kBlock = 256;
constexpr int kVecBlocks = 1024;  // fixed grid of the vector kernels
constexpr int64_t kMaxSpmvBlocks = (kMaxRows + kBlock - 1) / kBlock;
constexpr int64_t kPartials = 2 * (kMaxSpmvBlocks > kVecBlocks ? kMaxSpmvBlocks : kVecBlocks);

struct State {
  double bb, tol2, rz, rr, alpha, beta;
  int iter, done, converged, maxit;
  unsigned ticket[4];
  int bad_index;  // set when rowptr/colval fail validation
  int nonfinite;  // a reduction (r.z, r.r, p.q) came out NaN or Inf
};

// layout of the scratch array, in doubles: r | p | q | dinv | partials | state
constexpr int64_t kStateDoubles = (sizeof(State) + sizeof(double) - 1) / sizeof(double);
constexpr int64_t kScratchDoubles = 4 * kMaxRows + kPartials + kStateDoubles;

static __device__ __align__(256) double g_scratch[kScratchDoubles];

struct Views {
  double* r;
  double* p;
  double* q;
  double* dinv;
  double* partials;
  State* S;
};

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kBlock / 32; ++i) s += sh[i];
  __syncthreads();
  return s;
}

// every block writes its partial(s); the last block to arrive reduces them in block order
template <int NV>
__device__ bool last_block(unsigned* ticket, const double* partials, double* out, double* sh) {
  __shared__ bool last;
  __threadfence();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  for (int v = 0; v < NV; ++v) {
    double s = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += kBlock)
      s += __ldcg(partials + (int64_t)i * NV + v);
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[v] = s;
  }
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}

// rowptr was validated (monotone, within nnz) before any kernel reads through it; column
// ids outside [0, n) are skipped (the validation kernel reports them).
__device__ __forceinline__ double csr_row(int64_t r, int64_t n,
                                          const int32_t* __restrict__ rowptr,
                                          const int32_t* __restrict__ col,
                                          const double* __restrict__ val,
                                          const double* __restrict__ x) {
  double acc = 0.0;
  for (int32_t k = __ldg(rowptr + r); k < __ldg(rowptr + r + 1); ++k) {
    const int32_t c = __ldg(col + k);
    if ((uint32_t)c < (uint64_t)n) acc = fma(__ldg(val + k), __ldg(x + c), acc);
  }
  return acc;
}

// rowptr[0] == 0, rowptr non-decreasing, rowptr[n] <= nnz, column ids in [0, n)
__global__ void k_validate(int64_t n, int64_t nnz, const int32_t* __restrict__ rowptr,
                           const int32_t* __restrict__ col, State* S) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = rowptr[i], b = rowptr[i + 1];
    if ((i == 0 && a != 0) || b < a || (int64_t)b > nnz || a < 0) {
      atomicExch(&S->bad_index, 1);
      continue;
    }
  }
}

__global__ void k_validate_cols(int64_t n, const int32_t* __restrict__ rowptr,
                                const int32_t* __restrict__ col, State* S) {
  if (S->bad_index) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if ((uint32_t)col[k] >= (uint64_t)n) atomicExch(&S->bad_index, 1);
}

__global__ void k_init(int64_t n, const int32_t* __restrict__ rowptr,
                       const int32_t* __restrict__ col, const double* __restrict__ val,
                       const double* __restrict__ b, double* __restrict__ x, Views v,
                       double rtol2, int maxit) {
  __shared__ double sh[kBlock / 32];
  double rz = 0.0, bb = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double d = 1.0;
    for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (col[k] == i && val[k] != 0.0 && isfinite(val[k])) d = 1.0 / val[k];
    v.dinv[i] = d;
    const double bi = b[i];
    x[i] = 0.0;
    v.r[i] = bi;
    v.p[i] = d * bi;
    rz += bi * (d * bi);
    bb += bi * bi;
  }
  rz = block_sum(rz, sh);
  bb = block_sum(bb, sh);
  if (threadIdx.x == 0) {
    v.partials[2 * blockIdx.x] = rz;
    v.partials[2 * blockIdx.x + 1] = bb;
  }
  double tot[2];
  if (last_block<2>(&v.S->ticket[1], v.partials, tot, sh) && threadIdx.x == 0) {
    v.S->rz = tot[0];
    v.S->bb = tot[1];
    v.S->rr = tot[1];
    v.S->tol2 = rtol2 * tot[1];
    v.S->iter = 0;
    v.S->maxit = maxit;
    v.S->converged = tot[1] == 0.0;
    v.S->done = tot[1] == 0.0;
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      v.S->nonfinite = 1;
      v.S->done = 1;
    }
  }
}

// Restart from the current x once the recursively updated residual met the tolerance but the
// true one did not: r = b - A x, p = D^-1 r, r.z, with the iteration count kept.
__global__ void k_restart(int64_t n, const int32_t* __restrict__ rowptr,
                          const int32_t* __restrict__ col, const double* __restrict__ val,
                          const double* __restrict__ b, const double* __restrict__ x, Views v) {
  __shared__ double sh[kBlock / 32];
  double rz = 0.0, rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double ri = b[i] - csr_row(i, n, rowptr, col, val, x);
    v.r[i] = ri;
    v.p[i] = v.dinv[i] * ri;
    rz += ri * (v.dinv[i] * ri);
    rr += ri * ri;
  }
  rz = block_sum(rz, sh);
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    v.partials[2 * blockIdx.x] = rz;
    v.partials[2 * blockIdx.x + 1] = rr;
  }
  double tot[2];
  if (last_block<2>(&v.S->ticket[1], v.partials, tot, sh) && threadIdx.x == 0) {
    v.S->rz = tot[0];
    v.S->rr = tot[1];
    v.S->converged = 0;
    v.S->done = 0;
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      v.S->nonfinite = 1;
      v.S->done = 1;
    }
  }
}

__global__ void k_spmv_dot(int64_t n, const int32_t* __restrict__ rowptr,
                           const int32_t* __restrict__ col, const double* __restrict__ val,
                           Views v) {
  __shared__ double sh[kBlock / 32];
  if (v.S->done) return;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double d = 0.0;
  if (r < n) {
    const double y = csr_row(r, n, rowptr, col, val, v.p);
    v.q[r] = y;
    d = v.p[r] * y;
  }
  d = block_sum(d, sh);
  if (threadIdx.x == 0) v.partials[blockIdx.x] = d;
  double tot[1];
  if (last_block<1>(&v.S->ticket[0], v.partials, tot, sh) && threadIdx.x == 0) {
    if (!isfinite(tot[0])) {
      v.S->nonfinite = 1;
      v.S->done = 1;
      v.S->alpha = 0.0;
    } else {
      v.S->alpha = tot[0] != 0.0 ? v.S->rz / tot[0] : 0.0;
    }
  }
}

__global__ void k_update(int64_t n, double* __restrict__ x, Views v) {
  __shared__ double sh[kBlock / 32];
  if (v.S->done) return;
  const double alpha = v.S->alpha;
  double rz = 0.0, rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = fma(alpha, v.p[i], x[i]);
    const double ri = fma(-alpha, v.q[i], v.r[i]);
    v.r[i] = ri;
    rz += ri * (v.dinv[i] * ri);
    rr += ri * ri;
  }
  rz = block_sum(rz, sh);
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    v.partials[2 * blockIdx.x] = rz;
    v.partials[2 * blockIdx.x + 1] = rr;
  }
  double tot[2];
  if (last_block<2>(&v.S->ticket[1], v.partials, tot, sh) && threadIdx.x == 0) {
    State* S = v.S;
    S->iter += 1;
    S->rr = tot[1];
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      S->done = 1;
      S->nonfinite = 1;
    } else if (tot[1] <= S->tol2) {
      S->done = 1;
      S->converged = 1;
    } else if (S->iter >= S->maxit) {
      S->done = 1;
    }
    S->beta = S->rz != 0.0 ? tot[0] / S->rz : 0.0;
    S->rz = tot[0];
  }
}

__global__ void k_direction(int64_t n, Views v) {
  if (v.S->done) return;
  const double beta = v.S->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v.p[i] = fma(beta, v.p[i], v.dinv[i] * v.r[i]);
}

// true residual ||b - A x||^2 into S->rr
__global__ void k_residual(int64_t n, const int32_t* __restrict__ rowptr,
                           const int32_t* __restrict__ col, const double* __restrict__ val,
                           const double* __restrict__ b, const double* __restrict__ x, Views v) {
  __shared__ double sh[kBlock / 32];
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double d = 0.0;
  if (r < n) {
    const double ri = b[r] - csr_row(r, n, rowptr, col, val, x);
    d = ri * ri;
  }
  d = block_sum(d, sh);
  if (threadIdx.x == 0) v.partials[blockIdx.x] = d;
  double tot[1];
  if (last_block<1>(&v.S->ticket[2], v.partials, tot, sh) && threadIdx.x == 0)
    v.S->rr = tot[0];
}

// Device address of g_scratch, looked up once per device with that device current.
static std::mutex g_mutex;
static double* g_addr[128] = {nullptr};

static int scratch_address(int device, double** out) {
  if (device < 0 || device >= 128)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_cg_solve_noalloc: device id %d", device);
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p)
      return set_error(GFE_ERR_CUDA, "gfe_cg_solve_noalloc: cudaGetSymbolAddress failed: %s",
                       cudaGetErrorString(e));
    g_addr[device] = static_cast<double*>(p);
  }
  *out = g_addr[device];
  return GFE_OK;
}

// Device memory of the current GPU (a pointer into another GPU's memory would be read
// without peer access), or managed memory.
static bool on_device(const void* p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace noalloc
}  // namespace gfe

using namespace gfe;
using namespace gfe::noalloc;

extern "C" int gfe_cg_solve_noalloc(const int32_t* rowptr, const int32_t* colval,
                                    const double* val, int64_t n, int64_t nnz,
                                    const double* b, double* x,
                                    double rtol, int32_t maxiter, void* stream,
                                    int32_t* iterations, double* relres) {
  clear_error();
  if (n < 0 || nnz < 0 || nnz > INT32_MAX || !(rtol > 0.0) || maxiter < 1)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_cg_solve_noalloc: bad n, rtol or maxiter");
  if (n > kMaxRows)
    return set_error(GFE_ERR_INVALID_ARGUMENT,
                     "gfe_cg_solve_noalloc: %lld rows exceed the fixed scratch limit of %lld",
                     (long long)n, (long long)kMaxRows);
  if (n == 0) {
    if (iterations) *iterations = 0;
    if (relres) *relres = 0.0;
    return GFE_OK;
  }
  int dev = 0;
  GFE_CUDA_TRY(cudaGetDevice(&dev));
  if (!rowptr || !colval || !val || !b || !x || !on_device(rowptr, dev) ||
      !on_device(colval, dev) || !on_device(val, dev) || !on_device(b, dev) ||
      !on_device(x, dev))
    return set_error(GFE_ERR_INVALID_ARGUMENT,
                     "gfe_cg_solve_noalloc: rowptr, colval, val, b and x must be device memory "
                     "of the current GPU");
  double* base = nullptr;
  GFE_TRY(scratch_address(dev, &base));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  Views v;
  v.r = base;
  v.p = base + kMaxRows;
  v.q = base + 2 * kMaxRows;
  v.dinv = base + 3 * kMaxRows;
  v.partials = base + 4 * kMaxRows;
  v.S = reinterpret_cast<State*>(base + 4 * kMaxRows + kPartials);
  // state words start at zero on every call (tickets, counters, flags)
  GFE_CUDA_TRY(cudaMemsetAsync(v.S, 0, sizeof(State), st));
  const unsigned gs = (unsigned)((n + kBlock - 1) / kBlock);
  State h;
  k_validate<<<kVecBlocks, kBlock, 0, st>>>(n, nnz, rowptr, colval, v.S);
  k_validate_cols<<<kVecBlocks, kBlock, 0, st>>>(n, rowptr, colval, v.S);
  GFE_CUDA_TRY(cudaGetLastError());
  GFE_CUDA_TRY(cudaMemcpyAsync(&h, v.S, sizeof(State), cudaMemcpyDeviceToHost, st));
  GFE_CUDA_TRY(cudaStreamSynchronize(st));
  if (h.bad_index)
    return set_error(GFE_ERR_INVALID_ARGUMENT,
                     "gfe_cg_solve_noalloc: malformed CSR (rowptr or column ids out of range)");
  k_init<<<kVecBlocks, kBlock, 0, st>>>(n, rowptr, colval, val, b, x, v, rtol * rtol, maxiter);
  GFE_CUDA_TRY(cudaGetLastError());
  // The loop stops on the recursively updated residual; the true residual b - A x is then
  // recomputed, and CG restarts from x (at most kMaxRestarts times, within maxiter) when it
  // is still above rtol ||b||.
  constexpr int kMaxRestarts = 3;
  for (int restart = 0;; ++restart) {
    for (;;) {
      for (int k = 0; k < 25; ++k) {
        k_spmv_dot<<<gs, kBlock, 0, st>>>(n, rowptr, colval, val, v);
        k_update<<<kVecBlocks, kBlock, 0, st>>>(n, x, v);
        k_direction<<<kVecBlocks, kBlock, 0, st>>>(n, v);
      }
      GFE_CUDA_TRY(cudaGetLastError());
      GFE_CUDA_TRY(cudaMemcpyAsync(&h, v.S, sizeof(State), cudaMemcpyDeviceToHost, st));
      GFE_CUDA_TRY(cudaStreamSynchronize(st));
      if (h.done) break;
    }
    if (h.nonfinite) break;
    k_residual<<<gs, kBlock, 0, st>>>(n, rowptr, colval, val, b, x, v);
    GFE_CUDA_TRY(cudaGetLastError());
    GFE_CUDA_TRY(cudaMemcpyAsync(&h, v.S, sizeof(State), cudaMemcpyDeviceToHost, st));
    GFE_CUDA_TRY(cudaStreamSynchronize(st));
    const bool met = h.rr <= h.tol2;
    if (met || !h.converged || restart == kMaxRestarts || h.iter >= h.maxit) {
      h.converged = met;
      break;
    }
    k_restart<<<kVecBlocks, kBlock, 0, st>>>(n, rowptr, colval, val, b, x, v);
    GFE_CUDA_TRY(cudaGetLastError());
  }
  if (iterations) *iterations = h.iter;
  if (relres) *relres = h.bb > 0.0 && !h.nonfinite ? sqrt(h.rr / h.bb) : (h.nonfinite ? NAN : 0.0);
  if (h.nonfinite)
    return set_error(GFE_ERR_NONFINITE,
                     "gfe_cg_solve_noalloc: NaN or Inf in b, the matrix values or a reduction "
                     "after %d iterations", h.iter);
  if (!h.converged)
    return set_error(GFE_ERR_NOT_CONVERGED,
                     "gfe_cg_solve_noalloc: ||b - A x|| / ||b|| = %.3e above rtol %.3e after %d "
                     "iterations (x holds the last iterate)",
                     h.bb > 0.0 ? sqrt(h.rr / h.bb) : 0.0, rtol, h.iter);
  return GFE_OK;
}
