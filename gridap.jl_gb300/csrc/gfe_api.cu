// gfe_api.cu -- the exported C ABI (include/gfe.h): argument checking, host/device data
// movement and dispatch to the kernels. No exception or process exit crosses this layer.
#include <cstring>

#include "gfe_internal.h"

using namespace gfe;

namespace {



}  // namespace

extern "C" const char* gfe_last_error(void) { return g_last_error_ptr(); }

extern "C" const char* gfe_version(void) { return "gfe 0.1.0 (sm_103a)"; }

extern "C" int gfe_ctx_create(int device, gfe_ctx** out) {
  clear_error();
  if (!out) return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_ctx_create: out is NULL");
  *out = nullptr;
  int ndev = 0;
  GFE_CUDA_TRY(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_ctx_create: device %d of %d", device, ndev);
  DeviceGuard g(device);
  gfe_ctx* c = new gfe_ctx();
  c->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount,
                                                   device);
  if (e == cudaSuccess) {
    // a private stream-ordered pool that keeps freed memory for reuse by later steps
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    e = cudaMemPoolCreate(&c->pool, &props);
    if (e == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      e = cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  for (auto& s : c->scratch) s.owner = c;
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_err, sizeof(DevError));
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d_err, 0, sizeof(DevError), c->stream);
  if (e == cudaSuccess) e = cudaMallocHost(&c->h_pinned, 4096);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    int code = set_error(GFE_ERR_CUDA, "gfe_ctx_create: %s", cudaGetErrorString(e));
    gfe_ctx_destroy(c);
    return code;
  }
  *out = c;
  return GFE_OK;
}

extern "C" int gfe_ctx_destroy(gfe_ctx* c) {
  if (!c) return GFE_OK;
  DeviceGuard g(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->cg_exec) cudaGraphExecDestroy(c->cg_exec);
  gfe::fcg_cache_release(c);
  for (auto& s : c->scratch) s.release();
  timer_release(c);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->pool) cudaMemPoolDestroy(c->pool);
  if (c->d_err) cudaFree(c->d_err);
  if (c->h_pinned) cudaFreeHost(c->h_pinned);
  if (c->copy_fork) cudaEventDestroy(c->copy_fork);
  if (c->copy_join) cudaEventDestroy(c->copy_join);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return GFE_OK;
}

extern "C" int gfe_ctx_stream(gfe_ctx* c, void** stream) {
  clear_error();
  if (!c || !stream) return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_ctx_stream: NULL");
  *stream = (void*)c->stream;
  return GFE_OK;
}

extern "C" int gfe_ctx_synchronize(gfe_ctx* c) {
  clear_error();
  if (!c) return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_ctx_synchronize: NULL");
  DeviceGuard g(c->device);
  GFE_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return check_device_error(c, "synchronize");
}

extern "C" int gfe_ctx_kernel_launches(gfe_ctx* c, int64_t* count) {
  clear_error();
  if (!c || !count) return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_ctx_kernel_launches: NULL");
  *count = c->launches;
  return GFE_OK;
}

extern "C" int gfe_ctx_set_timing(gfe_ctx* c, int enable) {
  clear_error();
  if (!c) return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_ctx_set_timing: NULL");
  DeviceGuard g(c->device);
  GFE_TRY(timer_flush(c));
  c->timer.enabled = enable != 0;
  for (int k = 0; k < 8; ++k) {
    c->timer.total_ms[k] = 0.0;
    c->timer.count[k] = 0;
  }
  return GFE_OK;
}

extern "C" int gfe_ctx_set_wait_limit(gfe_ctx* c, uint64_t first_wait_ns) {
  clear_error();
  if (!c) return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_ctx_set_wait_limit: NULL");
  c->first_wait_ns = (unsigned long long)first_wait_ns;
  return GFE_OK;
}

extern "C" int gfe_ctx_kernel_time(gfe_ctx* c, int kernel, double* total_ms, int64_t* launches) {
  clear_error();
  if (!c || kernel < 0 || kernel >= 8 || !total_ms || !launches)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_ctx_kernel_time: bad arguments");
  DeviceGuard g(c->device);
  GFE_TRY(timer_flush(c));
  *total_ms = c->timer.total_ms[kernel];
  *launches = c->timer.count[kernel];
  return GFE_OK;
}

// ---- symbolic -----------------------------------------------------------------------------
static int symbolic_loop(gfe_ctx* ctx, int64_t ncells, int ndr, int ndc,
                         const int32_t* cell_rows, const int32_t* cell_cols,
                         const uint8_t* local_mask, int64_t nrows, int64_t ncols,
                         gfe_matrix** out, const char* who,
                         const gfe_problem* structured = nullptr) {
  gfe::NvtxRange nvtx_range(who);
  clear_error();
  if (!ctx || !out || ndr < 1 || ndc < 1 || ncells < 0 || nrows < 0 || ncols < 0 ||
      (ncells > 0 && (!cell_rows || !cell_cols)))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "%s: bad arguments", who);
  if (nrows > INT32_MAX || ncols > INT32_MAX)
    return set_error(GFE_ERR_UNSUPPORTED, "%s: more than 2^31 rows", who);
  *out = nullptr;
  DeviceGuard g(ctx->device);
  gfe_matrix* A = new gfe_matrix();
  A->ctx = ctx;
  for (gfe::DevBuf* b : {&A->rowptr, &A->colval, &A->val, &A->cell_rows, &A->cell_cols,
                         &A->ref_ptr, &A->refs, &A->refpos, &A->sell_ptr, &A->sell_col,
                         &A->sell_val64, &A->sell_val32, &A->dinv64, &A->dinv32,
                         &A->dia_val32, &A->mf_kap32, &A->mf_flag, &A->lmask})
    b->owner = ctx;
  A->nrows = nrows;
  A->ncols = ncols;
  A->nd = ndr;
  A->ndc = ndc == ndr ? 0 : ndc;
  A->ncells = ncells;
  const size_t rsz = sizeof(int32_t) * (size_t)ncells * ndr;
  const size_t csz = sizeof(int32_t) * (size_t)ncells * ndc;
  // square cells given one array for rows and columns (every FESpace assembled against
  // itself): one copy serves both
  A->cols_alias = cell_cols == cell_rows && ndc == ndr;
  int s = A->cell_rows.reserve(rsz);
  if (s == GFE_OK && !A->cols_alias) s = A->cell_cols.reserve(csz);
  // a structured problem's ids in host memory: the closed-form pattern build copies them
  // itself, beside its own kernels
  const bool host_ids = structured && A->cols_alias && !local_mask && rsz &&
                        !is_device_ptr(cell_rows);
  if (s == GFE_OK && rsz && !host_ids) {
    cudaError_t e = cudaMemcpyAsync(A->cell_rows.ptr, cell_rows, rsz, cudaMemcpyDefault,
                                    ctx->stream);
    if (e == cudaSuccess && !A->cols_alias)
      e = cudaMemcpyAsync(A->cell_cols.ptr, cell_cols, csz, cudaMemcpyDefault, ctx->stream);
    if (e != cudaSuccess) s = set_error(GFE_ERR_CUDA, "copy cell ids: %s", cudaGetErrorString(e));
  }
  if (s == GFE_OK && local_mask) {
    const size_t msz = (size_t)ndr * ndc;
    s = A->lmask.reserve(msz);
    if (s == GFE_OK) {
      cudaError_t e = cudaMemcpyAsync(A->lmask.ptr, local_mask, msz, cudaMemcpyDefault,
                                      ctx->stream);
      if (e != cudaSuccess) s = set_error(GFE_ERR_CUDA, "copy mask: %s", cudaGetErrorString(e));
      A->has_lmask = true;
    }
  }
  bool done = false;
  if (s == GFE_OK && structured)
    s = build_pattern_cartesian(ctx, A, structured->partition[0], structured->partition[1],
                                structured->partition[2], &done,
                                host_ids ? cell_rows : nullptr);
  if (s == GFE_OK && !done) s = build_pattern(ctx, A);
  if (s != GFE_OK) {
    delete A;
    return s;
  }
  *out = A;
  return GFE_OK;
}

extern "C" int gfe_symbolic_loop_matrix(gfe_ctx* ctx, int64_t ncells, int nd,
                                        const int32_t* cell_rows, const int32_t* cell_cols,
                                        int64_t nrows, int64_t ncols, gfe_matrix** out) {
  return symbolic_loop(ctx, ncells, nd, nd, cell_rows, cell_cols, nullptr, nrows, ncols, out,
                       "gfe_symbolic_loop_matrix");
}

extern "C" int gfe_symbolic_loop_matrix_rect(gfe_ctx* ctx, int64_t ncells, int nd_rows,
                                             int nd_cols, const int32_t* cell_rows,
                                             const int32_t* cell_cols, int64_t nrows,
                                             int64_t ncols, gfe_matrix** out) {
  return symbolic_loop(ctx, ncells, nd_rows, nd_cols, cell_rows, cell_cols, nullptr, nrows,
                       ncols, out, "gfe_symbolic_loop_matrix_rect");
}

extern "C" int gfe_symbolic_loop_matrix_problem(gfe_ctx* ctx, const gfe_problem* p,
                                                gfe_matrix** out) {
  if (!p || !p->cell_dof_ids || p->nd < 1)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_symbolic_loop_matrix_problem: bad problem");
  // Q1 hexahedra of a Cartesian grid: the closed-form pattern when the ids are its interior
  // numbering (checked on the device), otherwise the general symbolic loop
  const bool cart = p->dim == 3 && p->reffe == GFE_REFFE_Q1 && p->ncomp == 1 && p->nd == 8 &&
                    p->ncells == p->partition[0] * p->partition[1] * p->partition[2];
  return symbolic_loop(ctx, p->ncells, p->nd, p->nd, p->cell_dof_ids, p->cell_dof_ids, nullptr,
                       p->nfree, p->nfree, out, "gfe_symbolic_loop_matrix_problem",
                       cart ? p : nullptr);
}

extern "C" int gfe_symbolic_loop_matrix_masked(gfe_ctx* ctx, int64_t ncells, int nd_rows,
                                               int nd_cols, const int32_t* cell_rows,
                                               const int32_t* cell_cols,
                                               const uint8_t* local_mask, int64_t nrows,
                                               int64_t ncols, gfe_matrix** out) {
  if (!local_mask)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_symbolic_loop_matrix_masked: no mask");
  return symbolic_loop(ctx, ncells, nd_rows, nd_cols, cell_rows, cell_cols, local_mask, nrows,
                       ncols, out, "gfe_symbolic_loop_matrix_masked");
}

// The matrix's buffers return to the context's pool in stream order (no synchronisation).
// Destroy matrices before their context.
extern "C" int gfe_matrix_destroy(gfe_matrix* A) {
  if (!A) return GFE_OK;
  DeviceGuard g(A->ctx->device);
  delete A;
  return GFE_OK;
}

extern "C" int gfe_matrix_info(gfe_matrix* A, int64_t* nrows, int64_t* ncols, int64_t* nnz) {
  clear_error();
  if (!A) return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_matrix_info: NULL");
  if (nrows) *nrows = A->nrows;
  if (ncols) *ncols = A->ncols;
  if (nnz) *nnz = A->nnz;
  return GFE_OK;
}

__global__ void k_widen(const int32_t* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                        int64_t base) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (int64_t)in[i] + base;
}

extern "C" int gfe_matrix_export_csr(gfe_matrix* A, int index_base, int64_t* rowptr,
                                     int64_t* colval, double* nzval) {
  clear_error();
  if (!A || (index_base != 0 && index_base != 1))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_matrix_export_csr: bad arguments");
  gfe_ctx* ctx = A->ctx;
  DeviceGuard g(ctx->device);
  GFE_TRY(ensure_values(ctx, A));
  auto widen = [&](const int32_t* src, int64_t n, int64_t* dst) -> int {
    if (!dst || n == 0) return GFE_OK;
    const bool dev = is_device_ptr(dst);
    int64_t* d = dst;
    if (!dev) {
      GFE_TRY(ctx->scratch[SCR_TMP3].reserve(sizeof(int64_t) * n));
      d = ctx->scratch[SCR_TMP3].as<int64_t>();
    }
    k_widen<<<grid_for(n, 256), 256, 0, ctx->stream>>>(src, d, n, index_base);
    ctx->launches++;
    GFE_CUDA_TRY(cudaGetLastError());
    if (!dev) GFE_TRY(copy_out(ctx, dst, d, sizeof(int64_t) * n));
    return GFE_OK;
  };
  GFE_TRY(widen(A->rowptr.as<int32_t>(), A->nrows + 1, rowptr));
  GFE_TRY(widen(A->colval.as<int32_t>(), A->nnz, colval));
  if (nzval) GFE_TRY(copy_out(ctx, nzval, A->val.ptr, sizeof(double) * A->nnz));
  GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GFE_OK;
}

extern "C" int gfe_matrix_fillstored_zero(gfe_matrix* A) {
  clear_error();
  if (!A) return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_matrix_fillstored_zero: NULL");
  DeviceGuard g(A->ctx->device);
  if (A->nnz)
    GFE_CUDA_TRY(cudaMemsetAsync(A->val.ptr, 0, sizeof(double) * A->nnz, A->ctx->stream));
  A->val_pending = false;
  A->zf_values = false;
  A->plan_valid = false;
  A->dia_checked = false;
  A->mf_state = 0;
  return GFE_OK;
}

// ---- numeric, caller-provided cell arrays -------------------------------------------------
extern "C" int gfe_numeric_loop_matrix(gfe_ctx* ctx, gfe_matrix* A, const double* cellmats) {
  gfe::NvtxRange nvtx_range("gfe_numeric_loop_matrix");
  clear_error();
  if (!ctx || !A || (A->ncells > 0 && !cellmats) || A->ctx != ctx)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_numeric_loop_matrix: bad arguments");
  DeviceGuard g(ctx->device);
  GFE_TRY(ensure_values(ctx, A));
  A->zf_values = false;
  const void* d;
  GFE_TRY(device_view(ctx, cellmats, sizeof(double) * (size_t)A->ncells * A->nd * A->cols_per_cell(),
                      SCR_CELLMAT, &d));
  A->mf_state = 0;
  GFE_TRY(assemble_cellmats(ctx, A, (const double*)d));
  A->plan_valid = false;
  A->dia_checked = false;
  return GFE_OK;
}

extern "C" int gfe_numeric_loop_vector(gfe_ctx* ctx, int64_t ncells, int nd,
                                       const int32_t* cell_rows, const double* cellvecs,
                                       int64_t nrows, double* b) {
  gfe::NvtxRange nvtx_range("gfe_numeric_loop_vector");
  clear_error();
  if (!ctx || nd < 1 || ncells < 0 || nrows < 0 || !b ||
      (ncells > 0 && (!cell_rows || !cellvecs)))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_numeric_loop_vector: bad arguments");
  DeviceGuard g(ctx->device);
  const void* dr;
  const void* dv;
  GFE_TRY(device_view(ctx, cell_rows, sizeof(int32_t) * (size_t)ncells * nd, SCR_CELLIDS, &dr));
  GFE_TRY(device_view(ctx, cellvecs, sizeof(double) * (size_t)ncells * nd, SCR_CELLVEC, &dv));
  const bool bdev = is_device_ptr(b);
  double* db = b;
  if (!bdev) {
    GFE_TRY(ctx->scratch[SCR_VEC_B].reserve(sizeof(double) * (nrows > 0 ? nrows : 1)));
    db = ctx->scratch[SCR_VEC_B].as<double>();
    GFE_CUDA_TRY(cudaMemcpyAsync(db, b, sizeof(double) * nrows, cudaMemcpyHostToDevice,
                                 ctx->stream));
  }
  GFE_TRY(assemble_cellvecs(ctx, ncells, nd, (const int32_t*)dr, (const double*)dv, nrows, db));
  if (!bdev) GFE_TRY(copy_out(ctx, b, db, sizeof(double) * nrows));
  return GFE_OK;
}

// ---- fused --------------------------------------------------------------------------------
extern "C" int gfe_assemble_matrix_and_vector(gfe_ctx* ctx, const gfe_problem* p,
                                              gfe_matrix* A, double* b) {
  gfe::NvtxRange nvtx_range("gfe_assemble_matrix_and_vector");
  clear_error();
  if (!ctx || !p || (!A && !b) || p->ncells < 0 || (p->ncells > 0 && !p->cell_dof_ids))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_assemble_matrix_and_vector: bad arguments");
  if (A && A->ctx != ctx)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_assemble_matrix_and_vector: foreign matrix");
  if (A && A->nrows != p->nfree)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_assemble_matrix_and_vector: nfree %lld != "
                     "matrix rows %lld", (long long)p->nfree, (long long)A->nrows);
  DeviceGuard g(ctx->device);
  const bool bdev = b && is_device_ptr(b);
  double* db = b;
  if (b && !bdev) {
    GFE_TRY(ctx->scratch[SCR_VEC_B].reserve(sizeof(double) * (p->nfree > 0 ? p->nfree : 1)));
    db = ctx->scratch[SCR_VEC_B].as<double>();
  }
  if (A) {
    A->mf_state = 0;
    A->pmg_state = 0;
    A->p2mg_state = 0;
  }
  struct LiftReset {
    gfe_ctx* c;
    ~LiftReset() {
      c->lift_uD = nullptr;
      c->lift_ndiri = 0;
    }
  } lift_reset{ctx};
  if (A && b && p->dirichlet_values && p->ndirichlet > 0 && p->form != GFE_FORM_QUASILINEAR) {
    // nonzero Dirichlet data: the lift needs the matrix entries, so it comes with A and b
    const void* v;
    GFE_TRY(device_view(ctx, p->dirichlet_values, sizeof(double) * (size_t)p->ndirichlet,
                        SCR_DIRI, &v));
    ctx->lift_uD = static_cast<const double*>(v);
    ctx->lift_ndiri = p->ndirichlet;
  }
  GFE_TRY(assemble_problem(ctx, p, A, db));
  if (A) {
    A->plan_valid = false;
    A->dia_checked = false;
  }
  if (b && !bdev) GFE_TRY(copy_out(ctx, b, db, sizeof(double) * p->nfree));
  return GFE_OK;
}

// ---- solve --------------------------------------------------------------------------------
extern "C" int gfe_solve(gfe_ctx* ctx, gfe_matrix* A, const gfe_solver_opts* opts,
                         const double* b, double* x, gfe_solve_report* report) {
  gfe::NvtxRange nvtx_range("gfe_solve");
  clear_error();
  if (!ctx || !A || !opts || !b || !x || A->ctx != ctx)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_solve: bad arguments");
  if (!(opts->rtol > 0.0))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_solve: rtol must be positive");
  DeviceGuard g(ctx->device);
  GFE_TRY(ensure_values(ctx, A));
  const size_t n8 = sizeof(double) * (size_t)A->nrows;
  const void* db;
  GFE_TRY(device_view(ctx, b, n8, SCR_VEC_B, &db));
  const bool xdev = is_device_ptr(x);
  double* dx = x;
  if (!xdev) {
    GFE_TRY(ctx->scratch[SCR_VEC_X].reserve(n8 + 8));
    dx = ctx->scratch[SCR_VEC_X].as<double>();
    if (opts->initial_guess)  // the guess lives in the caller's host array
      GFE_CUDA_TRY(cudaMemcpyAsync(dx, x, n8, cudaMemcpyHostToDevice, ctx->stream));
  }
  gfe_solve_report rep;
  memset(&rep, 0, sizeof(rep));
  GFE_TRY(solve(ctx, A, opts, (const double*)db, dx, &rep));
  if (!xdev) GFE_TRY(copy_out(ctx, x, dx, n8));
  if (report) *report = rep;
  return check_device_error(ctx, "gfe_solve");
}

extern "C" int gfe_matrix_mul(gfe_ctx* ctx, gfe_matrix* A, const double* x, double* y) {
  gfe::NvtxRange nvtx_range("gfe_matrix_mul");
  clear_error();
  if (!ctx || !A || !x || !y || A->ctx != ctx)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_matrix_mul: bad arguments");
  DeviceGuard g(ctx->device);
  GFE_TRY(ensure_values(ctx, A));
  const void* dx;
  GFE_TRY(device_view(ctx, x, sizeof(double) * (size_t)A->ncols, SCR_TMP2, &dx));
  const bool ydev = is_device_ptr(y);
  double* dy = y;
  if (!ydev) {
    GFE_TRY(ctx->scratch[SCR_TMP3].reserve(sizeof(double) * (size_t)A->nrows + 8));
    dy = ctx->scratch[SCR_TMP3].as<double>();
  }
  GFE_TRY(spmv64(ctx, A, (const double*)dx, dy));
  if (!ydev) GFE_TRY(copy_out(ctx, y, dy, sizeof(double) * (size_t)A->nrows));
  return GFE_OK;
}
