// gfe_bicgstab.cu -- Jacobi-preconditioned BiCGStab in FP64 for non-symmetric systems (the
// Jacobians of quasilinear forms whose coefficient depends on u, Nitsche forms with a
// non-symmetric variant). Gridap's default for these is a direct solve (BackslashSolver,
// Algebra/LinearSolvers.jl:221-260); behind the same LinearSolver protocol this is the
// iterative GPU counterpart.
//
// Preconditioned BiCGStab (van der Vorst 1992, right preconditioning with M = diag(A)):
//   r = b - A x, rh = r, rho = alpha = omega = 1, v = p = 0
//   repeat: rho' = rh.r; beta = (rho'/rho)(alpha/omega); p = r + beta (p - omega v);
//           y = M^-1 p; v = A y; alpha = rho'/(rh.v); s = r - alpha v; z = M^-1 s;
//           t = A z; omega = (t.s)/(t.t); x += alpha y + omega z; r = s - omega t.
// The SpMV is the solver plan's sliced-ELL FP64 kernel. Dot products use a fixed grid with
// per-block partials summed in block order, so runs are deterministic. When the recursive
// residual meets the tolerance the true residual b - A x is formed; if it does not meet it,
// the iteration restarts from it (at most 20 restarts).
#include <cmath>
#include <vector>

#include "gfe_internal.h"

namespace gfe {
namespace {

constexpr int kBlk = 256;

// per-block partial sums of up to 3 dot products (a0.b0, a1.b1, a2.b2)
__global__ void __launch_bounds__(kBlk)
    k_dots(int64_t n, int k, const double* __restrict__ a0, const double* __restrict__ b0,
           const double* __restrict__ a1, const double* __restrict__ b1,
           const double* __restrict__ a2, const double* __restrict__ b2,
           double* __restrict__ partials) {
  __shared__ double sh[3][kBlk / 32];
  double s[3] = {0.0, 0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * kBlk + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kBlk) {
    s[0] += a0[i] * b0[i];
    if (k > 1) s[1] += a1[i] * b1[i];
    if (k > 2) s[2] += a2[i] * b2[i];
  }
  for (int j = 0; j < 3; ++j)
    for (int off = 16; off > 0; off >>= 1) s[j] += __shfl_down_sync(0xffffffffu, s[j], off);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
    for (int j = 0; j < 3; ++j) sh[j][wid] = s[j];
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < kBlk / 32; ++w) t += sh[threadIdx.x][w];
    partials[(int64_t)blockIdx.x * 3 + threadIdx.x] = t;
  }
}

// one thread per dot product: partials summed in block order
__global__ void k_sum_partials(int nblocks, const double* __restrict__ partials,
                               double* __restrict__ out) {
  if (threadIdx.x >= 3) return;
  double t = 0.0;
  for (int b = 0; b < nblocks; ++b) t += partials[(int64_t)b * 3 + threadIdx.x];
  out[threadIdx.x] = t;
}

// p = r + beta (p - omega v) (beta = 0 on the first step: p = r); y = dinv p
__global__ void k_bicg_dir(int64_t n, double beta, double omega, const double* __restrict__ r,
                           const double* __restrict__ v, const double* __restrict__ dinv,
                           double* __restrict__ p, double* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * kBlk + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kBlk) {
    const double pi = r[i] + beta * (p[i] - omega * v[i]);
    p[i] = pi;
    y[i] = dinv[i] * pi;
  }
}

// s = r - alpha v; z = dinv s
__global__ void k_bicg_half(int64_t n, double alpha, const double* __restrict__ r,
                            const double* __restrict__ v, const double* __restrict__ dinv,
                            double* __restrict__ s, double* __restrict__ z) {
  for (int64_t i = (int64_t)blockIdx.x * kBlk + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kBlk) {
    const double si = r[i] - alpha * v[i];
    s[i] = si;
    z[i] = dinv[i] * si;
  }
}

// x += alpha y + omega z; r = s - omega t
__global__ void k_bicg_update(int64_t n, double alpha, double omega,
                              const double* __restrict__ y, const double* __restrict__ z,
                              const double* __restrict__ s, const double* __restrict__ t,
                              double* __restrict__ x, double* __restrict__ r) {
  for (int64_t i = (int64_t)blockIdx.x * kBlk + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kBlk) {
    x[i] += alpha * y[i] + omega * z[i];
    r[i] = s[i] - omega * t[i];
  }
}

// r = b - Ax (Ax given); rh = r
__global__ void k_bicg_residual(int64_t n, const double* __restrict__ b,
                                const double* __restrict__ ax, double* __restrict__ r,
                                double* __restrict__ rh) {
  for (int64_t i = (int64_t)blockIdx.x * kBlk + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kBlk) {
    const double ri = b[i] - ax[i];
    r[i] = ri;
    rh[i] = ri;
  }
}

struct Dots {
  gfe_ctx* ctx;
  int64_t n;
  unsigned grid;
  double* partials;
  double* out;  // device, 3 values
  double h[3];
  int run(int k, const double* a0, const double* b0, const double* a1 = nullptr,
          const double* b1 = nullptr, const double* a2 = nullptr, const double* b2 = nullptr) {
    k_dots<<<grid, kBlk, 0, ctx->stream>>>(n, k, a0, b0, a1, b1, a2, b2, partials);
    k_sum_partials<<<1, 32, 0, ctx->stream>>>((int)grid, partials, out);
    ctx->launches += 2;
    GFE_CUDA_TRY(cudaGetLastError());
    return copy_out(ctx, h, out, sizeof(double) * 3);
  }
};

}  // namespace

// x (device, n) starts at zero; dinv = the Jacobi scaling (ones without a preconditioner).
int bicgstab(gfe_ctx* ctx, gfe_matrix* A, const double* dinv, const double* d_b, double* d_x,
             double rtol, int maxit, int* iterations) {
  const int64_t n = A->nrows;
  *iterations = 0;
  GFE_TRY(build_solver_plan(ctx, A));
  DevBuf work(ctx);
  const unsigned grid = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>((n + kBlk - 1) / kBlk, (int64_t)ctx->num_sms * 8));
  const size_t nn = (size_t)(n > 0 ? n : 1);
  GFE_TRY(work.reserve(sizeof(double) * (nn * 8 + (size_t)grid * 3 + 8)));
  double* r = work.as<double>();
  double* rh = r + nn;
  double* p = rh + nn;
  double* v = p + nn;
  double* s = v + nn;
  double* y = s + nn;
  double* z = y + nn;
  double* t = z + nn;
  Dots dots{ctx, n, grid, t + nn, t + nn + (size_t)grid * 3, {0, 0, 0}};
  GFE_CUDA_TRY(cudaMemsetAsync(d_x, 0, sizeof(double) * nn, ctx->stream));
  GFE_TRY(dots.run(1, d_b, d_b));
  const double bb = dots.h[0];
  if (!std::isfinite(bb)) return set_error(GFE_ERR_NONFINITE, "bicgstab: b is not finite");
  if (bb == 0.0) return GFE_OK;
  const double tol2 = rtol * rtol * bb;
  int it = 0;
  for (int restart = 0; restart <= 20 && it < maxit; ++restart) {
    // r = rh = b - A x
    GFE_TRY(spmv64(ctx, A, d_x, t));
    k_bicg_residual<<<grid, kBlk, 0, ctx->stream>>>(n, d_b, t, r, rh);
    ctx->launches++;
    GFE_TRY(dots.run(1, r, r));
    double rr = dots.h[0];
    if (!std::isfinite(rr)) return set_error(GFE_ERR_NONFINITE, "bicgstab: residual not finite");
    if (rr <= tol2) break;
    GFE_CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(double) * nn * 2, ctx->stream));  // p, v
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    bool first = true, breakdown = false;
    while (it < maxit) {
      if (!first) {  // rh.r and r.r of the updated residual
        GFE_TRY(dots.run(2, rh, r, r, r));
        rr = dots.h[1];
        if (!std::isfinite(rr))
          return set_error(GFE_ERR_NONFINITE, "bicgstab: residual not finite");
        if (rr <= tol2) break;
      } else {
        GFE_TRY(dots.run(1, rh, r));
      }
      const double rho1 = dots.h[0];
      if (rho1 == 0.0 || !std::isfinite(rho1)) {
        breakdown = true;
        break;
      }
      const double beta = first ? 0.0 : (rho1 / rho) * (alpha / omega);
      k_bicg_dir<<<grid, kBlk, 0, ctx->stream>>>(n, beta, omega, r, v, dinv, p, y);
      ctx->launches++;
      GFE_TRY(spmv64(ctx, A, y, v));
      GFE_TRY(dots.run(1, rh, v));
      const double rv = dots.h[0];
      if (rv == 0.0 || !std::isfinite(rv)) {
        breakdown = true;
        break;
      }
      alpha = rho1 / rv;
      if (!std::isfinite(alpha)) {
        breakdown = true;
        break;
      }
      k_bicg_half<<<grid, kBlk, 0, ctx->stream>>>(n, alpha, r, v, dinv, s, z);
      ctx->launches++;
      GFE_TRY(spmv64(ctx, A, z, t));
      GFE_TRY(dots.run(3, t, s, t, t, s, s));
      const double ts = dots.h[0], tt = dots.h[1], ss = dots.h[2];
      if (!std::isfinite(ts) || !std::isfinite(tt) || !std::isfinite(ss))
        return set_error(GFE_ERR_NONFINITE, "bicgstab: half-step residual not finite");
      // the half step already converged (s = r - alpha v small): x += alpha y and stop, before
      // t = A z ~ 0 makes omega = t.s / t.t meaningless
      const bool half_done = ss <= tol2;
      omega = (half_done || !(tt > 0.0)) ? 0.0 : ts / tt;
      if (!std::isfinite(omega)) omega = 0.0;
      k_bicg_update<<<grid, kBlk, 0, ctx->stream>>>(n, alpha, omega, y, z, s, t, d_x, r);
      ctx->launches++;
      GFE_CUDA_TRY(cudaGetLastError());
      ++it;
      rho = rho1;
      first = false;
      if (half_done) break;  // the restart loop confirms with the true residual
      if (omega == 0.0) {
        breakdown = true;
        break;
      }
    }
    (void)breakdown;  // a breakdown restarts from the true residual
  }
  *iterations = it;
  return GFE_OK;
}

}  // namespace gfe
