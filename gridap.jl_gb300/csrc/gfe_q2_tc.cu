// gfe_q2_tc.cu -- Q2 diffusion cell matrices and vectors on the 5th-generation tensor cores
// (tcgen05 kind::f16, FP16 operands with per-cell scaling, FP32 accumulation in tensor memory).
//
// For a cell with (tri)linear geometry Gridap's stiffness (Fields/FieldsInterfaces.jl:708-720)
//   K[i + 27 j] = sum_q (kappa invJt grad phi_i).(invJt grad phi_j) |det Jt| w_q
//              = sum_q sum_{k,l} B[q,k,i] G_q[k][l] B[q,l,j],
//   B[q,k,i] = d phi_hat_i / d xi_k (xi_q),  G_q = kappa |det Jt_q| w_q invJt_q^T invJt_q,
// is linear in the 6 distinct entries of each symmetric G_q. So every cell's 729 entries are
// one column of a single dense product
//   K[g, cell] = sum_{(q, kl)} E[g, (q, kl)] Gs[(q, kl), cell],      g = i + 27 j,
// with Gs the cell's 162 values (G_q00, G_q01, G_q02, G_q11, G_q12, G_q22) and E a constant
// table: B[q,k,i] B[q,k,j] for kl = (k, k), B[q,k,i] B[q,l,j] + B[q,l,i] B[q,k,j] for k < l
// (K = 176 after padding).
//
// Zero row sums. Every 27 x 27 block E[(i, j), (q, kl)] has zero row and column sums (sum_j
// B[q,l,j] = 0: constants are in the kernel of the gradient). Rounded to FP16 entry by entry,
// every cell matrix would inherit the same small defect in its row sums -- an O(1e-4) reaction
// term, identical in all cells, that moves the solution of the assembled system far more than
// random rounding does. So 27 more rows of the product carry each column's defect,
// S[j, (q, kl)] = 2^12 sum_i E16[(i, j), (q, kl)] (exact sums of the rounded table, scaled into
// FP16's range), and the epilogue subtracts 2^-12 (S Gs)[j] from the diagonal entry K[j][j]:
// every row and column of every cell matrix then sums to zero up to FP32 rounding.
//
// Two kernels:
//   k_q2_metric (a CTA per 64-cell tile, a thread per cell and q-plane): the Jacobians from
//     the tensor structure of the trilinear map (the nine points of a q-plane share its edge
//     vectors), G_q = kappa w adj(Jt Jt^T) / |det Jt| in FP32, scaled per cell and rounded to
//     FP16 straight into the MMA operand layout of the tile (64 cells x 176, K-major), the
//     per-cell scales, and the load vector b_i = sum_q f_q phi_i(xi_q) |det Jt_q| w_q in FP32;
//   k_q2_cells_tc (two CTA kinds over the rows of E, each keeping its 384 x 176 FP16 part of
//     E -- 135 KB -- resident in shared memory for the whole launch):
//       kind 0: g = 0 .. 369 and the defect rows of j = 0 .. 13 (whose diagonals g = 28 j);
//       kind 1: g = 370 .. 728 and the defect rows of j = 14 .. 26.
//     Warp 8 streams the metric tiles in with bulk (TMA) copies into a 3-deep ring and issues
//     3 x 11 MMAs (M = 128, N = 64, K = 16) per tile into one of two tensor-memory
//     accumulators (192 columns each); warps 0-7 read the accumulators back (tcgen05.ld, two
//     warps per 32-lane quadrant, 32 cells each), apply the defect correction and the cell
//     scale, and store the cell matrices with coalesced stores (a warp writes 32 consecutive
//     entries of one cell matrix per instruction).
// Every mbarrier wait is bounded (1 s) and reports GFE_ERR_TIMEOUT.
//
// Precision: FP16 operands carry 11 significant bits, as TF32; the per-cell scale (|kappa|
// times the first edge's length) keeps the scaled metric entries within FP16's normal range.
// The geometric factors are FP32: their rounding (1e-7) is far below the operand rounding that
// bounds this path (5e-4); the FP64 path (k_q2_cells_fp64) keeps FP64 geometry.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_fp16.h>
#include <vector>

#include "gfe_internal.h"

namespace gfe {
namespace q2tc {

constexpr int kNN = 27;                        // Q2 HEX nodes
constexpr int kNQ = 27;                        // degree-4 tensor Gauss points
constexpr int kNV = 8;                         // geometry vertices
constexpr int kRowsK = kNN * kNN;              // 729 matrix rows
constexpr int kSplit = 370;                    // first matrix row of kind 1
constexpr int kHalfRows = 384;                 // rows per CTA kind (3 M-tiles)
constexpr int kKG = kNQ * 6;                   // 162 metric columns
constexpr int kK = 176;                        // + 14 padding columns
constexpr int kCells = 64;                     // cells per tile (MMA N)
constexpr int kSBO = (kK / 8) * 128;           // bytes between 8-row groups (2816)
constexpr int kATile = 128 / 8 * kSBO;         // bytes of one 128-row M-tile (45056)
constexpr int kABytes = kHalfRows / 8 * kSBO;  // 135168
constexpr int kBBytes = kCells / 8 * kSBO;     // 22528: one metric tile
constexpr int kRing = 3;                       // metric tiles in flight
constexpr int kEpiWarps = 8;                   // two per tensor-memory lane quadrant
constexpr int kEpi = kEpiWarps * 32;
constexpr int kMmaWarp = kEpiWarps;
constexpr int kThreads = kEpi + 32;            // 288
constexpr int kTmemCols = 512;                 // two accumulators of 3 x 64 columns
constexpr int kMetricThreads = kCells * 3;     // k_q2_metric: a thread per cell and q-plane
constexpr float kDefectScale = 4096.f;         // 2^12
constexpr unsigned long long kWaitLimitNs = 1000000000ull;

// rows of the kinds: first matrix row, matrix rows, first defect column j, defect rows
__host__ __device__ constexpr int kind_g0(int h) { return h ? kSplit : 0; }
__host__ __device__ constexpr int kind_ng(int h) { return h ? kRowsK - kSplit : kSplit; }
__host__ __device__ constexpr int kind_j0(int h) { return h ? 14 : 0; }
__host__ __device__ constexpr int kind_nj(int h) { return h ? 13 : 14; }

struct Xi {
  float x[3];  // 1-D Gauss points on [0, 1]; q = q0 + 3 q1 + 9 q2
};

struct __align__(1024) Smem {
  uint8_t A[kABytes];
  uint8_t B[kRing][kBBytes];
  float scl[kRing + 1][kCells];  // the cells' metric scales of step j in slot j % 4
  float Cs[2][14][kCells];   // per accumulator: the defect rows of this kind
  uint64_t full[kRing], done[2], freeb[2], tab;
  uint32_t tmem_base;
  int error;
  int estop;  // the epilogue's decision to stop (written by one thread before a barrier)
};

__device__ __host__ __forceinline__ int canon_off(int row, int k) {
  return (row & 7) * 16 + (row >> 3) * kSBO + (k >> 3) * 128 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);        // start address
  d |= (uint64_t)((128 >> 4) & 0x3FFF) << 16;   // K-adjacent core matrices
  d |= (uint64_t)((kSBO >> 4) & 0x3FFF) << 32;  // next 8-row group
  d |= (uint64_t)1 << 46;                       // descriptor version (sm_100 family)
  return d;                                     // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: D = F32, A = B = F16, both K-major, N = 64, M = 128
__device__ __forceinline__ uint32_t idesc_f16() {
  return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(kCells >> 3) << 17) |
         ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait on an mbarrier phase: gives up after kWaitLimitNs of wall-clock time.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase) {
  const unsigned long long t0 = globaltimer_ns();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
    if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
  }
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void epilogue_sync() {
  asm volatile("bar.sync 2, %0;" ::"n"(kEpi) : "memory");
}

// 32 consecutive accumulator columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,"
      "%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, "
      "[%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}


// ---- the metric tiles --------------------------------------------------------------------
// CTA = one 64-cell tile, thread = (cell c, q-plane q2). Writes the tile's B operand (FP16,
// K-major canonical layout, gs + tile * kBBytes), the cells' scales and their load vectors.
__global__ void __launch_bounds__(kMetricThreads)
    k_q2_metric(int64_t ncells, const int32_t* __restrict__ cell_vertices,
                const double* __restrict__ coords, const double* __restrict__ tabs,
                const Xi xi, int coef_kind, const double* __restrict__ coef, int src_kind,
                const double* __restrict__ src, uint8_t* __restrict__ gs,
                float* __restrict__ scl, float* __restrict__ bvec, DevError* err) {
  __shared__ float X[kCells][kNV][3];
  __shared__ float fdv[kCells][kNQ + 1];
  __shared__ float phi2[kNQ * kNN];
  __shared__ float w[kNQ];
  const int tid = threadIdx.x;
  const int64_t tile = blockIdx.x, cell0 = tile * kCells;
  for (int i = tid; i < kNQ; i += kMetricThreads) w[i] = (float)tabs[i];
  for (int i = tid; i < kNQ * kNN; i += kMetricThreads) phi2[i] = (float)tabs[kNQ + i];
  for (int idx = tid; idx < kCells * kNV; idx += kMetricThreads) {
    const int cc = idx / kNV, a = idx % kNV;
    const int64_t cell = cell0 + cc;
    float x0 = 0.f, x1 = 0.f, x2 = 0.f;
    if (cell < ncells) {
      const double* x = coords + ((int64_t)__ldg(cell_vertices + cell * kNV + a) - 1) * 3;
      x0 = (float)__ldg(x);
      x1 = (float)__ldg(x + 1);
      x2 = (float)__ldg(x + 2);
    }
    X[cc][a][0] = x0;
    X[cc][a][1] = x1;
    X[cc][a][2] = x2;
  }
  __syncthreads();
  const int c = tid / 3, plane = tid % 3;
  const int64_t cell = cell0 + c;
  uint8_t* tb = gs + tile * kBBytes;
  auto put2 = [&](int k, float a, float b) {
    *reinterpret_cast<__half2*>(tb + canon_off(c, k)) = __floats2half2_rn(a, b);
  };
  if (cell >= ncells) {
    for (int q = 9 * plane; q < 9 * plane + 9; ++q) {
#pragma unroll
      for (int pr = 0; pr < 3; ++pr) put2(q * 6 + 2 * pr, 0.f, 0.f);
      fdv[c][q] = 0.f;
    }
    if (plane == 0) {
      for (int k = kKG; k < kK; k += 2) put2(k, 0.f, 0.f);
      scl[cell0 + c] = 1.f;
    }
  } else {
    const float kap = coef_kind == GFE_COEF_CELL   ? (float)__ldg(coef + cell)
                      : coef_kind == GFE_COEF_CONST ? (float)__ldg(coef)
                                                    : 1.f;
    const float fc = src_kind == GFE_SRC_CONST ? (float)__ldg(src) : 0.f;
    float Xr[kNV][3];
#pragma unroll
    for (int a = 0; a < kNV; ++a)
#pragma unroll
      for (int d = 0; d < 3; ++d) Xr[a][d] = X[c][a][d];
    const float ex = Xr[1][0] - Xr[0][0], ey = Xr[1][1] - Xr[0][1], ez = Xr[1][2] - Xr[0][2];
    float sk = fabsf(kap) * sqrtf(ex * ex + ey * ey + ez * ez);
    if (!(sk > 0.f) || !isfinite(sk)) sk = 1.f;
    const float isk = __fdividef(1.f, sk);
    // edge vectors of the trilinear map (vertex a = a0 + 2 a1 + 4 a2; l_0 = 1 - xi,
    // l_1 = xi), contracted with this plane's xi_2 where they depend on it:
    //   d x / d xi_0 = sum_{a1} l_{a1}(xi_1) D0[a1],
    //   d x / d xi_1 = sum_{a0} l_{a0}(xi_0) D1[a0],
    //   d x / d xi_2 = sum_{a0, a1} l_{a0}(xi_0) l_{a1}(xi_1) D2[a0][a1]
    const float t1 = plane == 0 ? xi.x[0] : plane == 1 ? xi.x[1] : xi.x[2], t0 = 1.f - t1;
    float D0[2][3], D1[2][3], D2[2][2][3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        D0[u][d] = t0 * (Xr[1 + 2 * u][d] - Xr[0 + 2 * u][d]) +
                   t1 * (Xr[5 + 2 * u][d] - Xr[4 + 2 * u][d]);
        D1[u][d] = t0 * (Xr[u + 2][d] - Xr[u][d]) + t1 * (Xr[u + 6][d] - Xr[u + 4][d]);
#pragma unroll
        for (int v = 0; v < 2; ++v) D2[u][v][d] = Xr[u + 2 * v + 4][d] - Xr[u + 2 * v][d];
      }
    }
    float R1[3][3];
#pragma unroll
    for (int q0 = 0; q0 < 3; ++q0)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        R1[q0][d] = (1.f - xi.x[q0]) * D1[0][d] + xi.x[q0] * D1[1][d];
#pragma unroll
    for (int q1 = 0; q1 < 3; ++q1) {
      const float u1 = xi.x[q1], u0 = 1.f - u1;
      float R0[3], T[2][3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        R0[d] = u0 * D0[0][d] + u1 * D0[1][d];
        T[0][d] = u0 * D2[0][0][d] + u1 * D2[0][1][d];
        T[1][d] = u0 * D2[1][0][d] + u1 * D2[1][1][d];
      }
#pragma unroll
      for (int q0 = 0; q0 < 3; ++q0) {
        const int q = q0 + 3 * q1 + 9 * plane;
        float J[3][3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          J[0][d] = R0[d];
          J[1][d] = R1[q0][d];
          J[2][d] = (1.f - xi.x[q0]) * T[0][d] + xi.x[q0] * T[1][d];
        }
        // G = kappa |det Jt| w invJt^T invJt = kappa w adj(M) / |det Jt| with M = Jt Jt^T
        // (invJt^T invJt = M^-1 = adj(M) / det(Jt)^2)
        const float det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) +
                          J[0][1] * (J[1][2] * J[2][0] - J[1][0] * J[2][2]) +
                          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        if (!(det != 0.f) || !isfinite(det)) {
          if (atomicCAS(&err->code, 0, GFE_ERR_DEGENERATE_CELL) == 0) err->index = cell;
        }
        float M[3][3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int l = k; l < 3; ++l)
            M[k][l] = J[k][0] * J[l][0] + J[k][1] * J[l][1] + J[k][2] * J[l][2];
        const float adj[6] = {M[1][1] * M[2][2] - M[1][2] * M[1][2],
                              M[0][2] * M[1][2] - M[0][1] * M[2][2],
                              M[0][1] * M[1][2] - M[0][2] * M[1][1],
                              M[0][0] * M[2][2] - M[0][2] * M[0][2],
                              M[0][1] * M[0][2] - M[0][0] * M[1][2],
                              M[0][0] * M[1][1] - M[0][1] * M[0][1]};
        const float adet = fabsf(det);
        const float wq = w[q];
        const float sc = __fdividef(kap * wq * isk, adet);
#pragma unroll
        for (int pr = 0; pr < 3; ++pr) put2(q * 6 + 2 * pr, sc * adj[2 * pr], sc * adj[2 * pr + 1]);
        float f = 0.f;
        if (src_kind == GFE_SRC_CONST)
          f = fc;
        else if (src_kind == GFE_SRC_QPOINT)
          f = (float)__ldg(src + cell * kNQ + q);
        fdv[c][q] = f * adet * wq;
      }
    }
    if (plane == 0) {
      for (int k = kKG; k < kK; k += 2) put2(k, 0.f, 0.f);
      scl[cell0 + c] = sk;
    }
  }
  __syncthreads();
  // load vectors: b_i = sum_q phi_i(xi_q) f_q |det Jt_q| w_q, coalesced over (cell, i)
  if (bvec) {
    for (int idx = tid; idx < kCells * kNN; idx += kMetricThreads) {
      const int cc = idx / kNN, i = idx % kNN;
      if (cell0 + cc >= ncells) continue;
      float acc = 0.f;
#pragma unroll 9
      for (int q = 0; q < kNQ; ++q) acc = fmaf(phi2[q * kNN + i], fdv[cc][q], acc);
      bvec[cell0 * kNN + idx] = src_kind == GFE_SRC_NONE ? 0.f : acc;
    }
  }
}

// ---- the tensor-core product -------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 1)
    k_q2_cells_tc(int64_t ncells, const uint8_t* __restrict__ etab,
                  const uint8_t* __restrict__ gs, const float* __restrict__ scl,
                  float* __restrict__ K, DevError* err) {
  extern __shared__ uint8_t smem_raw[];
  Smem& s = *reinterpret_cast<Smem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                     ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int half = (int)(blockIdx.x & 1);
  const int64_t pair = blockIdx.x >> 1, npairs = gridDim.x >> 1;
  const int64_t ntiles = (ncells + kCells - 1) / kCells;
  if (tid == 0) {
    s.error = 0;
    for (int r = 0; r < kRing; ++r)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s.full[r])));
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s.done[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&s.freeb[b])),
                   "r"(kEpi));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s.tab)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&s.tmem_base)),
                 "n"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s.tmem_base;

  if (warp == kMmaWarp) {
    // ---- loads and MMA issue (one thread) ----------------------------------------------
    if (lane == 0) {
      // this kind's part of E into shared memory: bulk copies completing on s.tab
      const uint32_t tab = smem_u32(&s.tab);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tab),
                   "r"(kABytes)
                   : "memory");
      const uint8_t* src_tab = etab + (size_t)half * kABytes;
      for (int c = 0; c < kABytes / kATile; ++c)  // one copy per M-tile
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
            "[%3];" ::"r"(smem_u32(s.A + c * kATile)),
            "l"(src_tab + c * kATile), "n"(kATile), "r"(tab)
            : "memory");
      // the metric tile of step j into ring slot j % kRing, its scales into slot j % 4
      const int64_t nsteps = pair < ntiles ? (ntiles - 1 - pair) / npairs + 1 : 0;
      int64_t issued = 0;
      auto issue = [&](int64_t j) {
        const int r = (int)(j % kRing), r4 = (int)(j % (kRing + 1));
        const int64_t t = pair + j * npairs;
        const uint32_t bar = smem_u32(&s.full[r]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                     "n"(kBBytes + kCells * 4)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
            "[%3];" ::"r"(smem_u32(s.B[r])),
            "l"(gs + t * kBBytes), "n"(kBBytes), "r"(bar)
            : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
            "[%3];" ::"r"(smem_u32(s.scl[r4])),
            "l"(scl + t * kCells), "n"(kCells * 4), "r"(bar)
            : "memory");
        issued = j + 1;
      };
      for (int64_t j = 0; j < kRing - 1 && j < nsteps; ++j) issue(j);
      bool ok = mbar_wait(tab, 0);
      const uint32_t idesc = idesc_f16();
      const uint32_t a0 = smem_u32(s.A);
      int64_t step = 0;
      for (; ok && step < nsteps; ++step) {
        const int b = (int)(step & 1), r = (int)(step % kRing);
        // the accumulator of step - 2 is drained (its epilogue also read scale slot
        // (step - 2) % 4, which the copy below refills)
        if (step >= 2 && !mbar_wait(smem_u32(&s.freeb[b]), (uint32_t)(((step >> 1) - 1) & 1))) {
          ok = false;
          break;
        }
        // the MMA of step - 1 has read its ring slot, which the copy for step + 2 reuses
        if (step >= 1 &&
            !mbar_wait(smem_u32(&s.done[(step - 1) & 1]), (uint32_t)(((step - 1) >> 1) & 1))) {
          ok = false;
          break;
        }
        if (step + kRing - 1 < nsteps) issue(step + kRing - 1);
        if (!mbar_wait(smem_u32(&s.full[r]), (uint32_t)((step / kRing) & 1))) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t b0 = smem_u32(s.B[r]);
        for (int mt = 0; mt < 3; ++mt) {
          const uint32_t dcol = tmem + (uint32_t)(b * 192 + mt * kCells);
          for (int ks = 0; ks < kK / 16; ++ks) {
            const uint64_t ad = smem_desc(a0 + mt * kATile + ks * 256);
            const uint64_t bd = smem_desc(b0 + ks * 256);
            const uint32_t acc = ks > 0 ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dcol),
                "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
          }
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&s.done[b]))
            : "memory");
      }
      // the last commits and copies complete before shared and tensor memory are released
      for (int64_t back = 1; back <= 2 && step - back >= 0; ++back) {
        const int64_t st = step - back;
        mbar_wait(smem_u32(&s.done[st & 1]), (uint32_t)((st >> 1) & 1));
      }
      for (int64_t j = step; j < issued; ++j)
        mbar_wait(smem_u32(&s.full[j % kRing]), (uint32_t)((j / kRing) & 1));
      if (!ok) atomicExch(&s.error, 1);
    }
    __syncwarp();
  } else {
    // ---- epilogue: accumulators to the cell matrices --------------------------------------
    const int g0 = kind_g0(half), ng = kind_ng(half), j0 = kind_j0(half), nj = kind_nj(half);
    const int quad = warp & 3, chalf = warp >> 2;  // lane quadrant, 32-cell half of the tile
    const uint32_t lanes = (uint32_t)(quad * 32) << 16;
    int64_t step = 0;
    for (int64_t t = pair; t < ntiles; t += npairs, ++step) {
      const int b = (int)(step & 1), r4 = (int)(step % (kRing + 1));
      // one thread waits and decides for the eight warps (the named barriers below need all
      // of them, so they leave together or none does)
      if (tid == 0) {
        int stop = s.error;
        if (!stop && !mbar_wait(smem_u32(&s.done[b]), (uint32_t)((step >> 1) & 1))) stop = 1;
        if (stop) atomicExch(&s.error, 1);
        s.estop = stop;
      }
      epilogue_sync();
      if (s.estop) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int64_t cell0 = t * kCells;
      const int live = (int)((ncells - cell0) < kCells ? (ncells - cell0) : kCells);
      const int cb = 32 * chalf;  // first cell of this warp's half
      uint32_t v[32];
      // M-tile 2 first: it holds the defect rows, which the diagonals of all tiles need
      tmem_ld32(tmem + lanes + (uint32_t)(b * 192 + 2 * kCells + cb), v);
      {
        const int lr = 256 + quad * 32 + lane;  // local row
        if (lr >= ng && lr < ng + nj) {
#pragma unroll
          for (int cc = 0; cc < 32; ++cc) s.Cs[b][lr - ng][cb + cc] = __uint_as_float(v[cc]);
        }
      }
      epilogue_sync();
      for (int mt = 2; mt >= 0; --mt) {
        if (mt < 2) {
          __syncwarp();
          tmem_ld32(tmem + lanes + (uint32_t)(b * 192 + mt * kCells + cb), v);
        }
        const int lr = mt * 128 + quad * 32 + lane;
        if (lr < ng) {
          const int g = g0 + lr;
          const int jd = g % 28 == 0 ? g / 28 - j0 : -1;  // diagonal entry (j, j), j = g / 28
          float* dst = K + (cell0 + cb) * kRowsK + g;
          if (jd >= 0) {
#pragma unroll
            for (int cc = 0; cc < 32; ++cc)
              v[cc] = __float_as_uint(__uint_as_float(v[cc]) - s.Cs[b][jd][cb + cc] / kDefectScale);
          }
          if (cb + 32 <= live) {
#pragma unroll
            for (int cc = 0; cc < 32; ++cc)
              dst[(int64_t)cc * kRowsK] = __uint_as_float(v[cc]) * s.scl[r4][cb + cc];
          } else {
#pragma unroll
            for (int cc = 0; cc < 32; ++cc)
              if (cb + cc < live)
                dst[(int64_t)cc * kRowsK] = __uint_as_float(v[cc]) * s.scl[r4][cb + cc];
          }
        }
      }
      // accumulator read, defects and scales used: the buffers may be refilled
      asm volatile("tcgen05.fence::before_thread_sync;");
      mbar_arrive(smem_u32(&s.freeb[b]));
    }
  }
  // release tensor memory (the allocating warp), after every role has finished
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == kMmaWarp)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "n"(kTmemCols));
  if (tid == 0 && s.error)
    if (atomicCAS(&err->code, 0, GFE_ERR_TIMEOUT) == 0) err->index = blockIdx.x;
}

// The E table in the operand layout of both CTA kinds (FP16, 2 x 384 rows, K = 176), from the
// FP64 reference tables w | phi2 | dphi1 | B[(q*3+k)*27 + i]: the matrix rows rounded to
// nearest, then the defect rows 2^12 sum_i E16[(i, j), :] (sums of the rounded entries).
void build_etab(const double* tabs, std::vector<uint16_t>& out) {
  const double* B = tabs + kNQ + kNQ * kNN + kNQ * kNV * 3;
  out.assign((size_t)2 * kABytes / 2, 0);
  auto put = [&](int h, int lr, int k, double v) {
    const __half hv = __double2half(v);
    uint16_t bits;
    memcpy(&bits, &hv, 2);
    out[((size_t)h * kABytes + (size_t)canon_off(lr, k)) / 2] = bits;
  };
  const int kk[6] = {0, 0, 0, 1, 1, 2}, ll[6] = {0, 1, 2, 1, 2, 2};
  for (int q = 0; q < kNQ; ++q)
    for (int kl = 0; kl < 6; ++kl) {
      const int k = kk[kl], l = ll[kl], col = q * 6 + kl;
      double colsum[kNN] = {0.0};
      for (int j = 0; j < kNN; ++j)
        for (int i = 0; i < kNN; ++i) {
          double v = B[(q * 3 + k) * kNN + i] * B[(q * 3 + l) * kNN + j];
          if (k != l) v += B[(q * 3 + l) * kNN + i] * B[(q * 3 + k) * kNN + j];
          colsum[j] += (double)__half2float(__double2half(v));
          const int g = i + kNN * j;
          const int h = g >= kSplit ? 1 : 0;
          put(h, g - kind_g0(h), col, v);
        }
      for (int j = 0; j < kNN; ++j) {
        const int h = j >= kind_j0(1) ? 1 : 0;
        put(h, kind_ng(h) + (j - kind_j0(h)), col, colsum[j] * (double)kDefectScale);
      }
    }
}

}  // namespace q2tc

size_t q2_tc_smem_bytes() { return sizeof(q2tc::Smem) + 1024; }

int launch_q2_cells_tc(gfe_ctx* ctx, int64_t ncells, const int32_t* cell_vertices,
                       const double* coords, const double* tabs, const double* htabs,
                       int coef_kind, const double* coef, int src_kind, const double* src,
                       float* K, float* bvec) {
  using namespace q2tc;
  // the E table depends only on the reference element: built and uploaded once per context
  DevBuf& et = ctx->scratch[SCR_Q2TAB];
  if (!ctx->q2tab_valid) {
    std::vector<uint16_t> h;
    build_etab(htabs, h);
    GFE_TRY(et.reserve(h.size() * 2));
    GFE_CUDA_TRY(cudaMemcpy(et.ptr, h.data(), h.size() * 2, cudaMemcpyHostToDevice));
    ctx->q2tab_valid = true;
  }
  Xi xi;
  {
    std::vector<double> x1, w1;
    GFE_TRY(tensor_quadrature(1, 4, x1, w1));
    if (x1.size() != 3) return set_error(GFE_ERR_UNSUPPORTED, "q2 tensor cores: 1-D rule");
    for (int q = 0; q < 3; ++q) xi.x[q] = (float)x1[q];
  }
  const int64_t ntiles = (ncells + kCells - 1) / kCells;
  if (ntiles < 1) return GFE_OK;
  // the metric tiles (FP16 operand layout) and per-cell scales, 16-byte aligned
  DevBuf& mb = ctx->scratch[SCR_TMP2];
  const size_t gs_bytes = (size_t)ntiles * kBBytes;
  GFE_TRY(mb.reserve(gs_bytes + (size_t)ntiles * kCells * sizeof(float)));
  uint8_t* gs = mb.as<uint8_t>();
  float* scl = reinterpret_cast<float*>(gs + gs_bytes);
  k_q2_metric<<<(unsigned)ntiles, kMetricThreads, 0, ctx->stream>>>(
      ncells, cell_vertices, coords, tabs, xi, coef_kind, coef, src_kind, src, gs, scl, bvec,
      ctx->d_err);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  const size_t sm = q2_tc_smem_bytes();
  auto kern = k_q2_cells_tc;
  GFE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  int64_t npairs = ctx->num_sms / 2;
  if (npairs > ntiles) npairs = ntiles;
  if (npairs < 1) npairs = 1;
  kern<<<(unsigned)(2 * npairs), kThreads, sm, ctx->stream>>>(ncells, et.as<uint8_t>(), gs, scl,
                                                              K, ctx->d_err);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

}  // namespace gfe
