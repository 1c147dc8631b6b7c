// gfe_q2_tc.cu -- Q2 diffusion cell matrices on the 5th-generation tensor cores (tcgen05, TF32
// operands, FP32 accumulation in tensor memory).
//
// For a cell with (tri)linear geometry the Q2 stiffness is K = B^T C with
//   B[(q,k), i] = d phi_hat_i / d xi_k (xi_q)          (reference table, every cell),
//   C[(q,k), j] = sum_l G_q[k][l] B[(q,l), j],
//   G_q = kappa |det Jt_q| w_q invJt_q^T invJt_q         (FP64 Jacobian, inverse, determinant),
// Gridap's sum over quadrature points of (kappa invJt grad phi_i).(invJt grad phi_j)|det Jt| w
// (Fields/FieldsInterfaces.jl:708-720) regrouped as one dense contraction per cell.
//
// A tile of 4 cells is one MMA problem  D[(cell, j), i] = sum_{qk} C_cell[qk][j] B[qk][i]:
//   A (M=128 x K=88, K-major): rows (cell, j), 108 live rows; the per-cell C^T built by the
//     CTA's threads in shared memory (TF32-rounded);
//   B (N=32 x K=88, K-major): the reference gradients, loaded once per CTA;
//   D (128 lanes x 32 columns FP32) in tensor memory, read back with tcgen05.ld.
// Operands use the no-swizzle K-major canonical layout: 8-row x 16-byte core matrices, the
// K-direction core matrices of one 8-row group contiguous (LBO = 128 B), 8-row groups
// SBO = 22 * 128 B apart. 11 MMAs of K = 8 cover K = 88. One elected thread issues them and
// commits to an mbarrier; every wait on it is bounded and reports GFE_ERR_TIMEOUT.
//
// Output: FP32 cell matrices, cell-major, Gridap's column-major order K[cell][i + j*27],
// written through shared memory with coalesced stores; FP32 cell vectors b[cell][i].
#include <cstdint>

#include "gfe_internal.h"

namespace gfe {
namespace q2tc {

constexpr int kNN = 27;          // Q2 HEX nodes
constexpr int kNQ = 27;          // degree-4 tensor Gauss points
constexpr int kNV = 8;           // geometry vertices
constexpr int kCellsPerTile = 4;
constexpr int kM = 128, kN = 32, kK = 88;  // padded MMA shape
constexpr int kKChunks = kK / 4;           // 16-byte chunks along K
constexpr int kSBO = kKChunks * 128;       // bytes between 8-row groups
constexpr int kThreads = 128;
constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // 1 s; an MMA tile takes ~us

struct __align__(16) Smem {
  uint8_t A[kM / 8 * kSBO];  // 45,056 B
  uint8_t B[kN / 8 * kSBO];  // 11,264 B
  float G[kCellsPerTile][kNQ][6];   // symmetric 3x3 metric per (cell, q)
  float dv[kCellsPerTile][kNQ];     // |det Jt| w per (cell, q)
  float Bref[kNQ * 3][kNN];         // B[(q,k), i] in FP32 for building C
  float out[kCellsPerTile * kNN * kNN];
  double dphi1[kNQ * kNV * 3];
  double w[kNQ];
  float phi2[kNQ * kNN];
  uint64_t mbar;
  uint32_t tmem_base;
  int error;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (row, k) in the no-swizzle K-major canonical layout
__device__ __forceinline__ int canon_off(int row, int k) {
  return (row & 7) * 16 + (row >> 3) * kSBO + (k >> 2) * 128 + (k & 3) * 4;
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);          // start address
  d |= (uint64_t)((128 >> 4) & 0x3FFF) << 16;     // leading (K-direction) byte offset
  d |= (uint64_t)((kSBO >> 4) & 0x3FFF) << 32;    // stride (8-row group) byte offset
  d |= (uint64_t)1 << 46;                         // descriptor version for sm_100 family
  return d;                                       // base offset 0, no swizzle
}

// kind::tf32 instruction descriptor: D = F32, A = B = TF32, both K-major, N, M
__device__ __forceinline__ uint32_t idesc_tf32() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kN >> 3) << 17) |
         ((uint32_t)(kM >> 4) << 24);
}

__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
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

__global__ void __launch_bounds__(kThreads, 1)
    k_q2_cells_tf32(int64_t ncells, const int32_t* __restrict__ cell_vertices,
                    const double* __restrict__ coords, const double* __restrict__ tabs,
                    int coef_kind, const double* __restrict__ coef, int src_kind,
                    const double* __restrict__ src, float* __restrict__ K,
                    float* __restrict__ bvec, DevError* err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  Smem& s = *reinterpret_cast<Smem*>(smem_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // tables: w[27] | phi2[27*27] | dphi1[27*8*3] | B[(q*3+k)*27 + i]  (FP64, from the host)
  const double* t_w = tabs;
  const double* t_phi2 = t_w + kNQ;
  const double* t_dphi1 = t_phi2 + kNQ * kNN;
  const double* t_B = t_dphi1 + kNQ * kNV * 3;
  for (int i = tid; i < kNQ; i += kThreads) s.w[i] = t_w[i];
  for (int i = tid; i < kNQ * kNN; i += kThreads) s.phi2[i] = (float)t_phi2[i];
  for (int i = tid; i < kNQ * kNV * 3; i += kThreads) s.dphi1[i] = t_dphi1[i];
  for (int i = tid; i < kNQ * 3 * kNN; i += kThreads) (&s.Bref[0][0])[i] = (float)t_B[i];
  // B operand: rows i (N), K index qk; zero padding
  for (int idx = tid; idx < kN * kK; idx += kThreads) {
    const int i = idx / kK, kk = idx % kK;
    const float v = (i < kNN && kk < kNQ * 3) ? to_tf32((float)t_B[kk * kNN + i]) : 0.f;
    *reinterpret_cast<float*>(s.B + canon_off(i, kk)) = v;
  }
  // A operand padding (rows >= 108, columns >= 81) stays zero for the whole kernel
  for (int idx = tid; idx < kM * kK; idx += kThreads) {
    const int m = idx / kK, kk = idx % kK;
    if (m >= kCellsPerTile * kNN || kk >= kNQ * 3)
      *reinterpret_cast<float*>(s.A + canon_off(m, kk)) = 0.f;
  }
  if (tid == 0) {
    s.error = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s.mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&s.tmem_base)),
                 "r"(32));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s.tmem_base;
  const uint32_t a_addr = smem_u32(s.A), b_addr = smem_u32(s.B), bar = smem_u32(&s.mbar);
  uint32_t phase = 0;
  const int64_t ntiles = (ncells + kCellsPerTile - 1) / kCellsPerTile;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t cell0 = tile * kCellsPerTile;
    // 1. FP64 Jacobian, inverse, determinant per (cell, q) -> FP32 metric G
    for (int cq = tid; cq < kCellsPerTile * kNQ; cq += kThreads) {
      const int c = cq / kNQ, q = cq % kNQ;
      const int64_t cell = cell0 + c;
      float* g = s.G[c][q];
      if (cell >= ncells) {
        for (int t = 0; t < 6; ++t) g[t] = 0.f;
        s.dv[c][q] = 0.f;
        continue;
      }
      double Jt[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      for (int a = 0; a < kNV; ++a) {
        const double* x = coords + ((int64_t)__ldg(cell_vertices + cell * kNV + a) - 1) * 3;
        const double x0 = __ldg(x), x1 = __ldg(x + 1), x2 = __ldg(x + 2);
        for (int k = 0; k < 3; ++k) {
          const double gk = s.dphi1[(q * kNV + a) * 3 + k];
          Jt[k][0] += gk * x0;
          Jt[k][1] += gk * x1;
          Jt[k][2] += gk * x2;
        }
      }
      const double a11 = Jt[0][0], a12 = Jt[0][1], a13 = Jt[0][2];
      const double a21 = Jt[1][0], a22 = Jt[1][1], a23 = Jt[1][2];
      const double a31 = Jt[2][0], a32 = Jt[2][1], a33 = Jt[2][2];
      const double det = a11 * a22 * a33 + a12 * a23 * a31 + a13 * a21 * a32 -
                         (a11 * a23 * a32 + a12 * a21 * a33 + a13 * a22 * a31);
      if (!(det != 0.0) || !isfinite(det)) {
        if (atomicCAS(&err->code, 0, GFE_ERR_DEGENERATE_CELL) == 0) err->index = cell;
      }
      const double cinv = 1.0 / det;
      double iJ[3][3];
      iJ[0][0] = (a22 * a33 - a23 * a32) * cinv;
      iJ[1][0] = -(a21 * a33 - a23 * a31) * cinv;
      iJ[2][0] = (a21 * a32 - a22 * a31) * cinv;
      iJ[0][1] = -(a12 * a33 - a13 * a32) * cinv;
      iJ[1][1] = (a11 * a33 - a13 * a31) * cinv;
      iJ[2][1] = -(a11 * a32 - a12 * a31) * cinv;
      iJ[0][2] = (a12 * a23 - a13 * a22) * cinv;
      iJ[1][2] = -(a11 * a23 - a13 * a21) * cinv;
      iJ[2][2] = (a11 * a22 - a12 * a21) * cinv;
      const double kap = coef_kind == GFE_COEF_CELL ? __ldg(coef + cell)
                         : coef_kind == GFE_COEF_CONST ? __ldg(coef) : 1.0;
      const double dvq = fabs(det) * s.w[q];
      const double sc = kap * dvq;
      int t = 0;
      for (int k = 0; k < 3; ++k)
        for (int l = k; l < 3; ++l) {
          const double v = iJ[0][k] * iJ[0][l] + iJ[1][k] * iJ[1][l] + iJ[2][k] * iJ[2][l];
          g[t++] = (float)(sc * v);
        }
      s.dv[c][q] = (float)dvq;
    }
    __syncthreads();
    // 2. A rows (cell, j): C_cell[(q,k)][j] = sum_l G[k][l] B[(q,l)][j]  (TF32-rounded)
    if (tid < kCellsPerTile * kNN) {
      const int c = tid / kNN, j = tid % kNN;
      for (int q = 0; q < kNQ; ++q) {
        const float* g = s.G[c][q];  // g00 g01 g02 g11 g12 g22
        const float b0 = s.Bref[q * 3 + 0][j], b1 = s.Bref[q * 3 + 1][j],
                    b2 = s.Bref[q * 3 + 2][j];
        const float c0 = g[0] * b0 + g[1] * b1 + g[2] * b2;
        const float c1 = g[1] * b0 + g[3] * b1 + g[4] * b2;
        const float c2 = g[2] * b0 + g[4] * b1 + g[5] * b2;
        *reinterpret_cast<float*>(s.A + canon_off(tid, q * 3 + 0)) = to_tf32(c0);
        *reinterpret_cast<float*>(s.A + canon_off(tid, q * 3 + 1)) = to_tf32(c1);
        *reinterpret_cast<float*>(s.A + canon_off(tid, q * 3 + 2)) = to_tf32(c2);
      }
    }
    // cell vectors: b_i = sum_q f_q phi_i dV_q (FP32)
    if (bvec && src_kind != GFE_SRC_NONE) {
      for (int ci = tid; ci < kCellsPerTile * kNN; ci += kThreads) {
        const int c = ci / kNN, i = ci % kNN;
        const int64_t cell = cell0 + c;
        if (cell >= ncells) continue;
        float acc = 0.f;
        for (int q = 0; q < kNQ; ++q) {
          const float fq = src_kind == GFE_SRC_CONST ? (float)__ldg(src)
                                                     : (float)__ldg(src + cell * kNQ + q);
          acc += (fq * s.phi2[q * kNN + i]) * s.dv[c][q];
        }
        bvec[cell * kNN + i] = acc;
      }
    }
    // make the generic-proxy smem writes visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    // 3. one thread issues the 11 MMAs (K = 8 each) and commits to the mbarrier
    if (tid == 0) {
      const uint32_t idesc = idesc_tf32();
      for (int ks = 0; ks < kK / 8; ++ks) {
        const uint64_t ad = smem_desc(a_addr + ks * 256);
        const uint64_t bd = smem_desc(b_addr + ks * 256);
        const uint32_t acc = ks > 0 ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              bar)
          : "memory");
    }
    // 4. wait (bounded), read the accumulator rows of this warp's 32 lanes
    const bool ok = mbar_wait(bar, phase);
    phase ^= 1u;
    if (!ok && lane == 0) atomicExch(&s.error, 1);
    __syncthreads();
    if (s.error) break;  // the whole CTA stops; TMEM is released below
    asm volatile("tcgen05.fence::after_thread_sync;");
    uint32_t r[32];
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
        "%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    // row m = (cell c, j) holds K_c[i][j] for i = 0..26 -> out[c][i + 27 j]
    const int m = tid;
    if (m < kCellsPerTile * kNN) {
      const int c = m / kNN, j = m % kNN;
#pragma unroll
      for (int i = 0; i < kNN; ++i) s.out[c * kNN * kNN + i + kNN * j] = __uint_as_float(r[i]);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    // 5. coalesced store of the tile's cell matrices (cell-major, contiguous)
    const int64_t live = (ncells - cell0) < kCellsPerTile ? (ncells - cell0) : kCellsPerTile;
    const int64_t nout = live * kNN * kNN;
    float* dst = K + cell0 * kNN * kNN;
    for (int64_t e = tid; e < nout; e += kThreads) dst[e] = s.out[e];
    __syncthreads();
  }
  // release tensor memory (same warp that allocated)
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(32));
  if (tid == 0 && s.error)
    if (atomicCAS(&err->code, 0, GFE_ERR_TIMEOUT) == 0) err->index = blockIdx.x;
}

}  // namespace q2tc

size_t q2_tf32_smem_bytes() { return sizeof(q2tc::Smem) + 1024; }

int launch_q2_cells_tf32(gfe_ctx* ctx, int64_t ncells, const int32_t* cell_vertices,
                         const double* coords, const double* tabs, int coef_kind,
                         const double* coef, int src_kind, const double* src, float* K,
                         float* bvec) {
  const size_t sm = q2_tf32_smem_bytes();
  auto kern = q2tc::k_q2_cells_tf32;
  GFE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  const int64_t ntiles = (ncells + q2tc::kCellsPerTile - 1) / q2tc::kCellsPerTile;
  const int64_t grid = ntiles < (int64_t)ctx->num_sms * 2 ? ntiles : (int64_t)ctx->num_sms * 2;
  kern<<<(unsigned)(grid > 0 ? grid : 1), q2tc::kThreads, sm, ctx->stream>>>(
      ncells, cell_vertices, coords, tabs, coef_kind, coef, src_kind, src, K, bvec, ctx->d_err);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

}  // namespace gfe
