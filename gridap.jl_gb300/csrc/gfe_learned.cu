// gfe_learned.cu -- learned block preconditioner for flexible CG.
//
// The mesh's cells are grouped in 2x2x2 blocks; block b owns the 27 nodes (3x3x3) of its
// cells, neighbouring blocks share the nodes on their common faces. A per-block MLP acts on
// the block's residual patch:
//     x_b  = [ r(block nodes) / s_b  (27),  log kappa(block cells) - mean (8),  0 (13) ]
//     y_b  = W3 relu(W2 relu(W1 x_b + b1) + b2) + b3          (27 outputs)
//     z    = sum_b chi * P_b^T ( s_b / (kappa_b h) * y_b ),    chi = 1 / (#blocks at the node)
// with s_b the RMS of the patch and kappa_b the geometric mean of the block's kappa. The
// scaling makes the map positively homogeneous in r and independent of the mesh size; the
// network is trained to return the block's local solve A_b^{-1} r_b (A restricted to the
// block's free dofs), computed in FP64 on residuals produced by the method's own FP64 CG
// solves. Because z depends non-linearly on r the outer solver is flexible CG.
//
// Inference runs on the tensor cores: a tile of 128 blocks is one M=128 MMA chain
// (tcgen05, kind::f16 with BF16 operands, FP32 accumulators in tensor memory):
//   layer 1: A1 (128 x 48) x W1^T (64 x 48) -> D1 (TMEM columns 0..63)
//   layer 2: relu(D1 + b1) -> A2 (128 x 64, BF16, shared) x W2^T -> D2 (columns 64..127)
//   layer 3: relu(D2 + b2) -> A3 x W3^T (32 x 64) -> D3 (columns 128..159), + b3, scaled.
// Operands use the no-swizzle K-major canonical layout (8-row x 16-byte core matrices).
// Training uses plain FP32 kernels (small GEMMs, backward pass, Adam).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "gfe_internal.h"

namespace gfe {
namespace learned {

constexpr int kP = 27;       // nodes per block
constexpr int kF = 8;        // kappa features per block
constexpr int kIn = 48;      // padded input width (35 used)
constexpr int kH = 64;       // hidden width
constexpr int kOut = 32;     // padded output width (27 used)
constexpr int kTile = 128;   // blocks per MMA tile
constexpr int kThreads = 128;
constexpr unsigned long long kWaitLimitNs = 1000000000ull;

// packed FP32 parameters: W1[kIn][kH] | b1[kH] | W2[kH][kH] | b2[kH] | W3[kH][kOut] | b3[kOut]
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kIn * kH;
constexpr int kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH;
constexpr int kOffW3 = kOffB2 + kH;
constexpr int kOffB3 = kOffW3 + kH * kOut;
constexpr int kNParams = kOffB3 + kOut;

}  // namespace learned
}  // namespace gfe

struct gfe_learned_pc {
  gfe_ctx* ctx = nullptr;
  int64_t nblocks = 0, ndofs = 0;
  double h = 1.0;
  gfe::DevBuf bdofs;    // int32 [nblocks][27] (0-based free dof or -1)
  gfe::DevBuf bfeat;    // float [nblocks][8]
  gfe::DevBuf bscale;   // float [nblocks]: 1 / (kappa_b h)
  gfe::DevBuf dptr;     // int64 [ndofs+1]
  gfe::DevBuf dref;     // int32: b*27 + slot, sorted
  gfe::DevBuf params;   // float [kNParams] (FP32 master copy)
  gfe::DevBuf wpack;    // bf16 weights in the MMA operand layout (W1t | W2t | W3t)
  gfe::DevBuf yblk;     // float [nblocks][27] block outputs
  bool has_weights = false;
};

namespace gfe {
namespace learned {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// BF16 canonical K-major, no swizzle: core matrix 8 rows x 16 B (8 bf16 along K)
__device__ __host__ __forceinline__ int canon_bf16(int row, int k, int kdim) {
  return (row & 7) * 16 + (row >> 3) * (kdim / 8) * 128 + (k >> 3) * 128 + (k & 7) * 2;
}
__device__ __forceinline__ uint64_t desc(uint32_t addr, int kdim) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((128 >> 4) & 0x3FFF) << 16;                  // K-adjacent core matrices
  d |= (uint64_t)((((kdim / 8) * 128) >> 4) & 0x3FFF) << 32;   // next 8-row group
  d |= (uint64_t)1 << 46;
  return d;
}
// kind::f16 descriptor: D F32, A = B = BF16, K-major, N, M = 128
__device__ __forceinline__ uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((128u >> 4) << 24);
}
__device__ __forceinline__ unsigned long long gtime() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool wait_bar(uint32_t bar, uint32_t phase) {
  const unsigned long long t0 = gtime();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
    if (gtime() - t0 > kWaitLimitNs) return false;
  }
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t id,
                                         uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(ad), "l"(bd), "r"(id), "r"(acc));
}
__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   bar)
               : "memory");
}
// 32 consecutive TMEM columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
      "%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// byte sizes of the operand tiles
constexpr int kA1Bytes = kTile * kIn * 2;     // 12 KB
constexpr int kA2Bytes = kTile * kH * 2;      // 16 KB
constexpr int kW1Bytes = kH * kIn * 2;        // 6 KB
constexpr int kW2Bytes = kH * kH * 2;         // 8 KB
constexpr int kW3Bytes = kOut * kH * 2;       // 4 KB
constexpr int kWBytes = kW1Bytes + kW2Bytes + kW3Bytes;

struct __align__(16) Smem {
  uint8_t a1[kA1Bytes];
  uint8_t a2[kA2Bytes];
  uint8_t w[kWBytes];
  float b1[kH], b2[kH], b3[kOut];
  float s[kTile];       // patch RMS
  uint64_t mbar;
  uint32_t tmem_base;
  int error;
};

// Block outputs y (scaled) for every block: yblk[b][27].
__global__ void __launch_bounds__(kThreads, 1)
    k_mlp_blocks(int64_t nblocks, const int32_t* __restrict__ bdofs,
                 const float* __restrict__ bfeat, const float* __restrict__ bscale,
                 const float* __restrict__ r, const uint8_t* __restrict__ wpack,
                 const float* __restrict__ params, float* __restrict__ yblk, DevError* err,
                 const int* skip) {
  if (skip && *skip) return;
  extern __shared__ __align__(1024) uint8_t raw[];
  Smem& s = *reinterpret_cast<Smem*>(raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < kWBytes / 16; i += kThreads)
    reinterpret_cast<uint4*>(s.w)[i] = reinterpret_cast<const uint4*>(wpack)[i];
  for (int i = tid; i < kH; i += kThreads) {
    s.b1[i] = params[kOffB1 + i];
    s.b2[i] = params[kOffB2 + i];
  }
  for (int i = tid; i < kOut; i += kThreads) s.b3[i] = params[kOffB3 + i];
  if (tid == 0) {
    s.error = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s.mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&s.tmem_base)),
                 "r"(256));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s.tmem_base, bar = smem_u32(&s.mbar);
  const uint32_t a1 = smem_u32(s.a1), a2 = smem_u32(s.a2);
  const uint32_t w1 = smem_u32(s.w), w2 = w1 + kW1Bytes, w3 = w2 + kW2Bytes;
  const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
  uint32_t phase = 0;
  const int64_t ntiles = (nblocks + kTile - 1) / kTile;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    // 1. inputs: row m = block tile*128+m
    const int m = tid;
    const int64_t b = tile * kTile + m;
    {
      float v[kP];
      float ss = 0.f;
      if (b < nblocks) {
#pragma unroll
        for (int j = 0; j < kP; ++j) {
          const int32_t d = __ldg(bdofs + b * kP + j);
          v[j] = d >= 0 ? __ldg(r + d) : 0.f;
          ss += v[j] * v[j];
        }
      } else {
#pragma unroll
        for (int j = 0; j < kP; ++j) v[j] = 0.f;
      }
      const float sc = sqrtf(ss / kP);
      s.s[m] = sc;
      const float inv = sc > 0.f ? 1.f / sc : 0.f;
      for (int k = 0; k < kIn; ++k) {
        float xk = 0.f;
        if (k < kP) xk = v[k] * inv;
        else if (k < kP + kF && b < nblocks) xk = __ldg(bfeat + b * kF + (k - kP));
        *reinterpret_cast<__nv_bfloat16*>(s.a1 + canon_bf16(m, k, kIn)) = __float2bfloat16(xk);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    bool ok = true;
    // 2. layer 1
    if (tid == 0) {
      for (int ks = 0; ks < kIn / 16; ++ks)
        mma_bf16(tmem, desc(a1 + ks * 256, kIn), desc(w1 + ks * 256, kIn), idesc_bf16(kH),
                 ks > 0);
      commit(bar);
    }
    ok = wait_bar(bar, phase) && ok;
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
    // relu(D1 + b1) -> A2 (BF16)
    for (int c0 = 0; c0 < kH; c0 += 32) {
      float v[32];
      tmem_ld32(tmem + lane_off + c0, v);
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const float hval = fmaxf(v[i] + s.b1[c0 + i], 0.f);
        *reinterpret_cast<__nv_bfloat16*>(s.a2 + canon_bf16(m, c0 + i, kH)) =
            __float2bfloat16(hval);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    // 3. layer 2 -> columns 64..127
    if (tid == 0) {
      for (int ks = 0; ks < kH / 16; ++ks)
        mma_bf16(tmem + 64, desc(a2 + ks * 256, kH), desc(w2 + ks * 256, kH), idesc_bf16(kH),
                 ks > 0);
      commit(bar);
    }
    ok = wait_bar(bar, phase) && ok;
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
    // relu(D2 + b2) -> A2 again (layer 2's operand reads finished with the commit)
    for (int c0 = 0; c0 < kH; c0 += 32) {
      float v[32];
      tmem_ld32(tmem + lane_off + 64 + c0, v);
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const float hval = fmaxf(v[i] + s.b2[c0 + i], 0.f);
        *reinterpret_cast<__nv_bfloat16*>(s.a2 + canon_bf16(m, c0 + i, kH)) =
            __float2bfloat16(hval);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    // 4. layer 3 -> columns 128..159
    if (tid == 0) {
      for (int ks = 0; ks < kH / 16; ++ks)
        mma_bf16(tmem + 128, desc(a2 + ks * 256, kH), desc(w3 + ks * 256, kH),
                 idesc_bf16(kOut), ks > 0);
      commit(bar);
    }
    ok = wait_bar(bar, phase) && ok;
    phase ^= 1u;
    if (!ok && lane == 0) atomicExch(&s.error, 1);
    __syncthreads();
    if (s.error) break;
    asm volatile("tcgen05.fence::after_thread_sync;");
    {
      float v[32];
      tmem_ld32(tmem + lane_off + 128, v);
      if (b < nblocks) {
        const float scale = s.s[m] * __ldg(bscale + b);
#pragma unroll
        for (int i = 0; i < kP; ++i) yblk[b * kP + i] = (v[i] + s.b3[i]) * scale;
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256));
  if (tid == 0 && s.error)
    if (atomicCAS(&err->code, 0, GFE_ERR_TIMEOUT) == 0) err->index = blockIdx.x;
}

// z[d] = base[d] + (1 / count) * sum of the block outputs at d, in block order (base may be
// null: 0).
__global__ void k_block_gather(int64_t n, const int64_t* __restrict__ dptr,
                               const int32_t* __restrict__ dref, const float* __restrict__ yblk,
                               const float* base, float* z, const int* skip) {
  if (skip && *skip) return;
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < n;
       d += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = dptr[d], e = dptr[d + 1];
    float acc = 0.f;
    for (int64_t k = a; k < e; ++k) acc += __ldg(yblk + dref[k]);
    const float v = e > a ? acc / (float)(e - a) : 0.f;
    z[d] = base ? base[d] + v : v;
  }
}

// Training samples from a residual / error pair (r, e = x* - x, both FP64, host or device) of
// the method's own FP64 iterations: the network input as in k_samples, the target the error
// patch e_b in the network's units (e_b / (s_b * bscale_b), s_b the RMS of the r patch).
__global__ void k_samples_error(int64_t nsamples, const int64_t* __restrict__ ids,
                                const int32_t* __restrict__ bdofs, const float* __restrict__ bfeat,
                                const float* __restrict__ bscale, const double* __restrict__ r,
                                const double* __restrict__ e, float* __restrict__ X,
                                float* __restrict__ T) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t sidx = (int64_t)blockIdx.x * 4 + w;
  if (sidx >= nsamples) return;
  const int64_t b = ids[sidx];
  const int32_t d = lane < kP ? bdofs[b * kP + lane] : -1;
  const double rb = d >= 0 ? r[d] : 0.0, eb = d >= 0 ? e[d] : 0.0;
  double ss = rb * rb;
  for (int off = 16; off > 0; off >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, off);
  const double sc = sqrt(ss / kP);
  const double inv = sc > 0.0 ? 1.0 / sc : 0.0;
  for (int k = lane; k < kIn; k += 32) {
    float xk = 0.f;
    if (k < kP) xk = (float)(__shfl_sync(0xffffffffu, rb, k) * inv);
    else if (k < kP + kF) xk = bfeat[b * kF + (k - kP)];
    X[sidx * kIn + k] = xk;
  }
  const double tscale = (sc > 0.0) ? 1.0 / (sc * (double)bscale[b]) : 0.0;
  if (lane < kOut) T[sidx * kOut + lane] = lane < kP ? (float)(eb * tscale) : 0.f;
}

// ---- training samples ------------------------------------------------------------------------
// One warp per sample: A_b (free dofs of the block) gathered from the CSR, FP64 Cholesky,
// y = A_b^{-1} r_b; inputs x_b and targets y_b / (s_b * bscale_b).
__global__ void k_samples(int64_t nsamples, const int64_t* __restrict__ ids,
                          const int32_t* __restrict__ bdofs, const float* __restrict__ bfeat,
                          const float* __restrict__ bscale, const int32_t* __restrict__ rowptr,
                          const int32_t* __restrict__ colval, const double* __restrict__ val,
                          const double* __restrict__ r, float* __restrict__ X,
                          float* __restrict__ T) {
  __shared__ double L[4][kP * kP];
  __shared__ double y[4][kP];
  __shared__ int32_t dof[4][kP];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t sidx = (int64_t)blockIdx.x * 4 + w;
  if (sidx >= nsamples) return;
  const int64_t b = ids[sidx];
  if (lane < kP) dof[w][lane] = bdofs[b * kP + lane];
  __syncwarp();
  double* Lw = L[w];
  // dense block matrix (identity rows/cols for absent dofs)
  for (int e = lane; e < kP * kP; e += 32) {
    const int i = e / kP, j = e % kP;
    const int32_t di = dof[w][i], dj = dof[w][j];
    double v = 0.0;
    if (di < 0 || dj < 0) {
      v = (i == j) ? 1.0 : 0.0;
    } else {
      int lo = rowptr[di], hi = rowptr[di + 1];
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (colval[mid] < dj) lo = mid + 1; else hi = mid;
      }
      if (lo < rowptr[di + 1] && colval[lo] == dj) v = val[lo];
    }
    Lw[i * kP + j] = v;
  }
  if (lane < kP) y[w][lane] = dof[w][lane] >= 0 ? r[dof[w][lane]] : 0.0;
  __syncwarp();
  // Cholesky (lower), column by column
  for (int k = 0; k < kP; ++k) {
    if (lane == 0) {
      double d = Lw[k * kP + k];
      for (int t = 0; t < k; ++t) d -= Lw[k * kP + t] * Lw[k * kP + t];
      Lw[k * kP + k] = sqrt(d > 0.0 ? d : 1e-300);
    }
    __syncwarp();
    for (int i = k + 1 + lane; i < kP; i += 32) {
      double s = Lw[i * kP + k];
      for (int t = 0; t < k; ++t) s -= Lw[i * kP + t] * Lw[k * kP + t];
      Lw[i * kP + k] = s / Lw[k * kP + k];
    }
    __syncwarp();
  }
  if (lane == 0) {  // forward and backward substitution
    double* yy = y[w];
    for (int i = 0; i < kP; ++i) {
      double s = yy[i];
      for (int t = 0; t < i; ++t) s -= Lw[i * kP + t] * yy[t];
      yy[i] = s / Lw[i * kP + i];
    }
    for (int i = kP - 1; i >= 0; --i) {
      double s = yy[i];
      for (int t = i + 1; t < kP; ++t) s -= Lw[t * kP + i] * yy[t];
      yy[i] = s / Lw[i * kP + i];
    }
  }
  __syncwarp();
  // patch RMS
  double rb = (lane < kP && dof[w][lane] >= 0) ? r[dof[w][lane]] : 0.0;
  double ss = rb * rb;
  for (int off = 16; off > 0; off >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, off);
  const double sc = sqrt(ss / kP);
  const double inv = sc > 0.0 ? 1.0 / sc : 0.0;
  for (int k = lane; k < kIn; k += 32) {
    float xk = 0.f;
    if (k < kP) xk = (float)((dof[w][k] >= 0 ? r[dof[w][k]] : 0.0) * inv);
    else if (k < kP + kF) xk = bfeat[b * kF + (k - kP)];
    X[sidx * kIn + k] = xk;
  }
  const double tscale = (sc > 0.0) ? 1.0 / (sc * (double)bscale[b]) : 0.0;
  for (int k = lane; k < kOut; k += 32)
    T[sidx * kOut + k] = k < kP ? (float)(y[w][k] * tscale) : 0.f;
}

// ---- training (FP32) ------------------------------------------------------------------------
// C[M][N] = beta*C + op(A)[M][K] op(B)[K][N]; ta/tb select transposes of row-major A/B.
__global__ void k_gemm(int M, int N, int K, const float* __restrict__ A, int lda, bool ta,
                       const float* __restrict__ B, int ldb, bool tb, float* __restrict__ C,
                       int ldc, float beta) {
  __shared__ float As[16][17], Bs[16][17];
  const int row = blockIdx.y * 16 + threadIdx.y, col = blockIdx.x * 16 + threadIdx.x;
  float acc = 0.f;
  for (int k0 = 0; k0 < K; k0 += 16) {
    const int ka = k0 + threadIdx.x, kb = k0 + threadIdx.y;
    As[threadIdx.y][threadIdx.x] =
        (row < M && ka < K) ? (ta ? A[(int64_t)ka * lda + row] : A[(int64_t)row * lda + ka]) : 0.f;
    Bs[threadIdx.y][threadIdx.x] =
        (kb < K && col < N) ? (tb ? B[(int64_t)col * ldb + kb] : B[(int64_t)kb * ldb + col]) : 0.f;
    __syncthreads();
#pragma unroll
    for (int t = 0; t < 16; ++t) acc = fmaf(As[threadIdx.y][t], Bs[t][threadIdx.x], acc);
    __syncthreads();
  }
  if (row < M && col < N) {
    float* c = C + (int64_t)row * ldc + col;
    *c = beta == 0.f ? acc : beta * (*c) + acc;
  }
}

// H = act(H + bias) rowwise (act: 0 none, 1 relu)
__global__ void k_bias_act(int M, int N, float* __restrict__ H, const float* __restrict__ bias,
                           int act) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)M * N) return;
  float v = H[i] + bias[i % N];
  if (act) v = fmaxf(v, 0.f);
  H[i] = v;
}

// dY = 2 (Y - T) / (M * 27) on the 27 live outputs; loss partial
__global__ void k_loss_grad(int M, const float* __restrict__ Y, const float* __restrict__ T,
                            float* __restrict__ dY, float* __restrict__ loss) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)M * kOut) return;
  const int c = (int)(i % kOut);
  float g = 0.f;
  if (c < kP) {
    const float d = Y[i] - T[i];
    g = 2.f * d / (float)((int64_t)M * kP);
    atomicAdd(loss, d * d / (float)((int64_t)M * kP));
  }
  dY[i] = g;
}

// dH *= (H > 0)
__global__ void k_relu_back(int64_t n, float* __restrict__ dH, const float* __restrict__ H) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !(H[i] > 0.f)) dH[i] = 0.f;
}

// column sums: g[j] = sum_i D[i][j]
__global__ void k_colsum(int M, int N, const float* __restrict__ D, float* __restrict__ g) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  float s = 0.f;
  for (int i = 0; i < M; ++i) s += D[(int64_t)i * N + j];
  g[j] = s;
}

__global__ void k_adam(int n, float* __restrict__ w, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2,
                       float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  m[i] = b1 * m[i] + (1.f - b1) * gi;
  v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
  w[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + 1e-8f);
}

// FP32 parameters -> BF16 operand tiles (B operands: rows = output features, K = inputs)
__global__ void k_pack_weights(const float* __restrict__ p, uint8_t* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < kH * kIn) {  // W1t[n][k] = W1[k][n]
    const int n = t / kIn, k = t % kIn;
    *reinterpret_cast<__nv_bfloat16*>(out + canon_bf16(n, k, kIn)) =
        __float2bfloat16(p[kOffW1 + k * kH + n]);
  }
  if (t < kH * kH) {
    const int n = t / kH, k = t % kH;
    *reinterpret_cast<__nv_bfloat16*>(out + kW1Bytes + canon_bf16(n, k, kH)) =
        __float2bfloat16(p[kOffW2 + k * kH + n]);
  }
  if (t < kOut * kH) {
    const int n = t / kH, k = t % kH;
    *reinterpret_cast<__nv_bfloat16*>(out + kW1Bytes + kW2Bytes + canon_bf16(n, k, kH)) =
        __float2bfloat16(p[kOffW3 + k * kOut + n]);
  }
}

}  // namespace learned

// ---- host --------------------------------------------------------------------------------
using namespace learned;

int64_t learned_ndofs(const gfe_learned_pc* pc) { return pc->ndofs; }

int learned_apply(gfe_ctx* ctx, gfe_learned_pc* pc, const float* d_r, float* d_z,
                  const int* skip) {
  return learned_apply_into(ctx, pc, d_r, nullptr, d_z, skip, true);
}

int learned_apply_into(gfe_ctx* ctx, gfe_learned_pc* pc, const float* d_r, const float* base,
                       float* d_z, const int* skip, bool timed) {
  if (!pc->has_weights) return set_error(GFE_ERR_INVALID_ARGUMENT, "learned pc: no weights");
  const size_t sm = sizeof(Smem) + 1024;
  auto kern = k_mlp_blocks;
  GFE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  const int64_t ntiles = (pc->nblocks + kTile - 1) / kTile;
  const int64_t grid = ntiles < (int64_t)ctx->num_sms ? ntiles : (int64_t)ctx->num_sms;
  if (timed) timer_begin(ctx, GFE_KT_PRECOND);
  kern<<<(unsigned)(grid > 0 ? grid : 1), kThreads, sm, ctx->stream>>>(
      pc->nblocks, pc->bdofs.as<int32_t>(), pc->bfeat.as<float>(), pc->bscale.as<float>(), d_r,
      pc->wpack.as<uint8_t>(), pc->params.as<float>(), pc->yblk.as<float>(), ctx->d_err, skip);
  k_block_gather<<<grid_for(pc->ndofs, 256, (int64_t)ctx->num_sms * 8), 256, 0, ctx->stream>>>(
      pc->ndofs, pc->dptr.as<int64_t>(), pc->dref.as<int32_t>(), pc->yblk.as<float>(), base,
      d_z, skip);
  if (timed) timer_end(ctx);
  ctx->launches += 2;
  GFE_CUDA_TRY(cudaGetLastError());
  return GFE_OK;
}

int learned_pack(gfe_ctx* ctx, gfe_learned_pc* pc) {
  GFE_TRY(pc->wpack.reserve(kWBytes));
  GFE_CUDA_TRY(cudaMemsetAsync(pc->wpack.ptr, 0, kWBytes, ctx->stream));
  k_pack_weights<<<grid_for(kH * kH, 256), 256, 0, ctx->stream>>>(pc->params.as<float>(),
                                                                  pc->wpack.as<uint8_t>());
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  pc->has_weights = true;
  return GFE_OK;
}

}  // namespace gfe

using namespace gfe;

extern "C" int gfe_learned_pc_create(gfe_ctx* ctx, const int64_t* partition,
                                     const double* domain, const int32_t* node_to_dof,
                                     int64_t nfree, const double* kappa_cell,
                                     gfe_learned_pc** out) {
  clear_error();
  if (!ctx || !partition || !domain || !node_to_dof || !kappa_cell || !out || nfree < 0)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_learned_pc_create: bad arguments");
  const int64_t nx = partition[0], ny = partition[1], nz = partition[2];
  if (nx < 2 || ny < 2 || nz < 2)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_learned_pc_create: partition < 2");
  const int64_t bx = (nx + 1) / 2, by = (ny + 1) / 2, bz = (nz + 1) / 2;
  const int64_t nb = bx * by * bz;
  const int64_t npx = nx + 1, npy = ny + 1;
  std::vector<int32_t> bd((size_t)nb * kP, -1);
  std::vector<float> bf((size_t)nb * kF, 0.f), bs(nb, 1.f);
  const double h = (domain[1] - domain[0]) / (double)nx;
  std::vector<int32_t> cnt(nfree, 0);
  for (int64_t b = 0; b < nb; ++b) {
    const int64_t i0 = 2 * (b % bx), j0 = 2 * ((b / bx) % by), k0 = 2 * (b / (bx * by));
    for (int s = 0; s < kP; ++s) {
      const int64_t i = i0 + s % 3, j = j0 + (s / 3) % 3, k = k0 + s / 9;
      if (i > nx || j > ny || k > nz) continue;
      const int32_t d = node_to_dof[i + npx * (j + npy * k)];
      if (d > 0) {
        bd[b * kP + s] = d - 1;
        cnt[d - 1] += 1;
      }
    }
    double lk[kF], mean = 0.0;
    int nl = 0;
    for (int c = 0; c < kF; ++c) {
      int64_t i = i0 + (c & 1), j = j0 + ((c >> 1) & 1), k = k0 + (c >> 2);
      i = i < nx ? i : nx - 1;
      j = j < ny ? j : ny - 1;
      k = k < nz ? k : nz - 1;
      lk[c] = std::log(kappa_cell[i + nx * (j + ny * k)]);
      mean += lk[c];
      ++nl;
    }
    mean /= nl;
    for (int c = 0; c < kF; ++c) bf[b * kF + c] = (float)(lk[c] - mean);
    bs[b] = (float)(1.0 / (std::exp(mean) * h));
  }
  // dof -> (block, slot) references in block order
  std::vector<int64_t> dp(nfree + 1, 0);
  for (int64_t d = 0; d < nfree; ++d) dp[d + 1] = dp[d] + cnt[d];
  std::vector<int32_t> dr(dp[nfree] > 0 ? dp[nfree] : 1);
  std::vector<int64_t> fill(dp.begin(), dp.end() - 1);
  for (int64_t b = 0; b < nb; ++b)
    for (int s = 0; s < kP; ++s) {
      const int32_t d = bd[b * kP + s];
      if (d >= 0) dr[fill[d]++] = (int32_t)(b * kP + s);
    }
  gfe_learned_pc* pc = new gfe_learned_pc();
  pc->ctx = ctx;
  pc->nblocks = nb;
  pc->ndofs = nfree;
  pc->h = h;
  for (DevBuf* d : {&pc->bdofs, &pc->bfeat, &pc->bscale, &pc->dptr, &pc->dref, &pc->params,
                    &pc->wpack, &pc->yblk})
    d->owner = ctx;
  int st = GFE_OK;
  auto up = [&](DevBuf& buf, const void* src, size_t n) {
    if (st != GFE_OK) return;
    st = buf.reserve(n);
    if (st == GFE_OK && cudaMemcpyAsync(buf.ptr, src, n, cudaMemcpyHostToDevice, ctx->stream) !=
                            cudaSuccess)
      st = set_error(GFE_ERR_CUDA, "gfe_learned_pc_create: copy failed");
  };
  up(pc->bdofs, bd.data(), bd.size() * sizeof(int32_t));
  up(pc->bfeat, bf.data(), bf.size() * sizeof(float));
  up(pc->bscale, bs.data(), bs.size() * sizeof(float));
  up(pc->dptr, dp.data(), dp.size() * sizeof(int64_t));
  up(pc->dref, dr.data(), dr.size() * sizeof(int32_t));
  if (st == GFE_OK) st = pc->yblk.reserve((size_t)nb * kP * sizeof(float));
  if (st == GFE_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    st = set_error(GFE_ERR_CUDA, "gfe_learned_pc_create: sync failed");
  if (st != GFE_OK) {
    delete pc;
    return st;
  }
  *out = pc;
  return GFE_OK;
}

extern "C" int gfe_learned_pc_destroy(gfe_learned_pc* pc) {
  delete pc;
  return GFE_OK;
}

extern "C" int gfe_learned_pc_set_weights(gfe_learned_pc* pc, const float* params) {
  clear_error();
  if (!pc || !params) return set_error(GFE_ERR_INVALID_ARGUMENT, "set_weights: NULL");
  GFE_TRY(pc->params.reserve(sizeof(float) * kNParams));
  GFE_CUDA_TRY(cudaMemcpyAsync(pc->params.ptr, params, sizeof(float) * kNParams,
                               cudaMemcpyDefault, pc->ctx->stream));
  return learned_pack(pc->ctx, pc);
}

extern "C" int gfe_learned_pc_get_weights(gfe_learned_pc* pc, float* params) {
  clear_error();
  if (!pc || !params || !pc->has_weights)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "get_weights: no weights");
  return copy_out(pc->ctx, params, pc->params.ptr, sizeof(float) * kNParams);
}

extern "C" int gfe_learned_pc_num_params(void) { return kNParams; }

extern "C" int gfe_learned_pc_apply(gfe_learned_pc* pc, const float* r, float* z) {
  gfe::NvtxRange nvtx_range("gfe_learned_pc_apply");
  clear_error();
  if (!pc || !r || !z || !is_device_ptr(r) || !is_device_ptr(z))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_learned_pc_apply: device vectors needed");
  GFE_TRY(learned_apply(pc->ctx, pc, r, z));
  return check_device_error(pc->ctx, "gfe_learned_pc_apply");
}

extern "C" int gfe_solve_fcg(gfe_ctx* ctx, gfe_matrix* A, gfe_learned_pc* pc,
                             const gfe_solver_opts* opts, const double* b, double* x,
                             gfe_solve_report* report) {
  gfe::NvtxRange nvtx_range("gfe_solve_fcg");
  clear_error();
  if (!ctx || !A || !opts || !b || !x || A->ctx != ctx || (pc && pc->ndofs != A->nrows))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_solve_fcg: bad arguments");
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
  ctx->err_staged = false;
  GFE_TRY(solve_fcg(ctx, A, pc, opts, (const double*)db, dx, &rep));
  if (!xdev) GFE_TRY(copy_out(ctx, x, dx, n8));
  if (report) *report = rep;
  // the error word came back with the solve's last wait (nothing ran after it)
  return opts->initial_guess ? check_device_error(ctx, "gfe_solve_fcg")
                             : check_staged_error(ctx, "gfe_solve_fcg");
}

extern "C" int gfe_learned_pc_samples(gfe_learned_pc* pc, gfe_matrix* A, const double* r,
                                      int64_t nsamples, const int64_t* block_ids, float* X,
                                      float* T) {
  clear_error();
  if (!pc || !A || !r || nsamples < 0 || !block_ids || !X || !T || A->nrows != pc->ndofs)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_learned_pc_samples: bad arguments");
  gfe_ctx* ctx = pc->ctx;
  if (nsamples == 0) return GFE_OK;
  GFE_TRY(ensure_values(ctx, A));
  const void *dr, *dids;
  GFE_TRY(device_view(ctx, r, sizeof(double) * pc->ndofs, SCR_TMP2, &dr));
  GFE_TRY(device_view(ctx, block_ids, sizeof(int64_t) * nsamples, SCR_TMP3, &dids));
  if (!is_device_ptr(X) || !is_device_ptr(T))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_learned_pc_samples: X, T device memory");
  k_samples<<<(unsigned)((nsamples + 3) / 4), 128, 0, ctx->stream>>>(
      nsamples, (const int64_t*)dids, pc->bdofs.as<int32_t>(), pc->bfeat.as<float>(),
      pc->bscale.as<float>(), A->rowptr.as<int32_t>(), A->colval.as<int32_t>(),
      A->val.as<double>(), (const double*)dr, X, T);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GFE_OK;
}

extern "C" int gfe_learned_pc_samples_error(gfe_learned_pc* pc, const double* r,
                                            const double* e, int64_t nsamples,
                                            const int64_t* block_ids, float* X, float* T) {
  clear_error();
  if (!pc || !r || !e || nsamples < 0 || !block_ids || !X || !T)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_learned_pc_samples_error: bad arguments");
  gfe_ctx* ctx = pc->ctx;
  if (nsamples == 0) return GFE_OK;
  const void *dr, *de, *dids;
  GFE_TRY(device_view(ctx, r, sizeof(double) * pc->ndofs, SCR_TMP2, &dr));
  GFE_TRY(device_view(ctx, e, sizeof(double) * pc->ndofs, SCR_TMP1, &de));
  GFE_TRY(device_view(ctx, block_ids, sizeof(int64_t) * nsamples, SCR_TMP3, &dids));
  if (!is_device_ptr(X) || !is_device_ptr(T))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_learned_pc_samples_error: X, T device memory");
  k_samples_error<<<(unsigned)((nsamples + 3) / 4), 128, 0, ctx->stream>>>(
      nsamples, (const int64_t*)dids, pc->bdofs.as<int32_t>(), pc->bfeat.as<float>(),
      pc->bscale.as<float>(), (const double*)dr, (const double*)de, X, T);
  ctx->launches++;
  GFE_CUDA_TRY(cudaGetLastError());
  GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GFE_OK;
}

// Trains the MLP on (X, T) (device arrays, n rows of 48 inputs / 32 targets) with Adam,
// minibatches taken in order, starting from the pc's current weights (or a scaled random
// init when it has none). Writes the mean loss of the last epoch to *loss.
extern "C" int gfe_learned_pc_train(gfe_learned_pc* pc, const float* X, const float* T,
                                    int64_t n, int32_t epochs, int32_t batch, float lr,
                                    uint64_t seed, float* loss) {
  gfe::NvtxRange nvtx_range("gfe_learned_pc_train");
  clear_error();
  if (!pc || !X || !T || n < 1 || epochs < 1 || batch < 1 || !is_device_ptr(X) ||
      !is_device_ptr(T))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_learned_pc_train: bad arguments");
  gfe_ctx* ctx = pc->ctx;
  if (!pc->has_weights) {
    // He-style init (deterministic LCG), zero biases
    std::vector<float> p(kNParams, 0.f);
    uint64_t s = seed * 6364136223846793005ull + 1442695040888963407ull;
    auto rnd = [&s]() {
      s = s * 6364136223846793005ull + 1442695040888963407ull;
      return ((s >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
    };
    for (int i = 0; i < kIn * kH; ++i) p[kOffW1 + i] = (float)(rnd() * std::sqrt(6.0 / 35.0));
    for (int i = 0; i < kH * kH; ++i) p[kOffW2 + i] = (float)(rnd() * std::sqrt(6.0 / kH));
    for (int i = 0; i < kH * kOut; ++i) p[kOffW3 + i] = (float)(rnd() * std::sqrt(3.0 / kH));
    GFE_TRY(pc->params.reserve(sizeof(float) * kNParams));
    GFE_CUDA_TRY(cudaMemcpyAsync(pc->params.ptr, p.data(), sizeof(float) * kNParams,
                                 cudaMemcpyHostToDevice, ctx->stream));
    GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  }
  const int B = batch;
  DevBuf work(ctx);
  const size_t nfl = (size_t)B * (kH * 4 + kOut * 2) + (size_t)kNParams * 3 + 64;
  GFE_TRY(work.reserve(sizeof(float) * nfl));
  float* H1 = work.as<float>();
  float* H2 = H1 + (size_t)B * kH;
  float* dH1 = H2 + (size_t)B * kH;
  float* dH2 = dH1 + (size_t)B * kH;
  float* Y = dH2 + (size_t)B * kH;
  float* dY = Y + (size_t)B * kOut;
  float* g = dY + (size_t)B * kOut;
  float* mom = g + kNParams;
  float* var = mom + kNParams;
  float* dloss = var + kNParams;
  GFE_CUDA_TRY(cudaMemsetAsync(mom, 0, sizeof(float) * (2 * kNParams + 64), ctx->stream));
  float* P = pc->params.as<float>();
  const dim3 tb(16, 16);
  auto gemm = [&](int M, int N, int K, const float* A, int lda, bool ta, const float* Bm,
                  int ldb, bool tbm, float* C, int ldc) {
    dim3 gr((N + 15) / 16, (M + 15) / 16);
    learned::k_gemm<<<gr, tb, 0, ctx->stream>>>(M, N, K, A, lda, ta, Bm, ldb, tbm, C, ldc, 0.f);
  };
  const float b1 = 0.9f, b2 = 0.999f;
  int64_t step = 0;
  float last = 0.f;
  for (int ep = 0; ep < epochs; ++ep) {
    GFE_CUDA_TRY(cudaMemsetAsync(dloss, 0, sizeof(float), ctx->stream));
    int64_t nb = 0;
    for (int64_t r0 = 0; r0 + B <= n; r0 += B, ++nb) {
      const float* Xb = X + r0 * kIn;
      const float* Tb = T + r0 * kOut;
      // forward
      gemm(B, kH, kIn, Xb, kIn, false, P + kOffW1, kH, false, H1, kH);
      learned::k_bias_act<<<grid_for((int64_t)B * kH, 256), 256, 0, ctx->stream>>>(
          B, kH, H1, P + kOffB1, 1);
      gemm(B, kH, kH, H1, kH, false, P + kOffW2, kH, false, H2, kH);
      learned::k_bias_act<<<grid_for((int64_t)B * kH, 256), 256, 0, ctx->stream>>>(
          B, kH, H2, P + kOffB2, 1);
      gemm(B, kOut, kH, H2, kH, false, P + kOffW3, kOut, false, Y, kOut);
      learned::k_bias_act<<<grid_for((int64_t)B * kOut, 256), 256, 0, ctx->stream>>>(
          B, kOut, Y, P + kOffB3, 0);
      learned::k_loss_grad<<<grid_for((int64_t)B * kOut, 256), 256, 0, ctx->stream>>>(
          B, Y, Tb, dY, dloss);
      // backward
      gemm(kH, kOut, B, H2, kH, true, dY, kOut, false, g + kOffW3, kOut);       // dW3
      learned::k_colsum<<<1, 64, 0, ctx->stream>>>(B, kOut, dY, g + kOffB3);     // db3
      gemm(B, kH, kOut, dY, kOut, false, P + kOffW3, kOut, true, dH2, kH);      // dH2
      learned::k_relu_back<<<grid_for((int64_t)B * kH, 256), 256, 0, ctx->stream>>>(
          (int64_t)B * kH, dH2, H2);
      gemm(kH, kH, B, H1, kH, true, dH2, kH, false, g + kOffW2, kH);            // dW2
      learned::k_colsum<<<1, 64, 0, ctx->stream>>>(B, kH, dH2, g + kOffB2);
      gemm(B, kH, kH, dH2, kH, false, P + kOffW2, kH, true, dH1, kH);           // dH1
      learned::k_relu_back<<<grid_for((int64_t)B * kH, 256), 256, 0, ctx->stream>>>(
          (int64_t)B * kH, dH1, H1);
      gemm(kIn, kH, B, Xb, kIn, true, dH1, kH, false, g + kOffW1, kH);          // dW1
      learned::k_colsum<<<1, 64, 0, ctx->stream>>>(B, kH, dH1, g + kOffB1);
      ++step;
      const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
      learned::k_adam<<<grid_for(kNParams, 256), 256, 0, ctx->stream>>>(kNParams, P, g, mom,
                                                                        var, lr, b1, b2, c1, c2);
      ctx->launches += 17;
    }
    float hl = 0.f;
    GFE_TRY(copy_out(ctx, &hl, dloss, sizeof(float)));
    last = nb > 0 ? hl / (float)nb : 0.f;
  }
  GFE_CUDA_TRY(cudaGetLastError());
  if (loss) *loss = last;
  return learned_pack(ctx, pc);
}
