// gfe_reduce.cuh -- deterministic block and grid reductions shared by the solver kernels
// (gfe_solve.cu) and the multigrid cycle (gfe_mg.cu): every block writes its partial sums, and
// the last block to finish adds them in block order. Included inside namespace gfe.
#pragma once

// Block sum of a double (all threads get the result in thread 0).
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < NT / 32; ++i) s += sh[i];
  __syncthreads();
  return s;
}

// Block sum of FP32 values: FP32 within each warp (shuffles), FP64 across the block's warps
// in warp order. Deterministic; avoids FP64 shuffles, which cost a full warp instruction on
// the FP64 pipe each.
template <int NT>
__device__ __forceinline__ double block_sum_f(float v, double* sh) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = (double)v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < NT / 32; ++i) s += sh[i];
  __syncthreads();
  return s;
}

// Linear block id and block count of 1-, 2- or 3-D grids.
__device__ __forceinline__ unsigned block_linear() {
  return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
}
__device__ __forceinline__ unsigned grid_blocks() {
  return gridDim.x * gridDim.y * gridDim.z;
}

// Called by every block after its thread 0 has written the block's partial(s). Returns true
// in the last block, with the partial sums of all blocks reduced in block order into
// out[0..nv). Only thread 0 fences before taking its ticket: the partials are its own writes,
// and a fence in every thread would wait for all of the block's outstanding stores.
template <int NT, int NV>
__device__ bool last_block_reduce(unsigned* ticket, const double* partials, int nblocks,
                                  double* out, double* sh) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    __threadfence();
    last = (atomicAdd(ticket, 1u) == (unsigned)nblocks - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  for (int v = 0; v < NV; ++v) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += NT) s += __ldcg(partials + (size_t)i * NV + v);
    s = block_sum<NT>(s, sh);
    if (threadIdx.x == 0) out[v] = s;
  }
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}
