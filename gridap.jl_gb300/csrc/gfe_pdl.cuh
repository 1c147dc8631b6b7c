// gfe_pdl.cuh -- programmatic dependent launch between consecutive kernels on a stream (or
// graph edges captured from one): a kernel launched with launch_pdl may become resident while
// the kernel before it still runs; it waits in pdl_wait(), before any memory access, until
// that kernel has completed and its writes are visible, and then lets the next kernel launch
// at once. Without the launch attribute both instructions return immediately. Included
// inside namespace gfe, after <utility> (std::forward).
#pragma once

__device__ __forceinline__ void pdl_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <class... P, class... A>
cudaError_t launch_pdl(void (*kern)(P...), dim3 grid, int block, size_t smem, cudaStream_t st,
                       A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}
