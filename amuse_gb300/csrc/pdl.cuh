// Programmatic dependent launch for the kernels of one force/step chain.
//
// A kernel launched with launch_pdl may be scheduled while the kernel before
// it in the stream is still running; it starts with pdl_wait()
// (griddepcontrol.wait), which returns once that kernel has completed and
// its memory is visible, so nothing is read early.  What overlaps is the
// launch and CTA scheduling latency of the dependent with the tail of its
// predecessor.  A kernel allows its dependent to be scheduled with
// pdl_trigger() (griddepcontrol.launch_dependents), which takes effect when
// every CTA has issued it or exited.  Both instructions are no-ops for a
// kernel launched without the attribute.
#pragma once
#include <cuda_runtime.h>

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
static inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                     cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}
