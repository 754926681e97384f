// salsa_k_f0.cu -- instantiation of the SALSA step kernel for KT=float, diagnostics=false.
#include "salsa_kernel_impl.cuh"

namespace salsa {
cudaError_t launch_f0(const DevParams &P, cudaStream_t st, int grid) { return launch_t<float, false>(P, st, grid); }
int blocks_per_sm_f0(const DevParams &P) { return blocks_per_sm_t<float, false>(P); }
}  // namespace salsa
