// salsa_k_f1.cu -- instantiation of the SALSA step kernel for KT=float, diagnostics=true.
#include "salsa_kernel_impl.cuh"

namespace salsa {
cudaError_t launch_f1(const DevParams &P, cudaStream_t st, int grid) { return launch_t<float, true>(P, st, grid); }
int blocks_per_sm_f1(const DevParams &P) { return blocks_per_sm_t<float, true>(P); }
}  // namespace salsa
