// salsa_k_d1.cu -- instantiation of the SALSA step kernel for KT=double, diagnostics=true.
#include "salsa_kernel_impl.cuh"

namespace salsa {
cudaError_t launch_d1(const DevParams &P, cudaStream_t st, int grid) { return launch_t<double, true>(P, st, grid); }
int blocks_per_sm_d1(const DevParams &P) { return blocks_per_sm_t<double, true>(P); }
}  // namespace salsa
