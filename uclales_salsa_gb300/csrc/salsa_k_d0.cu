// salsa_k_d0.cu -- instantiation of the SALSA step kernel for KT=double, diagnostics=false.
#include "salsa_kernel_impl.cuh"

namespace salsa {
cudaError_t launch_d0(const DevParams &P, cudaStream_t st, int grid) { return launch_t<double, false>(P, st, grid); }
int blocks_per_sm_d0(const DevParams &P) { return blocks_per_sm_t<double, false>(P); }
}  // namespace salsa
