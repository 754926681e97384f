// salsa_k_fs.cu -- instantiation of the SALSA step kernel for KT=float with secondary ice
// (and diagnostics): the tallies in the coagulation update and the three schemes after it.
#include "salsa_kernel_impl.cuh"

namespace salsa {
cudaError_t launch_fs(const DevParams &P, cudaStream_t st, int grid) { return launch_t<float, true, true>(P, st, grid); }
int blocks_per_sm_fs(const DevParams &P) { return blocks_per_sm_t<float, true, true>(P); }
}  // namespace salsa
