// salsa_k_ds.cu -- instantiation of the SALSA step kernel for KT=double with secondary ice
// (and diagnostics): the tallies in the coagulation update and the three schemes after it.
#include "salsa_kernel_impl.cuh"

namespace salsa {
cudaError_t launch_ds(const DevParams &P, cudaStream_t st, int grid) { return launch_t<double, true, true>(P, st, grid); }
int blocks_per_sm_ds(const DevParams &P) { return blocks_per_sm_t<double, true, true>(P); }
}  // namespace salsa
