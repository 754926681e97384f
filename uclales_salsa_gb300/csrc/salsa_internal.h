// salsa_internal.h -- access to a handle's internals from the translation units that
// implement further entry points of the C-ABI (C++ linkage; not part of the C-ABI).
#pragma once
#include <cuda_runtime.h>
#include <initializer_list>
#include "../../include/salsa_gb300.h"
#include "salsa_device.cuh"

namespace salsa {
// the layout part of the kernel parameters, the library stream, device and SM count
bool handle_params(const salsa_handle_t *h, DevParams *base, cudaStream_t *stream, int *device, int *nsm);
const salsa_config_t *handle_config(const salsa_handle_t *h);
// a device buffer of at least `bytes` owned by the handle (slot 0..3), grown on demand
void *handle_scratch(salsa_handle_t *h, int slot, size_t bytes);
// true when every non-NULL pointer is device (or managed) memory
bool device_ptrs(std::initializer_list<const void *> ps);
}  // namespace salsa
