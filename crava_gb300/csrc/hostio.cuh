// Kernel access to host memory (hostio.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace cg {
// device address of p, or nullptr when the device cannot address it
void *device_view(const void *p);
// true for page-locked or pageable host memory (false for device/managed)
bool is_host_memory(const void *p);
// 16-byte aligned kernel copy between device-addressable pointers
int copy_kernel(void *dst, const void *src, size_t bytes, cudaStream_t st);
}  // namespace cg
