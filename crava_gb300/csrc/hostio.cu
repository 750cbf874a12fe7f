// Kernel access to host memory.
//
// On GB300 the Grace host memory sits behind NVLink-C2C and is coherent with
// the GPU: a kernel can load and store page-locked (registered or
// cudaHostAlloc'd) host memory through its mapped device address, and, where
// the device reports pageable-memory access, any host address.  Streaming
// through kernels runs both link directions at once and lets the transform
// and bin kernels read their inputs from, and write their outputs to, host
// cubes directly (no staging copy in device memory).
#include "common.cuh"
#include "hostio.cuh"
#include "trace.cuh"

namespace cg {

// device address of p (device, managed, page-locked host, or pageable host
// memory when the device can address it); nullptr when the device cannot
// address p
void *device_view(const void *p)
{
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  switch (a.type) {
    case cudaMemoryTypeDevice:
    case cudaMemoryTypeManaged: return const_cast<void *>(p);
    case cudaMemoryTypeHost: {
      if (a.devicePointer) {
        // offset of p inside its registration: devicePointer maps p itself
        return a.devicePointer;
      }
      return nullptr;
    }
    default: {
      int dev = 0, pageable = 0;
      if (cudaGetDevice(&dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
      }
      return pageable ? const_cast<void *>(p) : nullptr;
    }
  }
}

bool is_host_memory(const void *p)
{
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return true;
  }
  return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeUnregistered;
}

// 16-byte grid-stride copy, four loads in flight per thread
__global__ void __launch_bounds__(256) k_copy16(uint4 *__restrict__ dst, const uint4 *__restrict__ src, long n16)
{
  const long stride = (long)gridDim.x * blockDim.x;
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n16; i += 4 * stride) {
    const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n16; i += stride) dst[i] = src[i];
}

int copy_kernel(void *dst, const void *src, size_t bytes, cudaStream_t st)
{
  if (bytes == 0) return CG_OK;
  if (((uintptr_t)dst | (uintptr_t)src | bytes) & 15) {
    set_error("cg_copy needs 16-byte aligned pointers and size");
    return CG_ERR_ARG;
  }
  const long n16 = (long)(bytes / 16);
  int dev = 0, nsm = 0;
  CG_CUDA(cudaGetDevice(&dev));
  CG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const long want = (n16 + 4L * 256 - 1) / (4L * 256);
  const int grid = (int)(want < 8L * nsm ? (want > 0 ? want : 1) : 8L * nsm);
  TraceScope ts("k_copy16", st, 2.0 * (double)bytes);
  k_copy16<<<grid, 256, 0, st>>>((uint4 *)dst, (const uint4 *)src, n16);
  CG_CHECK_LAUNCH("k_copy16");
  return CG_OK;
}

}  // namespace cg

using namespace cg;

extern "C" int cg_copy(void *dst, const void *src, size_t bytes, void *stream)
{
  if (!dst || !src) { set_error("cg_copy: null pointer"); return CG_ERR_ARG; }
  void *d = device_view(dst);
  const void *s = device_view(src);
  if (!d || !s) {
    set_error("cg_copy: the device cannot address %s (register host memory with cg_host_register)",
              !d ? "the destination" : "the source");
    return CG_ERR_UNSUPPORTED;
  }
  return copy_kernel(d, s, bytes, (cudaStream_t)stream);
}

extern "C" int cg_host_access(void)
{
  int dev = 0, pageable = 0, tables = 0, direct = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { (void)cudaGetLastError(); return 0; }
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) pageable = 0;
  if (cudaDeviceGetAttribute(&tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) tables = 0;
  if (cudaDeviceGetAttribute(&direct, cudaDevAttrCanUseHostPointerForRegisteredMem, dev) != cudaSuccess) direct = 0;
  (void)cudaGetLastError();
  return (pageable ? 1 : 0) | (tables ? 2 : 0) | (direct ? 4 : 0);
}
