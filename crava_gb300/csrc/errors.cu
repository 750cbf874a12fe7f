// Error text and status plumbing shared by every C-ABI entry point.
#include <cstdarg>
#include <cstdio>

#include "common.cuh"

namespace cg {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char *where)
{
  (void)cudaGetLastError();  // clear a non-sticky error so it is not reported twice
  set_error("CUDA error in %s: %s (%d)", where, cudaGetErrorString(e), (int)e);
  return CG_ERR_CUDA;
}

// Stream-ordered scratch allocation.  The device's default memory pool
// returns its memory at every synchronisation unless told otherwise, and the
// next cudaMallocAsync then maps it again; the library's pool keeps what it
// has (release threshold: unlimited), set once per device.  The attribute
// belongs to this process's pool, not to the GPU.
cudaError_t scratch_alloc(void **p, size_t bytes, cudaStream_t st)
{
  static bool done[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < 64 && !done[dev]) {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      unsigned long long keep = ~0ULL;
      (void)cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    (void)cudaGetLastError();
    done[dev] = true;
  }
  return cudaMallocAsync(p, bytes, st);
}

}  // namespace cg

extern "C" const char *cg_last_error(void) { return cg::g_err; }
extern "C" int cg_version(void) { return 100; }
