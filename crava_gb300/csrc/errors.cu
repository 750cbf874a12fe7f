// Error text and status plumbing shared by every C-ABI entry point.
#include <cstdarg>
#include <atomic>
#include <cstdio>
#include <mutex>

#include "common.cuh"

namespace cg {

static thread_local char g_err[512] = "";
static std::atomic<long> g_alloc_calls{0};

void count_alloc() { g_alloc_calls.fetch_add(1, std::memory_order_relaxed); }

cudaError_t dev_malloc(void **p, size_t bytes)
{
  count_alloc();
  return cudaMalloc(p, bytes);
}

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

// Stream-ordered scratch allocation from a memory pool of the library's own,
// one per device, created on first use.  A pool returns its memory at every
// synchronisation unless told otherwise, and the next allocation then maps it
// again; this pool keeps what it has (release threshold: unlimited).  It is
// not the device's default pool, so the host application's own
// cudaMallocAsync memory keeps the release behaviour the application chose.
// Scratch is returned with cudaFreeAsync, which finds the pool by itself.
cudaError_t scratch_alloc(void **p, size_t bytes, cudaStream_t st)
{
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  count_alloc();
  if (dev < 0 || dev >= 64) return cudaMallocAsync(p, bytes, st);
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!pools[dev]) {
      cudaMemPoolProps props = {};
      props.allocType = cudaMemAllocationTypePinned;
      props.handleTypes = cudaMemHandleTypeNone;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      cudaMemPool_t np = nullptr;
      count_alloc();
      e = cudaMemPoolCreate(&np, &props);
      if (e != cudaSuccess) return e;
      unsigned long long keep = ~0ULL;
      (void)cudaMemPoolSetAttribute(np, cudaMemPoolAttrReleaseThreshold, &keep);
      (void)cudaGetLastError();
      pools[dev] = np;
    }
    pool = pools[dev];
  }
  return cudaMallocFromPoolAsync(p, bytes, pool, st);
}

}  // namespace cg

extern "C" const char *cg_last_error(void) { return cg::g_err; }
extern "C" int cg_version(void) { return 100; }
extern "C" long cg_alloc_calls(void) { return cg::g_alloc_calls.load(); }
