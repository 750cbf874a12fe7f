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

}  // namespace cg

extern "C" const char *cg_last_error(void) { return cg::g_err; }
extern "C" int cg_version(void) { return 100; }
