// 3D transforms that allocate nothing.
//
// cg_fft3d_r2c / cg_fft3d_c2r keep their twiddle tables in device memory they
// cudaMalloc the first time a transform length is used.  Some callers cannot
// let a library allocate: code that runs while its application is capturing a
// CUDA graph with allocation forbidden, or a host program whose device memory
// is owned by its own allocator (a memory pool sized up front, a framework
// that accounts for every byte).  For them, cg_fft3d_r2c_noalloc and
// cg_fft3d_c2r_noalloc run the same transforms with the tables in the
// file-scope array below, which every GPU that loads the library holds until
// the process exits (kNoAllocTwiddles float2 = 128 KiB per device).
//
// Each call rebuilds the tables it needs in that array (a small kernel on the
// caller's stream), so every call shares the array and it keeps the last
// call's contents.  Calls whose transforms overlap on the GPU (different
// streams, or different devices' streams queued from host threads at the same
// time) race on it.
//
// The first call on a device looks the array's address up for that device
// (cudaGetSymbolAddress); make that first call before any stream capture.
//
// The column passes never take the TMA-fed kernel here (whatever the tuning
// table says), because that kernel allocates a device fault word on first
// use, and the launch tracer is off for these calls (it creates CUDA events).
#include <cmath>
#include <mutex>

#include "common.cuh"
#include "fft_fast.cuh"
#include "trace.cuh"

namespace cg {

constexpr int kNoAllocTwiddles = 16384;  // nxp + nyp + nzp entries at most
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) float2 g_noalloc_twiddles[kNoAllocTwiddles];

// device-side address of g_noalloc_twiddles, per device, looked up under the lock
static float2 *g_noalloc_ptr[kNoAllocMaxDevices];
static std::mutex g_noalloc_mu;

// tw[t] = exp(-2 pi i t / n) for the three axis tables laid out back to back
__global__ void k_noalloc_twiddles(float2 *tw, int n0, int n1, int n2)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  int n, o;
  if (t < n0) { n = n0; o = t; }
  else if (t < n0 + n1) { n = n1; o = t - n0; }
  else if (t < n0 + n1 + n2) { n = n2; o = t - n0 - n1; }
  else return;
  double s, c;
  sincospi(-2.0 * (double)o / (double)n, &s, &c);
  tw[t] = make_float2((float)c, (float)s);
}

static int noalloc_setup(float2 **ptr)
{
  int dev = 0;
  CG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) {
    set_error("device %d beyond the %d devices the no-allocation transforms support", dev, kNoAllocMaxDevices);
    return CG_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_twiddles);
    if (e != cudaSuccess || !p) return cuda_status(e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress");
    g_noalloc_ptr[dev] = (float2 *)p;
  }
  *ptr = g_noalloc_ptr[dev];
  return CG_OK;
}

static int noalloc_fft(float *buf, int nxp, int nyp, int nzp, int cubetype, bool forward, cudaStream_t st)
{
  if (!buf) { set_error("null buffer"); return CG_ERR_ARG; }
  if (nxp < 2 || nyp < 1 || nzp < 1 || (nxp % 2)) {
    set_error("no-allocation transforms take even nxp >= 2 and nyp, nzp >= 1 (got %d x %d x %d)", nxp, nyp, nzp);
    return CG_ERR_ARG;
  }
  if (cubetype < CG_DATA || cubetype > CG_OPERATOR) { set_error("cubetype %d is not valid", cubetype); return CG_ERR_ARG; }
  if ((long)nxp + nyp + nzp > kNoAllocTwiddles) {
    set_error("nxp + nyp + nzp = %ld exceeds the %d-entry twiddle array of the no-allocation transforms",
              (long)nxp + nyp + nzp, kNoAllocTwiddles);
    return CG_ERR_ARG;
  }
  // check every axis before queuing anything, so an unsupported size leaves buffer and array untouched
  AxisPlan p;
  const int lens[2] = {nyp, nzp};
  for (int a = 0; a < 2; a++) {
    const int n = lens[a];
    if (n == 1) continue;
    if (!make_axis_plan(n, &p) || !(n == 64 || n == 80 || n == 96 || n == 100 || n == 120 || n == 128 || n == 160 ||
                                    n == 192 || n == 200 || n == 240 || n == 256 || n == 320 || n == 384 ||
                                    n == 400 || n == 480 || n == 512)) {
      set_error("axis length %d has no specialised transform; the no-allocation transforms support 64, 80, 96, "
                "100, 120, 128, 160, 192, 200, 240, 256, 320, 384, 400, 480 and 512", n);
      return CG_ERR_UNSUPPORTED;
    }
  }
  {
    const int m = nxp / 2;
    if (!(m == 32 || m == 40 || m == 48 || m == 50 || m == 60 || m == 64 || m == 80 || m == 96 || m == 100 ||
          m == 120 || m == 128 || m == 160 || m == 192 || m == 200 || m == 240 || m == 256)) {
      set_error("nxp %d has no specialised transform; the no-allocation transforms support nxp = 2m for m in "
                "32, 40, 48, 50, 60, 64, 80, 96, 100, 120, 128, 160, 192, 200, 240, 256", nxp);
      return CG_ERR_UNSUPPORTED;
    }
  }
  float2 *tw = nullptr;
  int rc = noalloc_setup(&tw);
  if (rc) return rc;
  TraceSuppress quiet;
  const float2 *twx = tw, *twy = tw + nxp, *twz = tw + nxp + nyp;
  k_noalloc_twiddles<<<ceil_div((long)nxp + nyp + nzp, 256), 256, 0, st>>>(tw, nxp, nyp, nzp);
  CG_CHECK_LAUNCH("k_noalloc_twiddles");
  const int cnxp = nxp / 2 + 1;
  const double N = (double)nxp * nyp * nzp;
  const bool covlike = (cubetype == CG_COVARIANCE || cubetype == CG_OPERATOR);
  CubeSet cs, none;
  for (int i = 0; i < kMaxBatch; i++) { cs.ptr[i] = nullptr; none.ptr[i] = nullptr; }
  cs.ptr[0] = buf;
  int done = 0;
  auto cols = [&](int n, long axis_stride, long batch_stride, int nbatch, const float2 *t, int sign) -> int {
    if (n == 1) return CG_OK;
    int r = fast_cols(cs, 1, n, cnxp, axis_stride, batch_stride, nbatch, sign, t, st, &done, /*no_alloc=*/true);
    if (r < 0) return r;
    if (r == 0 || done != cnxp) {
      set_error("axis length %d has no specialised transform; the no-allocation transforms support 64, 80, 96, "
                "100, 120, 128, 160, 192, 200, 240, 256, 320, 384, 400, 480 and 512", n);
      return CG_ERR_UNSUPPORTED;
    }
    return CG_OK;
  };
  auto rows = [&](float scale) -> int {
    int r = fast_rows(forward, cs, none, 1, nxp, nyp * nzp, scale, twx, st);
    if (r < 0) return r;
    if (r == 0) {
      set_error("nxp %d has no specialised transform; the no-allocation transforms support nxp = 2m for m in "
                "32, 40, 48, 50, 60, 64, 80, 96, 100, 120, 128, 160, 192, 200, 240, 256", nxp);
      return CG_ERR_UNSUPPORTED;
    }
    return CG_OK;
  };
  if (forward) {
    const float pre = covlike ? 1.0f : (float)(1.0 / sqrt(N));
    if ((rc = rows(pre))) return rc;
    if ((rc = cols(nyp, cnxp, (long)nyp * cnxp, nzp, twy, -1))) return rc;
    if ((rc = cols(nzp, (long)cnxp * nyp, cnxp, nyp, twz, -1))) return rc;
  } else {
    const float post = covlike ? (float)(1.0 / N) : (float)(1.0 / sqrt(N));
    if ((rc = cols(nzp, (long)cnxp * nyp, cnxp, nyp, twz, +1))) return rc;
    if ((rc = cols(nyp, cnxp, (long)nyp * cnxp, nzp, twy, +1))) return rc;
    if ((rc = rows(post))) return rc;
  }
  return CG_OK;
}

}  // namespace cg

using namespace cg;

extern "C" int cg_fft3d_r2c_noalloc(float *buf, int nxp, int nyp, int nzp, int cubetype, void *stream)
{
  return noalloc_fft(buf, nxp, nyp, nzp, cubetype, true, (cudaStream_t)stream);
}

extern "C" int cg_fft3d_c2r_noalloc(float *buf, int nxp, int nyp, int nzp, int cubetype, void *stream)
{
  return noalloc_fft(buf, nxp, nyp, nzp, cubetype, false, (cudaStream_t)stream);
}
