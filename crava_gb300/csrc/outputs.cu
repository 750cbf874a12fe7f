// The step after the bin loop: output grids of the inversion.
//
//   * FFTGrid::expTransf / logTransf (src/fftgrid.cpp:1726-1763) -- the
//     log-domain posterior means become Vp, Vs and density for output
//     (ParameterOutput::writeParameters, src/parameteroutput.cpp:87-108);
//     the exp can also be fused into the last pass of the inverse transform;
//   * SeismicParametersHolder::updatePriorVar and createPostCov00
//     (src/seismicparametersholder.cpp:771-807): the posterior variances at
//     lag 0 and the vertical covariance function at lateral lag 0, read from
//     the real-domain posterior covariance grids.
#include "common.cuh"
#include "fft.cuh"
#include "trace.cuh"

namespace cg {

__global__ void k_exp_transf(float4 *__restrict__ v4, float *__restrict__ tail, long n4, long ntail)
{
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
    float4 a = v4[i];
    a.x = epilogue<float>(a.x, kEpiExp);
    a.y = epilogue<float>(a.y, kEpiExp);
    a.z = epilogue<float>(a.z, kEpiExp);
    a.w = epilogue<float>(a.w, kEpiExp);
    v4[i] = a;
  }
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < ntail; i += stride) tail[i] = epilogue<float>(tail[i], kEpiExp);
}

// FFTGrid::logTransf: RMISSING and values <= 0 become 0, the rest log(value)
__device__ __forceinline__ float log_transf(float v) { return (v == kRMissing || v <= 0.0f) ? 0.0f : logf(v); }

__global__ void k_log_transf(float4 *__restrict__ v4, float *__restrict__ tail, long n4, long ntail)
{
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
    float4 a = v4[i];
    a.x = log_transf(a.x);
    a.y = log_transf(a.y);
    a.z = log_transf(a.z);
    a.w = log_transf(a.w);
    v4[i] = a;
  }
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < ntail; i += stride) tail[i] = log_transf(tail[i]);
}

static int elementwise(bool expo, float *buf, long n, cudaStream_t st)
{
  if (!buf || n < 0) { set_error("bad argument"); return CG_ERR_ARG; }
  if (((uintptr_t)buf) & 15) { set_error("buffer must be 16-byte aligned"); return CG_ERR_ARG; }
  if (n == 0) return CG_OK;
  const long n4 = n / 4, ntail = n - 4 * n4;
  int dev = 0, nsm = 0;
  CG_CUDA(cudaGetDevice(&dev));
  CG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const long want = ceil_div(n4 > 0 ? n4 : 1, 256);
  const int grid = (int)(want < 8L * nsm ? want : 8L * nsm);
  TraceScope ts(expo ? "k_exp_transf" : "k_log_transf", st, 8.0 * n);
  if (expo) k_exp_transf<<<grid, 256, 0, st>>>((float4 *)buf, buf + 4 * n4, n4, ntail);
  else k_log_transf<<<grid, 256, 0, st>>>((float4 *)buf, buf + 4 * n4, n4, ntail);
  CG_CHECK_LAUNCH(expo ? "k_exp_transf" : "k_log_transf");
  return CG_OK;
}

}  // namespace cg

using namespace cg;

extern "C" int cg_exp_transform(float *buf, long n, void *stream)
{
  return elementwise(true, buf, n, (cudaStream_t)stream);
}

extern "C" int cg_log_transform(float *buf, long n, void *stream)
{
  return elementwise(false, buf, n, (cudaStream_t)stream);
}

extern "C" int cg_fft3d_c2r_exp_batch(float *const *bufs, int count, int nxp, int nyp, int nzp, int cubetype,
                                      void *stream)
{
  if (!bufs || count < 1) { set_error("bad argument"); return CG_ERR_ARG; }
  return fft3d_c2r_epi<float>((void *const *)bufs, count, nxp, nyp, nzp, cubetype, kEpiExp, (cudaStream_t)stream);
}

extern "C" int cg_cov_origin(const float *const *cov_real, int nxp, int nyp, int nzp, int nz, double *post_var0,
                             float *post_cov00, void *stream)
{
  if (!cov_real || !post_var0 || nxp < 1 || nyp < 1 || nzp < 1 || nz < 1 || nz > nzp) {
    set_error("cg_cov_origin: bad argument");
    return CG_ERR_ARG;
  }
  for (int t = 0; t < 6; t++)
    if (!cov_real[t]) { set_error("cg_cov_origin: null covariance grid %d", t); return CG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  const size_t plane = sizeof(float) * (size_t)(2 * (nxp / 2 + 1)) * nyp;  // one z-plane of the real cube
  float origin[6];
  for (int t = 0; t < 6; t++)
    CG_CUDA(cudaMemcpyAsync(&origin[t], cov_real[t], sizeof(float), cudaMemcpyDeviceToHost, st));
  if (post_cov00)  // (0,0,k) for k < nz of the alpha, beta and rho grids
    for (int t = 0; t < 3; t++)
      CG_CUDA(cudaMemcpy2DAsync(post_cov00 + (size_t)t * nz, sizeof(float), cov_real[t], plane, sizeof(float), nz,
                                cudaMemcpyDeviceToHost, st));
  CG_CUDA(cudaStreamSynchronize(st));
  // grid order 00 11 22 01 02 12 -> symmetric 3x3 (getOrigin stores float values in the double matrix)
  post_var0[0] = origin[0]; post_var0[4] = origin[1]; post_var0[8] = origin[2];
  post_var0[1] = post_var0[3] = origin[3];
  post_var0[2] = post_var0[6] = origin[4];
  post_var0[5] = post_var0[7] = origin[5];
  return CG_OK;
}
