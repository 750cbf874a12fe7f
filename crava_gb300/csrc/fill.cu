// Real-domain correlation cubes for the plain (reference-dataflow) form:
// FFTGrid::fillInParamCorr (src/fftgrid.cpp:1072-1119, times the
// multiplyByScalar of SeismicParametersHolder::initializeCorrelations,
// src/seismicparametersholder.cpp:198-223) and FFTGrid::fillInErrCorr
// (src/fftgrid.cpp:1018-1070), one thread per padded cell, same float
// arithmetic as the reference.
#include "common.cuh"
#include "fill.cuh"
#include "trace.cuh"

namespace cg {

#define CG_RMISSING (-99999.000f)

// The temporal lag k + cycleI*gradI + cycleJ*gradJ of one cell with the
// reference's float roundings: a multiply and two adds, never contracted into
// FMAs, since the error-correlation window (|lag| < 1) makes the cube depend
// on the lag's last bit when the gradients are nonzero.
__device__ __forceinline__ float corr_lag(int k, int cycleI, int cycleJ, float gradI, float gradJ)
{
  return __fadd_rn(__fadd_rn((float)k, __fmul_rn((float)cycleI, gradI)), __fmul_rn((float)cycleJ, gradJ));
}

// (1 - f) a + f b, then times c and s, each operation rounded on its own as
// the reference's float expression is; FP64 for the FP64 tables
__device__ __forceinline__ float lerp_scaled(float f, float a, float b, float c, float s)
{
  const float v = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, f), a), __fmul_rn(f, b));
  return __fmul_rn(__fmul_rn(v, c), s);
}
__device__ __forceinline__ double lerp_scaled(float f, float a, float b, float c, double s)
{
  return ((1.0 - (double)f) * a + (double)f * b) * c * s;
}

// R = float is the reference's arithmetic; R = double keeps the float lag
// (subK) and evaluates the interpolation in FP64, as the FP64 oracle does
template <typename R>
__global__ void k_fill_param_corr(R *buf, int nxp, int nyp, int nzp, const float *__restrict__ corr_xy,
                                  const float *__restrict__ circ_t, float gradI, float gradJ, R scalar)
{
  const int rnxp = 2 * (nxp / 2 + 1);
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long n = (long)rnxp * nyp * nzp;
  if (idx >= n) return;
  const int i = (int)(idx % rnxp);
  const int j = (int)((idx / rnxp) % nyp);
  const int k = (int)(idx / ((long)rnxp * nyp));
  if (i < nxp) {
    int cycleI = i - nxp; if (i < -cycleI) cycleI = i;
    int cycleJ = j - nyp; if (j < -cycleJ) cycleJ = j;
    float subK = corr_lag(k, cycleI, cycleJ, gradI, gradJ);
    int baseK = (int)floorf(subK);
    subK -= baseK;
    baseK %= nzp;
    if (baseK < 0) baseK += nzp;
    buf[idx] = lerp_scaled(subK, circ_t[baseK], circ_t[baseK != nzp - 1 ? baseK + 1 : 0], corr_xy[i + nxp * j],
                           scalar);
  } else {
    buf[idx] = (R)CG_RMISSING * scalar;
  }
}

template <typename R>
__global__ void k_fill_err_corr(R *buf, int nxp, int nyp, int nzp, const float *__restrict__ corr_xy,
                                float gradI, float gradJ)
{
  const int rnxp = 2 * (nxp / 2 + 1);
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long n = (long)rnxp * nyp * nzp;
  if (idx >= n) return;
  const int i = (int)(idx % rnxp);
  const int j = (int)((idx / rnxp) % nyp);
  const int k = (int)(idx / ((long)rnxp * nyp));
  const int range = 1;
  int cycleI = i - nxp; if (i < -cycleI) cycleI = i;
  int cycleJ = j - nyp; if (j < -cycleJ) cycleJ = j;
  float subK = corr_lag(k, cycleI, cycleJ, gradI, gradJ);
  R value;
  if (i < nxp) {
    if (fabsf(subK) < range * 1.0f || fabsf(subK - nzp) < range * 1.0f) {
      int baseK = (int)subK;
      subK -= baseK;
      if (baseK < -range) baseK += nzp * ((-range - baseK + nzp - 1) / nzp);
      if (baseK >= range) baseK -= nzp * ((baseK - range) / nzp + 1);
      if (baseK < 0) { baseK = -1 - baseK; subK = 1 - subK; }
      value = (1 - (R)subK) * (R)corr_xy[i + nxp * j];
    } else {
      value = 0;
    }
  } else {
    value = (R)CG_RMISSING;
  }
  buf[idx] = value;
}

template <typename R>
int fill_param_corr(R *buf, int nxp, int nyp, int nzp, const float *corr_xy, const float *circ_corr_t, float grad_i,
                    float grad_j, R scalar, cudaStream_t st)
{
  if (!buf || !corr_xy || !circ_corr_t || nxp < 1 || nyp < 1 || nzp < 1) { set_error("cg_fill_param_corr: bad argument"); return CG_ERR_ARG; }
  const long n = 2L * (nxp / 2 + 1) * nyp * nzp;
  TraceScope ts("k_fill_param_corr", st, (double)sizeof(R) * n);
  k_fill_param_corr<R><<<ceil_div(n, 256), 256, 0, st>>>(buf, nxp, nyp, nzp, corr_xy, circ_corr_t, grad_i, grad_j,
                                                          scalar);
  CG_CHECK_LAUNCH("k_fill_param_corr");
  return CG_OK;
}

template <typename R>
int fill_err_corr(R *buf, int nxp, int nyp, int nzp, const float *corr_xy, float grad_i, float grad_j, cudaStream_t st)
{
  if (!buf || !corr_xy || nxp < 1 || nyp < 1 || nzp < 1) { set_error("cg_fill_err_corr: bad argument"); return CG_ERR_ARG; }
  const long n = 2L * (nxp / 2 + 1) * nyp * nzp;
  TraceScope ts("k_fill_err_corr", st, (double)sizeof(R) * n);
  k_fill_err_corr<R><<<ceil_div(n, 256), 256, 0, st>>>(buf, nxp, nyp, nzp, corr_xy, grad_i, grad_j);
  CG_CHECK_LAUNCH("k_fill_err_corr");
  return CG_OK;
}

template int fill_param_corr<float>(float *, int, int, int, const float *, const float *, float, float, float,
                                    cudaStream_t);
template int fill_param_corr<double>(double *, int, int, int, const float *, const float *, float, float, double,
                                     cudaStream_t);
template int fill_err_corr<float>(float *, int, int, int, const float *, float, float, cudaStream_t);
template int fill_err_corr<double>(double *, int, int, int, const float *, float, float, cudaStream_t);

}  // namespace cg

using namespace cg;

extern "C" int cg_fill_param_corr(float *buf, int nxp, int nyp, int nzp, const float *corr_xy,
                                  const float *circ_corr_t, float grad_i, float grad_j, float scalar, void *stream)
{
  return fill_param_corr<float>(buf, nxp, nyp, nzp, corr_xy, circ_corr_t, grad_i, grad_j, scalar,
                                (cudaStream_t)stream);
}

extern "C" int cg_fill_err_corr(float *buf, int nxp, int nyp, int nzp, const float *corr_xy, float grad_i,
                                float grad_j, void *stream)
{
  return fill_err_corr<float>(buf, nxp, nyp, nzp, corr_xy, grad_i, grad_j, (cudaStream_t)stream);
}

// FFTGrid::multiplyByScalar / add (src/fftgrid.cpp:1985-1996, :1870-1891)
// over the whole padded buffer, vectorised by float4 where aligned.
__global__ void k_scale(float *buf, long n, float s)
{
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long n4 = n / 4;
  if (i < n4) {
    float4 v = reinterpret_cast<float4 *>(buf)[i];
    v.x *= s; v.y *= s; v.z *= s; v.w *= s;
    reinterpret_cast<float4 *>(buf)[i] = v;
  }
  if (i < n - 4 * n4) buf[4 * n4 + i] *= s;
}

__global__ void k_add(float *y, const float *x, long n)
{
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long n4 = n / 4;
  if (i < n4) {
    float4 a = reinterpret_cast<float4 *>(y)[i];
    const float4 b = reinterpret_cast<const float4 *>(x)[i];
    a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w;
    reinterpret_cast<float4 *>(y)[i] = a;
  }
  if (i < n - 4 * n4) y[4 * n4 + i] += x[4 * n4 + i];
}

extern "C" int cg_scale(float *buf, long n, float s, void *stream)
{
  if (!buf || n < 0 || ((uintptr_t)buf & 15)) { cg::set_error("cg_scale: bad argument (buffer must be 16-byte aligned)"); return CG_ERR_ARG; }
  if (n == 0) return CG_OK;
  cg::TraceScope ts("k_scale", (cudaStream_t)stream, 8.0 * n);
  k_scale<<<cg::ceil_div(n / 4 + 4, 256), 256, 0, (cudaStream_t)stream>>>(buf, n, s);
  CG_CHECK_LAUNCH("k_scale");
  return CG_OK;
}

extern "C" int cg_add(float *y, const float *x, long n, void *stream)
{
  if (!y || !x || n < 0 || ((uintptr_t)y & 15) || ((uintptr_t)x & 15)) { cg::set_error("cg_add: bad argument (buffers must be 16-byte aligned)"); return CG_ERR_ARG; }
  if (n == 0) return CG_OK;
  cg::TraceScope ts("k_add", (cudaStream_t)stream, 12.0 * n);
  k_add<<<cg::ceil_div(n / 4 + 4, 256), 256, 0, (cudaStream_t)stream>>>(y, x, n);
  CG_CHECK_LAUNCH("k_add");
  return CG_OK;
}
