// 4D time-lapse: the step between two vintages -- State4D::evolve
// (src/state4d.cpp:800-996) -- and the generalised-exponential correlation
// cube it transforms for the covariance increment (FFTGrid::fillInGenExpCorr,
// src/fftgrid.cpp:1144-1187).
//
// Per bin, with the 6-parameter state (static + dynamic means, 6x6 Hermitian
// covariance) as spectra:
//   mu  <- E mu + c sqrt(N) [bin (0,0,0) only: a constant in the real domain]
//   Sig <- E Sig E^T + C Re(Lambda(bin))
// E, c, C from the time evolution model; Lambda the transformed correlation
// cube.  The reference forms these products in FP64 and stores FP32; on this
// part FP64 runs at a small fraction of the FP32 rate, so the kernel forms
// them in FP32 (row by row: 684 FMAs per bin instead of 1728 FP64 ones) and
// stays within a few FP32 roundings of the reference.
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "trace.cuh"

namespace cg {

#define CG_RMISSING_F (-99999.000f)

// subK = k + cycleI*gradI + cycleJ*gradJ with separate float roundings (as the
// reference's float expression, no FMA contraction)
__device__ __forceinline__ float genexp_lag(int k, int ci, int cj, float gi, float gj)
{
  return __fadd_rn(__fadd_rn((float)k, __fmul_rn((float)ci, gi)), __fmul_rn((float)cj, gj));
}

__global__ void k_fill_genexp(float *buf, int nxp, int nyp, int nzp, double rx, double ry, double rz, float gi,
                              float gj)
{
  const int rnxp = 2 * (nxp / 2 + 1);
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long n = (long)rnxp * nyp * nzp;
  if (idx >= n) return;
  const int i = (int)(idx % rnxp);
  const int j = (int)((idx / rnxp) % nyp);
  const int k = (int)(idx / ((long)rnxp * nyp));
  if (i >= nxp) {
    buf[idx] = CG_RMISSING_F;
    return;
  }
  int ci = i - nxp; if (i < -ci) ci = i;
  int cj = j - nyp; if (j < -cj) cj = j;
  float subK = genexp_lag(k, ci, cj, gi, gj);
  // cyclic reduction into [-nzp/2, nzp/2) by whole periods, as the reference's loops add or subtract nzp
  // one period at a time; lags many periods away (steep gradients) are reduced in one step first
  const double half = nzp / 2.0;
  if (fabs((double)subK) > 64.0 * nzp) subK -= (float)nzp * floorf((subK + (float)half) / (float)nzp);
  for (int it = 0; it < 130 && subK < -half; it++) subK = __fadd_rn(subK, (float)nzp);
  for (int it = 0; it < 130 && subK >= half; it++) subK = __fadd_rn(subK, -(float)nzp);
  const double q = (double)(float)(ci * ci) / (rx * rx) + (double)(cj * cj) / (ry * ry) +
                   (double)__fmul_rn(subK, subK) / (rz * rz);
  buf[idx] = (float)exp(-3.0 * sqrt(q));
}

struct EvolveArgs {
  float2 *mu[6];      // mu_s 0..2, mu_d 3..5
  float2 *sig[21];    // ss (00 01 02 11 12 22), dd (33 34 35 44 45 55), sd (03 04 05 13 14 15 23 24 25)
  const float2 *lam;  // transformed correlation cube, or null (no covariance increment)
  float E[36], C[36], c[6];
  float c_scale;      // float(sqrt(N)) for the (0,0,0) bin
  long csize;
};

// index into sig[] of the entry (d1, d2), d1 <= d2, and whether it is stored
__host__ __device__ constexpr int sig_index(int d1, int d2)
{
  return d1 < 3 && d2 < 3   ? (d1 == 0 ? d2 : d1 == 1 ? 2 + d2 : 5)                       // ss
         : d1 >= 3          ? 6 + (d1 == 3 ? d2 - 3 : d1 == 4 ? 2 + d2 - 3 : 5)            // dd
                            : 12 + 3 * d1 + (d2 - 3);                                       // sd
}

__global__ void __launch_bounds__(128) k_state4d_evolve(const __grid_constant__ EvolveArgs a)
{
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.csize) return;
  // means
  float2 m[6];
#pragma unroll
  for (int d = 0; d < 6; d++) m[d] = a.mu[d][b];
  const float cs = b == 0 ? a.c_scale : 0.0f;
#pragma unroll
  for (int d = 0; d < 6; d++) {
    float re = a.c[d] * cs, im = 0.0f;
#pragma unroll
    for (int e = 0; e < 6; e++) {
      re = fmaf(a.E[d * 6 + e], m[e].x, re);
      im = fmaf(a.E[d * 6 + e], m[e].y, im);
    }
    a.mu[d][b] = make_float2(re, im);
  }
  // covariance: the full Hermitian 6x6 from its stored triangle
  float2 S[6][6];
#pragma unroll
  for (int d1 = 0; d1 < 6; d1++)
#pragma unroll
    for (int d2 = d1; d2 < 6; d2++) {
      const float2 v = a.sig[sig_index(d1, d2)][b];
      S[d1][d2] = v;
      S[d2][d1] = make_float2(v.x, -v.y);
    }
  const float lre = a.lam ? a.lam[b].x : 0.0f;
  // row d1 of E S, then the stored entries (d1, d2 >= d1) of (E S) E^T + C Re(Lambda)
  float2 out[21];
#pragma unroll
  for (int d1 = 0; d1 < 6; d1++) {
    float2 r[6];
#pragma unroll
    for (int q = 0; q < 6; q++) {
      float re = 0.0f, im = 0.0f;
#pragma unroll
      for (int p = 0; p < 6; p++) {
        re = fmaf(a.E[d1 * 6 + p], S[p][q].x, re);
        im = fmaf(a.E[d1 * 6 + p], S[p][q].y, im);
      }
      r[q] = make_float2(re, im);
    }
#pragma unroll
    for (int d2 = d1; d2 < 6; d2++) {
      float re = a.C[d1 * 6 + d2] * lre, im = 0.0f;
#pragma unroll
      for (int q = 0; q < 6; q++) {
        re = fmaf(r[q].x, a.E[d2 * 6 + q], re);
        im = fmaf(r[q].y, a.E[d2 * 6 + q], im);
      }
      out[sig_index(d1, d2)] = make_float2(re, im);
    }
  }
#pragma unroll
  for (int t = 0; t < 21; t++) a.sig[t][b] = out[t];
}

}  // namespace cg

using namespace cg;

extern "C" int cg_fill_genexp_corr(float *buf, int nxp, int nyp, int nzp, double range_x, double range_y,
                                   double range_z, float grad_i, float grad_j, void *stream)
{
  if (!buf || nxp < 1 || nyp < 1 || nzp < 1 || !(range_x > 0) || !(range_y > 0) || !(range_z > 0) ||
      !std::isfinite(grad_i) || !std::isfinite(grad_j)) {
    set_error("cg_fill_genexp_corr: bad argument (positive ranges, finite gradients)");
    return CG_ERR_ARG;
  }
  const long n = 2L * (nxp / 2 + 1) * nyp * nzp;
  TraceScope ts("k_fill_genexp", (cudaStream_t)stream, 4.0 * n);
  k_fill_genexp<<<ceil_div(n, 256), 256, 0, (cudaStream_t)stream>>>(buf, nxp, nyp, nzp, range_x, range_y, range_z,
                                                                     grad_i, grad_j);
  CG_CHECK_LAUNCH("k_fill_genexp");
  return CG_OK;
}

extern "C" int cg_state4d_evolve(float *const *mu_s, float *const *mu_d, float *const *ss, float *const *sd,
                                 float *const *dd, const float *lambda_spec, const double *evolution,
                                 const double *mean_correction, const double *cov_correction, int nxp, int nyp,
                                 int nzp, void *stream)
{
  if (!mu_s || !mu_d || !ss || !sd || !dd || !evolution || !mean_correction || !cov_correction || nxp < 1 ||
      nyp < 1 || nzp < 1) {
    set_error("cg_state4d_evolve: bad argument");
    return CG_ERR_ARG;
  }
  EvolveArgs a;
  memset(&a, 0, sizeof(a));
  for (int t = 0; t < 3; t++) { a.mu[t] = (float2 *)mu_s[t]; a.mu[3 + t] = (float2 *)mu_d[t]; }
  for (int t = 0; t < 6; t++) { a.sig[t] = (float2 *)ss[t]; a.sig[6 + t] = (float2 *)dd[t]; }
  for (int t = 0; t < 9; t++) a.sig[12 + t] = (float2 *)sd[t];
  for (int t = 0; t < 6; t++) if (!a.mu[t]) { set_error("cg_state4d_evolve: null mean grid"); return CG_ERR_ARG; }
  for (int t = 0; t < 21; t++) if (!a.sig[t]) { set_error("cg_state4d_evolve: null covariance grid"); return CG_ERR_ARG; }
  a.lam = (const float2 *)lambda_spec;
  for (int t = 0; t < 36; t++) { a.E[t] = (float)evolution[t]; a.C[t] = (float)cov_correction[t]; }
  for (int t = 0; t < 6; t++) a.c[t] = (float)mean_correction[t];
  a.c_scale = (float)std::sqrt((double)nxp * nyp * nzp);
  a.csize = (long)(nxp / 2 + 1) * nyp * nzp;
  TraceScope ts("k_state4d_evolve", (cudaStream_t)stream, 8.0 * a.csize * (27 + 27 + (lambda_spec ? 1 : 0)));
  k_state4d_evolve<<<ceil_div(a.csize, 128), 128, 0, (cudaStream_t)stream>>>(a);
  CG_CHECK_LAUNCH("k_state4d_evolve");
  return CG_OK;
}
