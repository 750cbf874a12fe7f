// Per-frequency-bin Gaussian posterior of Crava::computePostMeanResidAndFFTCov
// (src/crava.cpp:1084-1247).
//
// Two GPU forms:
//   plain  -- the reference dataflow: the prior comes from six covariance
//             spectra and the error correlation from a seventh, all read from
//             HBM per bin; arithmetic in the reference's order
//             (invertSeismicData, src/crava.cpp:1389-1438, lib_matr.c), FP32.
//   fused  -- the prior and error covariances are regenerated per bin from the
//             separable spectra c(i,j,k) = Cxy(i,j) Ct(k) (fillInParamCorr /
//             fillInErrCorr with zero correlation gradients; with nonzero
//             gradients each bin's two scales are read from a per-bin table
//             built by cg_prior_spectra_grad), the per-k
//             matrices K S0 K^H and the error-term matrix are precomputed once
//             per model, and the posterior is formed from one Cholesky factor:
//               Sd = s M + lam E + D,  Y = L^-1 K S0,  v = L^-1 (d - K mu)
//               mu+ = mu + s Y^H v,  S+ = s S0 - s^2 Y^H Y,  res = d - K mu+
//             FP32, or MIXED (bins whose Cholesky condition estimate exceeds a
//             threshold are queued and redone in FP64 with one step of
//             iterative refinement), or FP64 throughout.
// Bins outside the inversion band keep prior mean, data and covariance, as in
// the reference; with the in-place buffers only the covariance is written.
#include <cmath>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "fft.cuh"
#include "fill.cuh"
#include "posterior.cuh"
#include "fused_bins.cuh"
#include "linalg.cuh"
#include "plain_bin.cuh"
#include "trace.cuh"

namespace cg {

// ---------------------------------------------------------------------------
// plain (reference-order) kernel
// ---------------------------------------------------------------------------
struct PlainArgs {
  float2 *data[kMaxTheta];
  float2 *mean[3];
  float2 *cov[6];
  const float2 *errcorr;
  const float2 *K;
  const float2 *em1, *em2, *em3;
  const unsigned char *band;
  float c0[kMaxTheta * kMaxTheta];  // float(0.5*(1-wnc)*errThetaCov[l][m])
  float cw[kMaxTheta];              // float(wnc*errThetaCov[l][l])
  float sig0[6];                    // float(priorVar0): 00 11 22 01 02 12
  int plane;
  long csize;
  int is4d;
  int *counters;
};

// SeismicParametersHolder::getParameterCovariance (src/seismicparametersholder.cpp:409-428)
__device__ __forceinline__ float2 param_cov_entry(float2 v, float s)
{
  if (s != 0.0f) v.x = v.x / s;
  return make_float2(sqrtf(v.x * v.x) * s, 0.0f);
}

template <int NT>
__global__ void __launch_bounds__(128) k_invert_plain(const __grid_constant__ PlainArgs a)
{
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.csize) return;
  const int k = (int)(b / a.plane);

  // findParameterVariances (src/seismicparametersholder.cpp:357-407)
  float2 c6[6];
#pragma unroll
  for (int t = 0; t < 6; t++) c6[t] = a.cov[t][b];
  if (a.is4d) {
#pragma unroll
    for (int t = 0; t < 3; t++) c6[t] = make_float2(sqrtf(c6[t].x * c6[t].x + c6[t].y * c6[t].y), 0.0f);
  } else {
#pragma unroll
    for (int t = 0; t < 6; t++) c6[t] = param_cov_entry(c6[t], a.sig0[t]);
  }
  float2 S[3][3];
  S[0][0] = c6[0]; S[1][1] = c6[1]; S[2][2] = c6[2];
  S[0][1] = c6[3]; S[1][0] = make_float2(c6[3].x, -c6[3].y);
  S[0][2] = c6[4]; S[2][0] = make_float2(c6[4].x, -c6[4].y);
  S[1][2] = c6[5]; S[2][1] = make_float2(c6[5].x, -c6[5].y);

  if (a.band[k]) {
    float2 res[NT], mu[3];
#pragma unroll
    for (int l = 0; l < NT; l++) res[l] = a.data[l][b];
#pragma unroll
    for (int p = 0; p < 3; p++) mu[p] = a.mean[p][b];
    const float2 ec = a.errcorr[b];
    const float lam = sqrtf(ec.x * ec.x);
    float cond;
    if (plain_solve<float, NT>(a.K + (long)k * NT * 3, a.em1 + (long)k * NT, a.em2 + (long)k * NT,
                               a.em3 + (long)k * NT, a.c0, a.cw, lam, S, mu, res, &cond)) {
#pragma unroll
      for (int l = 0; l < NT; l++) a.data[l][b] = res[l];
#pragma unroll
      for (int p = 0; p < 3; p++) a.mean[p][b] = mu[p];
    } else if (a.counters) {
      atomicAdd(&a.counters[1], 1);
    }
  }
  a.cov[0][b] = S[0][0];
  a.cov[1][b] = S[1][1];
  a.cov[2][b] = S[2][2];
  a.cov[3][b] = S[0][1];
  a.cov[4][b] = S[0][2];
  a.cov[5][b] = S[1][2];
}

// one bin of k_invert_fused (plane k, bin ij of the plane)
template <typename T, int NT, int MODE, bool TAB>
__device__ __forceinline__ void fused_bin(const FusedArgs<T> &a, const KTab<T> &kt, int k, int ij)
{
  const long b = (long)k * a.plane + ij;
  T s, lam;
  bin_scales<T, TAB>(a, ij, k, s, lam);
  if (!kt.band) {
    write_prior_cov<T>(a, b, s);
    return;
  }
  C2<T> d[NT], mu[3], cov[6], L[NT * (NT + 1) / 2];
#pragma unroll
  for (int l = 0; l < NT; l++) d[l] = a.data[l][b];
#pragma unroll
  for (int p = 0; p < 3; p++) mu[p] = a.mean[p][b];
  build_sd<T, NT>(kt, s, lam, L);
  T cond = 0, inv[NT];
  const bool ok = chol_std<T, NT>(L, inv, cond);
  if (MODE == 1) {
    const bool flag = !ok || cond > (T)a.cond_thr;
    const unsigned m = __ballot_sync(__activemask(), flag);
    if (flag) {
      const int lane = threadIdx.x & 31;
      const int leader = __ffs(m) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(&a.counters[0], __popc(m));
      base = __shfl_sync(m, base, leader);
      const int pos = base + __popc(m & ((1u << lane) - 1u));
      if (pos < a.queue_cap) {
        a.queue[pos] = (int)b;
        return;  // the FP64 pass writes this bin
      }
      atomicAdd(&a.counters[2], 1);  // queue full: keep the FP32 answer
    }
  }
  if (!ok) {
    if (a.counters) atomicAdd(&a.counters[1], 1);
    write_prior_cov<T>(a, b, s);
    return;
  }
  posterior_from_chol<T, NT>(kt, a.sig0, s, lam, L, inv, d, mu, cov, MODE == 2);
#pragma unroll
  for (int l = 0; l < NT; l++) a.data[l][b] = d[l];
#pragma unroll
  for (int p = 0; p < 3; p++) a.mean[p][b] = mu[p];
#pragma unroll
  for (int t = 0; t < 6; t++) a.cov[t][b] = cov[t];
}

// MODE 0: FP32, 1: MIXED (FP32 + queue), 2: FP64 (T = double).  MINB is the
// resident-CTA target handed to the register allocator (1 = unconstrained,
// 6 = at most 85 registers).  A CTA solves nruns runs of blockDim.x bins of
// one plane, so the per-k table is staged once for all of them.
template <typename T, int NT, int MODE, int MINB = 1, bool TAB = false>
__global__ void __launch_bounds__(128, MINB) k_invert_fused(FusedArgs<T> a, int nruns)
{
  __shared__ KTab<T> kt;
  const int k = a.k0 + blockIdx.y;
  {
    const int *src = (const int *)&a.ktab[k];
    int *dst = (int *)&kt;
    for (int t = threadIdx.x; t < (int)(sizeof(KTab<T>) / sizeof(int)); t += blockDim.x) dst[t] = src[t];
  }
  __syncthreads();
#pragma unroll 1
  for (int r = 0; r < nruns; r++) {
    const int ij = (blockIdx.x * nruns + r) * blockDim.x + threadIdx.x;
    if (ij >= a.plane) return;
    fused_bin<T, NT, MODE, TAB>(a, kt, k, ij);
  }
}

// Information-form bin solve (FP32; MODE 0 FP32, 1 MIXED with the FP64 queue
// of k_invert_fixup64, which redoes a queued bin with the Cholesky of Sd).
// Per in-band bin: w_m = 1/(lam mu_m + 1), Q = Sigma0^-1/s + sum w_m P_m,
// S+ = Q^-1 from the 3x3 Cholesky of Q (its squared pivot ratio is the
// condition estimate), r = d - K mu, b = sum_m G_m w_m (v_m^H r),
// mu+ = mu + S+ b, residual = d - K mu+.  s = 0 keeps the prior (S+ = 0).
struct InfoArgs {
  float s0i[6];  // Sigma0^-1, bin order 00 11 22 01 02 12
};

// one bin of k_invert_info (plane k, bin ij of the plane)
template <int NT, int MODE, bool TAB>
__device__ __forceinline__ void info_bin(const FusedArgs<float> &a, const ITab &it, const InfoArgs &ia, int k, int ij)
{
  const long b = (long)k * a.plane + ij;
  float s, lam;
  bin_scales<float, TAB>(a, ij, k, s, lam);
  if (!it.band) {
    write_prior_cov<float>(a, b, s);
    return;
  }
  float2 d[NT], mu[3];
#pragma unroll
  for (int l = 0; l < NT; l++) d[l] = a.data[l][b];
#pragma unroll
  for (int p = 0; p < 3; p++) mu[p] = a.mean[p][b];
  float2 S01, S02, S12;
  float S00, S11, S22;
  if (s > 0.0f) {
    const float is = 1.0f / s;
    float w[NT];
#pragma unroll
    for (int m = 0; m < NT; m++) w[m] = 1.0f / (lam * it.mu[m] + 1.0f);
    float q00 = ia.s0i[0] * is, q11 = ia.s0i[1] * is, q22 = ia.s0i[2] * is;
    float2 q01 = make_float2(ia.s0i[3] * is, 0.0f), q02 = make_float2(ia.s0i[4] * is, 0.0f),
           q12 = make_float2(ia.s0i[5] * is, 0.0f);
#pragma unroll
    for (int m = 0; m < NT; m++) {
      const float *P = it.P[m];
      q00 += w[m] * P[0];
      q11 += w[m] * P[1];
      q22 += w[m] * P[2];
      q01.x += w[m] * P[3]; q01.y += w[m] * P[4];
      q02.x += w[m] * P[5]; q02.y += w[m] * P[6];
      q12.x += w[m] * P[7]; q12.y += w[m] * P[8];
    }
    // Q = L L^H, L lower: L10 = conj(q01)/L00, L20 = conj(q02)/L00, L21 = (conj(q12) - L20 conj(L10))/L11
    bool ok = q00 > 0.0f;
    const float r0 = rsqrtf(q00), l00 = q00 * r0;
    const float2 l10 = make_float2(q01.x * r0, -q01.y * r0), l20 = make_float2(q02.x * r0, -q02.y * r0);
    const float p1 = q11 - (l10.x * l10.x + l10.y * l10.y);
    ok = ok && p1 > 0.0f;
    const float r1 = rsqrtf(p1), l11 = p1 * r1;
    const float2 t21 = csub<float>(make_float2(q12.x, -q12.y), cmulc<float>(l20, l10));
    const float2 l21 = make_float2(t21.x * r1, t21.y * r1);
    const float p2 = q22 - (l20.x * l20.x + l20.y * l20.y) - (l21.x * l21.x + l21.y * l21.y);
    ok = ok && p2 > 0.0f;
    const float r2 = rsqrtf(p2), l22 = p2 * r2;
    const float dmax = fmaxf(l00, fmaxf(l11, l22)), dmin = fminf(l00, fminf(l11, l22));
    const float cond = (dmax / dmin) * (dmax / dmin);
    if (MODE == 1) {
      const bool flag = !ok || cond > a.cond_thr;
      const unsigned msk = __ballot_sync(__activemask(), flag);
      if (flag) {
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(msk) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&a.counters[0], __popc(msk));
        base = __shfl_sync(msk, base, leader);
        const int pos = base + __popc(msk & ((1u << lane) - 1u));
        if (pos < a.queue_cap) {
          a.queue[pos] = (int)b;
          return;  // the FP64 pass writes this bin
        }
        atomicAdd(&a.counters[2], 1);  // queue full: keep the FP32 answer
      }
    }
    if (!ok) {
      atomicAdd(&a.counters[1], 1);
      write_prior_cov<float>(a, b, s);
      return;
    }
    // M = L^-1 (lower), S+ = M^H M
    const float m00 = r0, m11 = r1, m22 = r2;
    const float2 m10 = make_float2(-l10.x * m00 * m11, -l10.y * m00 * m11);
    const float2 m21 = make_float2(-l21.x * m11 * m22, -l21.y * m11 * m22);
    const float2 t20 = cadd<float>(make_float2(l20.x * m00, l20.y * m00), cmul<float>(l21, m10));
    const float2 m20 = make_float2(-t20.x * m22, -t20.y * m22);
    S00 = m00 * m00 + (m10.x * m10.x + m10.y * m10.y) + (m20.x * m20.x + m20.y * m20.y);
    S11 = m11 * m11 + (m21.x * m21.x + m21.y * m21.y);
    S22 = m22 * m22;
    // S01 = conj(m10) m11 + conj(m20) m21, S02 = conj(m20) m22, S12 = conj(m21) m22
    S01 = cadd<float>(make_float2(m10.x * m11, -m10.y * m11), cmulc<float>(m21, m20));
    S02 = make_float2(m20.x * m22, -m20.y * m22);
    S12 = make_float2(m21.x * m22, -m21.y * m22);
    // r = d - K mu, b = sum_m G_m w_m (v_m^H r), mu+ = mu + S+ b
    float2 r[NT];
#pragma unroll
    for (int l = 0; l < NT; l++) {
      float2 km = make_float2(0.f, 0.f);
#pragma unroll
      for (int p = 0; p < 3; p++) km = cadd<float>(km, cmul<float>(it.K[l][p], mu[p]));
      r[l] = csub<float>(d[l], km);
    }
    float2 bb[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
    for (int m = 0; m < NT; m++) {
      float2 h = make_float2(0.f, 0.f);
#pragma unroll
      for (int l = 0; l < NT; l++) h = cadd<float>(h, cmulc<float>(r[l], it.V[l][m]));  // conj(v) r
      h = make_float2(h.x * w[m], h.y * w[m]);
#pragma unroll
      for (int p = 0; p < 3; p++) bb[p] = cadd<float>(bb[p], cmul<float>(it.G[m][p], h));
    }
    // S+ rows: (S00, S01, S02), (conj S01, S11, S12), (conj S02, conj S12, S22)
    const float2 u0 = cadd<float>(cadd<float>(make_float2(S00 * bb[0].x, S00 * bb[0].y), cmul<float>(S01, bb[1])),
                                  cmul<float>(S02, bb[2]));
    const float2 u1 = cadd<float>(cadd<float>(cmulc<float>(bb[0], S01), make_float2(S11 * bb[1].x, S11 * bb[1].y)),
                                  cmul<float>(S12, bb[2]));
    const float2 u2 = cadd<float>(cadd<float>(cmulc<float>(bb[0], S02), cmulc<float>(bb[1], S12)),
                                  make_float2(S22 * bb[2].x, S22 * bb[2].y));
    mu[0] = cadd<float>(mu[0], u0);
    mu[1] = cadd<float>(mu[1], u1);
    mu[2] = cadd<float>(mu[2], u2);
  } else {
    S00 = S11 = S22 = 0.0f;
    S01 = S02 = S12 = make_float2(0.f, 0.f);
  }
#pragma unroll
  for (int l = 0; l < NT; l++) {
    float2 km = make_float2(0.f, 0.f);
#pragma unroll
    for (int p = 0; p < 3; p++) km = cadd<float>(km, cmul<float>(it.K[l][p], mu[p]));
    a.data[l][b] = csub<float>(d[l], km);
  }
#pragma unroll
  for (int p = 0; p < 3; p++) a.mean[p][b] = mu[p];
  a.cov[0][b] = make_float2(S00, 0.f);
  a.cov[1][b] = make_float2(S11, 0.f);
  a.cov[2][b] = make_float2(S22, 0.f);
  a.cov[3][b] = S01;
  a.cov[4][b] = S02;
  a.cov[5][b] = S12;
}

// threads per CTA of k_invert_info: the 85-register build runs 256-thread CTAs
// (three per SM), the others 128; a CTA solves up to kInfoBlocks runs of that
// many bins of one plane, so the per-k table is staged once for all of them
__host__ __device__ constexpr int info_threads(int minb) { return minb == 6 ? 256 : 128; }
constexpr int kInfoBlocks = 8;

template <int NT, int MODE, int MINB, bool TAB = false>
__global__ void __launch_bounds__(info_threads(MINB), MINB * 128 / info_threads(MINB))
    k_invert_info(FusedArgs<float> a, const ITab *__restrict__ itab, InfoArgs ia, int nruns)
{
  __shared__ ITab it;
  const int k = a.k0 + blockIdx.y;
  {
    const int *src = (const int *)&itab[k];
    int *dst = (int *)&it;
    for (int t = threadIdx.x; t < (int)(sizeof(ITab) / sizeof(int)); t += blockDim.x) dst[t] = src[t];
  }
  __syncthreads();
#pragma unroll 1
  for (int r = 0; r < nruns; r++) {
    const int ij = (blockIdx.x * nruns + r) * blockDim.x + threadIdx.x;
    if (ij >= a.plane) return;
    info_bin<NT, MODE, TAB>(a, it, ia, k, ij);
  }
}

struct S0Args {
  double v[9];
};

// FP64 redo of the bins the MIXED pass queued.
template <int NT, bool TAB = false>
__global__ void __launch_bounds__(128) k_invert_fixup64(FusedArgs<float> a, const KTab<double> *__restrict__ ktd,
                                                        S0Args s0)
{
  const double *sig0d = s0.v;
  const int nq = min(*((volatile int *)&a.counters[0]), a.queue_cap);
  const int q0 = a.chunked ? *((volatile int *)&a.counters[3]) : 0;
  for (int q = q0 + blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
    const long b = a.queue[q];
    const int k = (int)(b / a.plane);
    const int ij = (int)(b - (long)k * a.plane);
    const KTab<double> &kt = ktd[k];
    float sf, lamf;
    bin_scales<float, TAB>(a, ij, k, sf, lamf);
    const double s = sf, lam = lamf;
    double2 d[NT], mu[3], cov[6], L[NT * (NT + 1) / 2];
#pragma unroll
    for (int l = 0; l < NT; l++) { float2 v = a.data[l][b]; d[l] = make_double2(v.x, v.y); }
#pragma unroll
    for (int p = 0; p < 3; p++) { float2 v = a.mean[p][b]; mu[p] = make_double2(v.x, v.y); }
    build_sd<double, NT>(kt, s, lam, L);
    double cond, inv[NT];
    if (!chol_std<double, NT>(L, inv, cond)) {
      atomicAdd(&a.counters[1], 1);
#pragma unroll
      for (int t = 0; t < 6; t++) a.cov[t][b] = make_float2((float)(s * sig0d[t]), 0.0f);
      continue;
    }
    posterior_from_chol<double, NT>(kt, sig0d, s, lam, L, inv, d, mu, cov, true);
#pragma unroll
    for (int l = 0; l < NT; l++) a.data[l][b] = make_float2((float)d[l].x, (float)d[l].y);
#pragma unroll
    for (int p = 0; p < 3; p++) a.mean[p][b] = make_float2((float)mu[p].x, (float)mu[p].y);
#pragma unroll
    for (int t = 0; t < 6; t++) a.cov[t][b] = make_float2((float)cov[t].x, (float)cov[t].y);
  }
}

__global__ void k_f2d(const float *in, double *out, long n)
{
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int check_ws(Workspace *w)
{
  if (!w) { set_error("null workspace"); return CG_ERR_ARG; }
  if (!w->model_set) { set_error("cg_workspace_set_model has not been called"); return CG_ERR_STATE; }
  int dev = -1;
  CG_CUDA(cudaGetDevice(&dev));
  if (dev != w->device) { set_error("workspace belongs to device %d, current device is %d", w->device, dev); return CG_ERR_STATE; }
  return CG_OK;
}

}  // namespace cg

using namespace cg;

extern "C" int cg_workspace_create(cg_workspace *out, int nxp, int nyp, int nzp, int ntheta)
{
  if (!out) { set_error("null output handle"); return CG_ERR_ARG; }
  *out = nullptr;
  if (nxp < 1 || nyp < 1 || nzp < 1 || nxp > kMaxFFT || nyp > kMaxFFT || nzp > kMaxFFT) {
    set_error("bad dimensions %d x %d x %d", nxp, nyp, nzp);
    return CG_ERR_ARG;
  }
  if (ntheta < 1 || ntheta > kMaxTheta) { set_error("ntheta %d outside 1..%d", ntheta, kMaxTheta); return CG_ERR_ARG; }
  cg_workspace_s *w = new cg_workspace_s();
  memset((Workspace *)w, 0, sizeof(Workspace));
  CG_CUDA(cudaGetDevice(&w->device));
  w->nxp = nxp; w->nyp = nyp; w->nzp = nzp; w->ntheta = ntheta;
  const int cnxp = nxp / 2 + 1, cnzp = nzp / 2 + 1;
  const long csize = (long)cnxp * nyp * nzp;
  w->queue_cap = (int)std::min<long>(csize, std::max<long>(1 << 16, csize / 8));
  cudaError_t e = cudaSuccess;
#define WS_ALLOC(ptr, bytes) if (e == cudaSuccess) e = (count_alloc(), cudaMalloc((void **)&(ptr), (bytes)))
  WS_ALLOC(w->ktab_f, sizeof(KTab<float>) * nzp);
  WS_ALLOC(w->ktab_d, sizeof(KTab<double>) * nzp);
  // uploaded tables, packed in one block: etc | K | em1 | em2 | em3 | band
  const size_t o_k = sizeof(double) * ntheta * ntheta, n_k = sizeof(float2) * (size_t)nzp * ntheta * 3;
  const size_t n_em = sizeof(float2) * (size_t)nzp * ntheta;
  w->model_bytes = o_k + n_k + 3 * n_em + (size_t)nzp;
  WS_ALLOC(w->model_dev, w->model_bytes);
  if (e == cudaSuccess) e = (count_alloc(), cudaMallocHost(&w->model_host, w->model_bytes));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->model_copied, cudaEventDisableTiming);
  if (e == cudaSuccess) {
    char *base = (char *)w->model_dev;
    w->etc = (double *)base;
    w->K = (float2 *)(base + o_k);
    w->em1 = (float2 *)(base + o_k + n_k);
    w->em2 = (float2 *)(base + o_k + n_k + n_em);
    w->em3 = (float2 *)(base + o_k + n_k + 2 * n_em);
    w->band = (unsigned char *)(base + o_k + n_k + 3 * n_em);
  }
  WS_ALLOC(w->cxy_f, sizeof(float) * 2 * (size_t)cnxp * nyp);
  WS_ALLOC(w->ct_f, sizeof(float) * 2 * (size_t)cnzp);
  WS_ALLOC(w->cxy_d, sizeof(double) * 2 * (size_t)cnxp * nyp);
  WS_ALLOC(w->ct_d, sizeof(double) * 2 * (size_t)cnzp);
  WS_ALLOC(w->queue, sizeof(int) * (size_t)w->queue_cap);
  WS_ALLOC(w->counters, sizeof(int) * 4);
  WS_ALLOC(w->itab, sizeof(ITab) * nzp);
#undef WS_ALLOC
  if (e == cudaSuccess) e = cudaMemset(w->counters, 0, sizeof(int) * 4);
  if (e != cudaSuccess) {
    cg_workspace_destroy(w);
    return cuda_status(e, "cg_workspace_create");
  }
  *out = w;
  return CG_OK;
}

extern "C" void cg_workspace_destroy(cg_workspace w)
{
  if (!w) return;
  void *ptrs[] = {w->ktab_f, w->ktab_d, w->model_dev, w->cxy_f, w->ct_f, w->cxy_d, w->ct_d, w->queue, w->counters,
                  w->itab, w->sl_f, w->sl_d};
  if (w->model_copied) {
    cudaEventSynchronize(w->model_copied);
    cudaEventDestroy(w->model_copied);
  }
  if (w->model_host) cudaFreeHost(w->model_host);
  for (void *p : ptrs)
    if (p) cudaFree(p);
  delete w;
}

extern "C" int cg_workspace_set_model_async(cg_workspace w, const cg_model *m, void *stream)
{
  if (!w || !m) { set_error("null argument"); return CG_ERR_ARG; }
  if (m->ntheta != w->ntheta) { set_error("model ntheta %d != workspace ntheta %d", m->ntheta, w->ntheta); return CG_ERR_ARG; }
  if (!m->K || !m->em1 || !m->em2 || !m->em3 || !m->band || !m->err_theta_cov || !m->sigma0) {
    set_error("model table pointer is null");
    return CG_ERR_ARG;
  }
  int dev = -1;
  CG_CUDA(cudaGetDevice(&dev));
  if (dev != w->device) { set_error("workspace belongs to device %d, current device is %d", w->device, dev); return CG_ERR_STATE; }
  cudaStream_t st = (cudaStream_t)stream;
  const int nt = w->ntheta, nzp = w->nzp;
  // the previous model's upload must have left the staging copy
  CG_CUDA(cudaEventSynchronize(w->model_copied));
  char *h = (char *)w->model_host;
  const size_t n_etc = sizeof(double) * nt * nt, n_k = sizeof(float2) * (size_t)nzp * nt * 3;
  const size_t n_em = sizeof(float2) * (size_t)nzp * nt;
  memcpy(h, m->err_theta_cov, n_etc);
  memcpy(h + n_etc, m->K, n_k);
  memcpy(h + n_etc + n_k, m->em1, n_em);
  memcpy(h + n_etc + n_k + n_em, m->em2, n_em);
  memcpy(h + n_etc + n_k + 2 * n_em, m->em3, n_em);
  memcpy(h + n_etc + n_k + 3 * n_em, m->band, (size_t)nzp);
  CG_CUDA(cudaMemcpyAsync(w->model_dev, w->model_host, w->model_bytes, cudaMemcpyHostToDevice, st));
  CG_CUDA(cudaEventRecord(w->model_copied, st));
  w->wnc = m->wnc;
  w->is4d = m->is4d;
  w->cond_threshold = m->cond_threshold > 0 ? m->cond_threshold : 1.0e3;
  for (int t = 0; t < nt * nt; t++) w->etc_host[t] = m->err_theta_cov[t];
  for (int t = 0; t < 9; t++) { w->sigma0[t] = m->sigma0[t]; w->sigma0f[t] = (float)m->sigma0[t]; }
  long nb = 0;
  for (int k = 0; k < nzp; k++) nb += m->band[k] ? 1 : 0;
  w->inband_bins = nb * (long)(w->nxp / 2 + 1) * w->nyp;
  // conjugate symmetry in k of everything the set-up kernel reads (K, errMult1..3, band): then it computes
  // planes 0..nzp/2 and mirrors them
  bool sym = true;
  for (int k = 1; k < nzp && sym; k++) {
    const int km = nzp - k;
    if (km <= k) break;
    sym = m->band[k] == m->band[km];
    const float *arrs[4] = {m->K, m->em1, m->em2, m->em3};
    const long per[4] = {(long)nt * 3, nt, nt, nt};
    for (int a = 0; a < 4 && sym; a++)
      for (long i = 0; i < per[a] && sym; i++) {
        const float *x = arrs[a] + 2 * ((long)k * per[a] + i), *y = arrs[a] + 2 * ((long)km * per[a] + i);
        sym = x[0] == y[0] && x[1] == -y[1];
      }
  }
  PrepArgs pa;
  pa.nt = nt;
  pa.nzp = nzp;
  pa.sym = sym ? 1 : 0;
  pa.wnc = m->wnc;
  pa.is4d = m->is4d;
  pa.K = w->K; pa.em1 = w->em1; pa.em2 = w->em2; pa.em3 = w->em3; pa.band = w->band; pa.etc = w->etc;
  // the prior the reference multiplies into the covariance cubes is float(priorVar0)
  for (int t = 0; t < 9; t++) pa.s0[t] = (double)(float)m->sigma0[t];
  pa.tf = w->ktab_f; pa.td = w->ktab_d; pa.ti = w->itab;
  {
    TraceScope ts("k_prep_model", st, 0.0);
    const int prc = launch_prep_model(pa, sym ? nzp / 2 + 1 : nzp, st);
    if (prc) return prc;
    CG_CHECK_LAUNCH("k_prep_model");
  }
  // The information form needs a 3D model with a positive error diagonal in every in-band plane
  // (D_l = wnc errThetaCov_ll (Re e3_l)^2, the product the set-up kernel forms) and an invertible prior.
  w->info_ok = false;
  if (!w->is4d) {
    bool pos = true;
    for (int k = 0; k < nzp && pos; k++) {
      if (!m->band[k]) continue;
      for (int l = 0; l < nt; l++) {
        const double e3 = (double)m->em3[2 * ((long)k * nt + l)];
        if (!((double)m->wnc * m->err_theta_cov[l * nt + l] * e3 * e3 > 0.0)) { pos = false; break; }
      }
    }
    // Sigma0^-1 (the float prior the tables use) by cofactors in double
    const double *a = pa.s0;
    const double det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
                       a[2] * (a[3] * a[7] - a[4] * a[6]);
    if (pos && det > 0.0) {
      const double i00 = (a[4] * a[8] - a[5] * a[7]) / det, i11 = (a[0] * a[8] - a[2] * a[6]) / det;
      const double i22 = (a[0] * a[4] - a[1] * a[3]) / det, i01 = -(a[1] * a[8] - a[2] * a[7]) / det;
      const double i02 = (a[1] * a[5] - a[2] * a[4]) / det, i12 = -(a[0] * a[5] - a[2] * a[3]) / det;
      const double inv6[6] = {i00, i11, i22, i01, i02, i12};
      for (int q = 0; q < 6; q++) w->sig0inv[q] = (float)inv6[q];
      w->info_ok = true;
    }
  }
  w->model_set = true;
  return CG_OK;
}

extern "C" int cg_workspace_set_model(cg_workspace w, const cg_model *m)
{
  const int rc = cg_workspace_set_model_async(w, m, nullptr);
  if (rc) return rc;
  CG_CUDA(cudaDeviceSynchronize());
  return CG_OK;
}

extern "C" int cg_workspace_reset_stats(cg_workspace w, void *stream)
{
  if (!w) { set_error("null workspace"); return CG_ERR_ARG; }
  CG_CUDA(cudaMemsetAsync(w->counters, 0, sizeof(int) * 4, (cudaStream_t)stream));
  return CG_OK;
}

extern "C" int cg_workspace_stats(cg_workspace w, int *flagged, int *failed, int *overflow)
{
  if (!w) { set_error("null workspace"); return CG_ERR_ARG; }
  int h[4];
  CG_CUDA(cudaDeviceSynchronize());
  CG_CUDA(cudaMemcpy(h, w->counters, sizeof(h), cudaMemcpyDeviceToHost));
  if (flagged) *flagged = h[0];
  if (failed) *failed = h[1];
  if (overflow) *overflow = h[2];
  return CG_OK;
}

extern "C" int cg_invert_bins_plain(cg_workspace w, float *const *data, float *const *mean, float *const *cov,
                                    const float *errcorr, void *stream)
{
  int rc = check_ws(w);
  if (rc) return rc;
  if (!data || !mean || !cov || !errcorr) { set_error("null buffer argument"); return CG_ERR_ARG; }
  const int nt = w->ntheta;
  PlainArgs a;
  memset(&a, 0, sizeof(a));
  for (int l = 0; l < nt; l++) { if (!data[l]) { set_error("null data[%d]", l); return CG_ERR_ARG; } a.data[l] = (float2 *)data[l]; }
  for (int p = 0; p < 3; p++) { if (!mean[p]) { set_error("null mean[%d]", p); return CG_ERR_ARG; } a.mean[p] = (float2 *)mean[p]; }
  for (int t = 0; t < 6; t++) { if (!cov[t]) { set_error("null cov[%d]", t); return CG_ERR_ARG; } a.cov[t] = (float2 *)cov[t]; }
  a.errcorr = (const float2 *)errcorr;
  a.K = w->K; a.em1 = w->em1; a.em2 = w->em2; a.em3 = w->em3; a.band = w->band;
  const double *etc = w->etc_host;
  for (int l = 0; l < nt; l++) {
    for (int m = 0; m < nt; m++) a.c0[l * nt + m] = (float)(0.5 * (1.0 - w->wnc) * etc[l * nt + m]);
    a.cw[l] = (float)(w->wnc * etc[l * nt + l]);
  }
  const int pq[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  for (int t = 0; t < 6; t++) a.sig0[t] = w->sigma0f[pq[t][0] * 3 + pq[t][1]];
  const int cnxp = w->nxp / 2 + 1;
  a.plane = cnxp * w->nyp;
  a.csize = (long)a.plane * w->nzp;
  a.is4d = w->is4d;
  a.counters = w->counters;
  const int threads = 128;
  const long blocks = (a.csize + threads - 1) / threads;
  const long outband = a.csize - w->inband_bins;
  TraceScope ts("k_invert_plain", (cudaStream_t)stream,
                8.0 * w->inband_bins * ((nt + 3 + 7) + (nt + 3 + 6)) + 8.0 * outband * 12);
  return dispatch_nt(nt, [&](auto NTc) -> int {
    constexpr int NT = decltype(NTc)::value;
    k_invert_plain<NT><<<(unsigned)blocks, threads, 0, (cudaStream_t)stream>>>(a);
    CG_CHECK_LAUNCH("k_invert_plain");
    return CG_OK;
  });
}

// zero-padded copies of the lateral correlation surface (nxp x nyp at the
// rnxp pitch, n1 = rnxp * nyp values) and of the temporal correlation (nzp
// values into the rnzp that follow), in one launch
__global__ void k_pad_prior(const float *__restrict__ corr_xy, const float *__restrict__ circ_t, float *cxy,
                            float *ct, int nxp, int nzp, int rnxp, long n1, long n)
{
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (i < n1) {
    const int x = (int)(i % rnxp);
    cxy[i] = x < nxp ? corr_xy[(i / rnxp) * nxp + x] : 0.0f;
  } else {
    const int z = (int)(i - n1);
    ct[z] = z < nzp ? circ_t[z] : 0.0f;
  }
}

// pad a real nxp x nyp surface into the FFTGrid layout and transform it
template <typename T>
static int prior_tables(Workspace *w, const float *corr_xy, const float *circ_corr_t, T *cxy, T *ct, cudaStream_t st)
{
  const int nxp = w->nxp, nyp = w->nyp, nzp = w->nzp;
  const int rnxp = 2 * (nxp / 2 + 1), rnzp = 2 * (nzp / 2 + 1);
  if (sizeof(T) == 4) {
    const long n1 = (long)rnxp * nyp, n2 = rnzp;
    k_pad_prior<<<ceil_div(n1 + n2, 256), 256, 0, st>>>(corr_xy, circ_corr_t, (float *)cxy, (float *)ct, nxp, nzp,
                                                        rnxp, n1, n1 + n2);
    CG_CHECK_LAUNCH("k_pad_prior");
  } else {
    // float -> double into the padded layout, row by row through the float staging buffers
    CG_CUDA(cudaMemsetAsync(w->cxy_f, 0, sizeof(float) * (size_t)rnxp * nyp, st));
    CG_CUDA(cudaMemcpy2DAsync(w->cxy_f, sizeof(float) * rnxp, corr_xy, sizeof(float) * nxp, sizeof(float) * nxp,
                              nyp, cudaMemcpyDeviceToDevice, st));
    CG_CUDA(cudaMemsetAsync(w->ct_f, 0, sizeof(float) * (size_t)rnzp, st));
    CG_CUDA(cudaMemcpyAsync(w->ct_f, circ_corr_t, sizeof(float) * nzp, cudaMemcpyDeviceToDevice, st));
    long n1 = (long)rnxp * nyp, n2 = rnzp;
    k_f2d<<<ceil_div(n1, 256), 256, 0, st>>>(w->cxy_f, (double *)cxy, n1);
    k_f2d<<<ceil_div(n2, 256), 256, 0, st>>>(w->ct_f, (double *)ct, n2);
    CG_CHECK_LAUNCH("k_f2d");
  }
  void *b1[1] = {cxy};
  int rc = fft3d<T>(b1, 1, nxp, nyp, 1, CG_COVARIANCE, true, st);
  if (rc) return rc;
  void *b2[1] = {ct};
  return fft3d<T>(b2, 1, nzp, 1, 1, CG_COVARIANCE, true, st);
}

extern "C" int cg_prior_spectra(cg_workspace w, const float *corr_xy, const float *circ_corr_t, int precision,
                                void *stream)
{
  int rc = check_ws(w);
  if (rc) return rc;
  if (!corr_xy || !circ_corr_t) { set_error("null correlation input"); return CG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  w->sl_on = w->sl_d_on = false;
  if (precision == CG_PREC_FP64) {
    rc = prior_tables<double>(w, corr_xy, circ_corr_t, w->cxy_d, w->ct_d, st);
    if (rc) return rc;
  }
  return prior_tables<float>(w, corr_xy, circ_corr_t, w->cxy_f, w->ct_f, st);
}

namespace cg {
// (|Re P|, |Re E|) of every bin: the prior scale and error eigenvalue the bin
// solve takes from the covariance and error-correlation spectra
// (SeismicParametersHolder::getParameterCovariance keeps |Re| of the
// covariance, src/seismicparametersholder.cpp:407-425); out may alias P
template <typename T>
__global__ void k_scale_table(const C2<T> *P, const C2<T> *E, C2<T> *out, long n)
{
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  const T re_p = P[b].x, re_e = E[b].x;
  if constexpr (sizeof(T) == 4) out[b] = mk<T>(fabsf(re_p), fabsf(re_e));
  else out[b] = mk<T>(fabs(re_p), fabs(re_e));
}
}  // namespace cg

extern "C" int cg_prior_spectra_grad(cg_workspace w, const float *corr_xy, const float *circ_corr_t, float grad_i,
                                     float grad_j, int precision, void *stream)
{
  int rc = check_ws(w);
  if (rc) return rc;
  if (grad_i == 0.0f && grad_j == 0.0f) return cg_prior_spectra(w, corr_xy, circ_corr_t, precision, stream);
  if (!corr_xy || !circ_corr_t) { set_error("null correlation input"); return CG_ERR_ARG; }
  if (!(std::isfinite(grad_i) && std::isfinite(grad_j))) { set_error("correlation gradients must be finite"); return CG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  const int nxp = w->nxp, nyp = w->nyp, nzp = w->nzp;
  const long csize = (long)(nxp / 2 + 1) * nyp * nzp;  // bins; a real cube is the same bytes as csize float2
  w->sl_on = w->sl_d_on = false;
  if (!w->sl_f) CG_CUDA(dev_malloc((void **)&w->sl_f, sizeof(float2) * csize));
  if (precision == CG_PREC_FP64 && !w->sl_d) CG_CUDA(dev_malloc((void **)&w->sl_d, sizeof(double2) * csize));
  float *P = (float *)w->sl_f, *E = nullptr;
  CG_CUDA(scratch_alloc((void **)&E, sizeof(float2) * csize, st));
  // the parameter-correlation cube (fillInParamCorr, unit scalar) in the table's own memory and the
  // error-correlation cube (fillInErrCorr) beside it, both transformed as FFTCovGrids transforms covariances
  rc = fill_param_corr<float>(P, nxp, nyp, nzp, corr_xy, circ_corr_t, grad_i, grad_j, 1.0f, st);
  if (!rc) rc = fill_err_corr<float>(E, nxp, nyp, nzp, corr_xy, grad_i, grad_j, st);
  if (!rc) {
    void *b[2] = {P, E};
    rc = fft3d<float>(b, 2, nxp, nyp, nzp, CG_COVARIANCE, true, st);
  }
  if (!rc) {
    TraceScope ts("k_scale_table", st, 24.0 * csize);
    k_scale_table<float><<<(unsigned)ceil_div(csize, 256), 256, 0, st>>>((const float2 *)P, (const float2 *)E,
                                                                         (float2 *)P, csize);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_status(e, "k_scale_table");
  }
  if (!rc && precision == CG_PREC_FP64) {
    // the same cubes filled and transformed in FP64
    double *Pd = (double *)w->sl_d, *Ed = nullptr;
    cudaError_t e = scratch_alloc((void **)&Ed, sizeof(double2) * csize, st);
    if (e == cudaSuccess) {
      rc = fill_param_corr<double>(Pd, nxp, nyp, nzp, corr_xy, circ_corr_t, grad_i, grad_j, 1.0, st);
      if (!rc) rc = fill_err_corr<double>(Ed, nxp, nyp, nzp, corr_xy, grad_i, grad_j, st);
      if (!rc) {
        void *b[2] = {Pd, Ed};
        rc = fft3d<double>(b, 2, nxp, nyp, nzp, CG_COVARIANCE, true, st);
      }
      if (!rc) k_scale_table<double><<<(unsigned)ceil_div(csize, 256), 256, 0, st>>>((const double2 *)Pd,
                                                                                     (const double2 *)Ed,
                                                                                     (double2 *)Pd, csize);
      e = cudaGetLastError();
      cudaFreeAsync(Ed, st);
    }
    if (!rc && e != cudaSuccess) rc = cuda_status(e, "FP64 scale table");
  }
  cudaFreeAsync(E, st);
  if (rc) return rc;
  w->sl_on = true;
  w->sl_d_on = precision == CG_PREC_FP64;
  return CG_OK;
}

// Occupancy variant of the FP32 fused kernels (tuning key CG_TUNE_BIN_MINB).
// Measured at 256^3 with five stacks, capping registers for 6 resident CTAs
// (85 registers) is 1.34x faster than the unconstrained build despite a small
// spill; with six or more stacks the cap spills heavily, so those default to
// the unconstrained build.
static int bin_minb(int ntheta) { return cg_tune_get(CG_TUNE_BIN_MINB, ntheta); }

namespace cg {
template <typename T>
int fill_fused_args(Workspace *w, void *const *data, void *const *mean, void *const *cov, FusedArgs<T> *out)
{
  FusedArgs<T> &a = *out;
  memset(&a, 0, sizeof(a));
  for (int l = 0; l < w->ntheta; l++) { if (!data[l]) { set_error("null data[%d]", l); return CG_ERR_ARG; } a.data[l] = (C2<T> *)data[l]; }
  for (int p = 0; p < 3; p++) { if (!mean[p]) { set_error("null mean[%d]", p); return CG_ERR_ARG; } a.mean[p] = (C2<T> *)mean[p]; }
  for (int t = 0; t < 6; t++) { if (!cov[t]) { set_error("null cov[%d]", t); return CG_ERR_ARG; } a.cov[t] = (C2<T> *)cov[t]; }
  a.cxy = (const float2 *)w->cxy_f;
  a.ct = (const float2 *)w->ct_f;
  a.cxy_d = (const double2 *)w->cxy_d;
  a.ct_d = (const double2 *)w->ct_d;
  a.sl = w->sl_on ? (const float2 *)w->sl_f : nullptr;
  a.sl_d = w->sl_on && w->sl_d_on ? (const double2 *)w->sl_d : nullptr;
  a.ktab = (const KTab<T> *)(sizeof(T) == 8 ? (const void *)w->ktab_d : (const void *)w->ktab_f);
  const int pq[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  for (int t = 0; t < 6; t++) a.sig0[t] = (T)w->sigma0f[pq[t][0] * 3 + pq[t][1]];
  a.cnxp = w->nxp / 2 + 1;
  a.nyp = w->nyp;
  a.nzp = w->nzp;
  a.plane = a.cnxp * w->nyp;
  a.cond_thr = (float)w->cond_threshold;
  a.queue = w->queue;
  a.queue_cap = w->queue_cap;
  a.counters = w->counters;
  a.k0 = 0;
  a.chunked = 0;
  return CG_OK;
}
template int fill_fused_args<float>(Workspace *, void *const *, void *const *, void *const *, FusedArgs<float> *);
template int fill_fused_args<double>(Workspace *, void *const *, void *const *, void *const *, FusedArgs<double> *);
}  // namespace cg

// bin runs per CTA: up to kInfoBlocks while the grid of `threads`-thread CTAs
// over nk planes keeps about four waves of 768 threads per SM
static int bin_runs(const Workspace *w, long plane, int threads, int nk)
{
  const int forced = cg_tune_get(CG_TUNE_BIN_RUNS, w->ntheta);
  if (forced > 0) return forced < kInfoBlocks ? forced : kInfoBlocks;
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, w->device);
  const long runs = (long)ceil_div(plane, threads) * nk;
  const long want = 4L * (nsm > 0 ? nsm : 1) * (768 / threads);
  return (int)(runs / want < 1 ? 1 : runs / want > kInfoBlocks ? kInfoBlocks : runs / want);
}

// the information form (CG_TUNE_BIN_FORM 1) when the model has its tables
static bool use_info(const Workspace *w, int nt) { return w->info_ok && cg_tune_get(CG_TUNE_BIN_FORM, nt) == 1; }

template <int NT, int MODE>
static void launch_info(const FusedArgs<float> &a, const Workspace *w, dim3 grid, int threads, cudaStream_t st)
{
  InfoArgs ia;
  for (int q = 0; q < 6; q++) ia.s0i[q] = w->sig0inv[q];
  const int mb = cg_tune_get(CG_TUNE_BIN_MINB, NT);
  threads = info_threads(mb == 6 || mb == 5 ? mb : 4);
  if (a.sl) threads = info_threads(4);  // the per-bin prior table has one build
  const int nruns = bin_runs(w, a.plane, threads, (int)grid.y);
  grid.x = ceil_div(a.plane, (long)threads * nruns);
  if (a.sl) k_invert_info<NT, MODE, 4, true><<<grid, threads, 0, st>>>(a, w->itab, ia, nruns);
  else if (mb == 6) k_invert_info<NT, MODE, 6><<<grid, threads, 0, st>>>(a, w->itab, ia, nruns);
  else if (mb == 5) k_invert_info<NT, MODE, 5><<<grid, threads, 0, st>>>(a, w->itab, ia, nruns);
  else k_invert_info<NT, MODE, 4><<<grid, threads, 0, st>>>(a, w->itab, ia, nruns);
}

template <typename T>
static int fused_launch(Workspace *w, void *const *data, void *const *mean, void *const *cov, int precision,
                        cudaStream_t st, int k0 = 0, int nk = -1, bool chunked = false)
{
  const int nt = w->ntheta;
  FusedArgs<T> a;
  int rc = fill_fused_args(w, data, mean, cov, &a);
  if (rc) return rc;
  if (nk < 0) nk = w->nzp;
  if (k0 < 0 || nk < 1 || k0 + nk > w->nzp) { set_error("z-plane range %d + %d outside 0..%d", k0, nk, w->nzp); return CG_ERR_ARG; }
  a.k0 = k0;
  a.chunked = chunked ? 1 : 0;
  const int pq[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  const int threads = 128;
  dim3 grid(ceil_div(a.plane, threads), nk);
  const int fruns = bin_runs(w, a.plane, threads, nk);  // Cholesky-form kernel: runs per CTA
  const dim3 fgrid(ceil_div(a.plane, (long)threads * fruns), nk);
  const long outband = (long)a.plane * w->nzp - w->inband_bins;
  const double fbytes = (double)sizeof(C2<T>) * (w->inband_bins * (double)((nt + 3) + (nt + 3 + 6)) + outband * 6.0) *
                        ((double)nk / w->nzp);
  return dispatch_nt(nt, [&](auto NTc) -> int {
    constexpr int NT = decltype(NTc)::value;
    if constexpr (sizeof(T) == 8) {
      TraceScope ts("k_invert_fused_fp64", st, fbytes);
      if (a.sl) k_invert_fused<T, NT, 2, 1, true><<<fgrid, threads, 0, st>>>(a, fruns);
      else k_invert_fused<T, NT, 2><<<fgrid, threads, 0, st>>>(a, fruns);
    } else if (precision == CG_PREC_MIXED) {
      // the queue position counter starts at zero for every inversion (stream ordered); a z-chunk of a
      // chunked inversion appends to the queue and its fix-up starts where the chunk's entries start
      cudaError_t me = chunked ? cudaMemcpyAsync(w->counters + 3, w->counters, sizeof(int), cudaMemcpyDeviceToDevice, st)
                               : cudaMemsetAsync(w->counters, 0, sizeof(int), st);
      if (me != cudaSuccess) return cuda_status(me, "queue reset");
      if (use_info(w, NT)) {
        TraceScope ts("k_invert_info_mixed", st, fbytes);
        launch_info<NT, 1>(a, w, grid, threads, st);
      } else {
        TraceScope ts("k_invert_fused_mixed", st, fbytes);
        if (a.sl) k_invert_fused<T, NT, 1, 1, true><<<fgrid, threads, 0, st>>>(a, fruns);
        else if (bin_minb(NT) == 6) k_invert_fused<T, NT, 1, 6><<<fgrid, threads, 0, st>>>(a, fruns);
        else if (bin_minb(NT) == 5) k_invert_fused<T, NT, 1, 5><<<fgrid, threads, 0, st>>>(a, fruns);
        else if (bin_minb(NT) == 4) k_invert_fused<T, NT, 1, 4><<<fgrid, threads, 0, st>>>(a, fruns);
        else k_invert_fused<T, NT, 1, 1><<<fgrid, threads, 0, st>>>(a, fruns);
      }
      CG_CHECK_LAUNCH("k_invert_fused");
      S0Args sd;
      for (int t = 0; t < 6; t++) sd.v[t] = (double)w->sigma0f[pq[t][0] * 3 + pq[t][1]];
      FusedArgs<float> af;
      memcpy(&af, &a, sizeof(af));
      int nsm = 0;
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, w->device);
      // grid-stride over the queue: one CTA per 8192 bins of the launch, at most four per SM, so that a small
      // cube's (usually empty) fix-up does not hold hundreds of CTA slots beside other cubes' kernels
      const int fix_ctas = (int)std::min<long>((long)nsm * 4, std::max<long>(1, (long)a.plane * nk / 8192));
      TraceScope ts("k_invert_fixup64", st, 0.0);
      if (af.sl) k_invert_fixup64<NT, true><<<fix_ctas, 128, 0, st>>>(af, w->ktab_d, sd);
      else k_invert_fixup64<NT><<<fix_ctas, 128, 0, st>>>(af, w->ktab_d, sd);
    } else if (use_info(w, NT)) {
      TraceScope ts("k_invert_info_fp32", st, fbytes);
      launch_info<NT, 0>(a, w, grid, threads, st);
    } else {
      TraceScope ts("k_invert_fused_fp32", st, fbytes);
      // the FP32 mode spills more than MIXED under the 85-register cap (228 B against 128 B at five
      // stacks; 0.47 against 0.39 ms at 256^3): its tight setting is the 128-register build
      if (a.sl) k_invert_fused<T, NT, 0, 1, true><<<fgrid, threads, 0, st>>>(a, fruns);
      else if (bin_minb(NT) == 6 || bin_minb(NT) == 4) k_invert_fused<T, NT, 0, 4><<<fgrid, threads, 0, st>>>(a, fruns);
      else if (bin_minb(NT) == 5) k_invert_fused<T, NT, 0, 5><<<fgrid, threads, 0, st>>>(a, fruns);
      else k_invert_fused<T, NT, 0, 1><<<fgrid, threads, 0, st>>>(a, fruns);
    }
    CG_CHECK_LAUNCH("k_invert_fused");
    return CG_OK;
  });
}

int cg::fused_bins_range(Workspace *w, void *const *data, void *const *mean, void *const *cov, int precision, int k0,
                         int nk, bool chunked, cudaStream_t st)
{
  return fused_launch<float>(w, data, mean, cov, precision, st, k0, nk, chunked);
}

extern "C" int cg_invert_bins_fused(cg_workspace w, float *const *data, float *const *mean, float *const *cov,
                                    int precision, void *stream)
{
  int rc = check_ws(w);
  if (rc) return rc;
  if (!data || !mean || !cov) { set_error("null buffer argument"); return CG_ERR_ARG; }
  if (w->is4d) { set_error("the fused form needs a separable 3-parameter prior; use cg_invert_bins_plain for 4D"); return CG_ERR_UNSUPPORTED; }
  if (precision != CG_PREC_FP32 && precision != CG_PREC_MIXED) { set_error("precision %d not valid for FP32 buffers", precision); return CG_ERR_ARG; }
  return fused_launch<float>(w, (void *const *)data, (void *const *)mean, (void *const *)cov, precision,
                             (cudaStream_t)stream);
}

extern "C" int cg_invert_bins_fused_f64(cg_workspace w, double *const *data, double *const *mean,
                                        double *const *cov, void *stream)
{
  int rc = check_ws(w);
  if (rc) return rc;
  if (!data || !mean || !cov) { set_error("null buffer argument"); return CG_ERR_ARG; }
  if (w->is4d) { set_error("the fused form needs a separable 3-parameter prior"); return CG_ERR_UNSUPPORTED; }
  return fused_launch<double>(w, (void *const *)data, (void *const *)mean, (void *const *)cov, CG_PREC_FP64,
                              (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// Condition estimates of the in-band bins (diagnostic)
// ---------------------------------------------------------------------------
namespace cg {

// One thread per bin of plane blockIdx.y.  hist[0 .. nb-1]: FP64 Cholesky of
// Sd = s M + lam E + D (the Cholesky form's guard estimate: squared ratio of
// the largest to the smallest pivot), hist[nb .. 2nb-1]: the 3 x 3
// information-form matrix in FP32, computed as the default kernel's guard
// does.  Bucket floor(log10(cond)) clamped to 0 .. nb-2; bucket nb-1 counts
// failed factorisations.
template <int NT>
__global__ void __launch_bounds__(128) k_cond_hist(const float2 *__restrict__ cxy, const float2 *__restrict__ ct,
                                                   const float2 *__restrict__ sl,
                                                   const KTab<double> *__restrict__ ktd, const ITab *__restrict__ itab,
                                                   InfoArgs ia, int plane, int nzp, bool info,
                                                   unsigned long long *hist, int nb)
{
  __shared__ unsigned int h[2 * kCondBucketsMax];
  for (int i = threadIdx.x; i < 2 * nb; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const int k = blockIdx.y;
  const int ij = blockIdx.x * blockDim.x + threadIdx.x;
  const KTab<double> &kt = ktd[k];
  if (ij < plane && kt.band) {
    const int cnzp = nzp / 2 + 1;
    float sf, lamf;
    if (sl) {
      const float2 v = sl[(long)k * plane + ij];
      sf = v.x;
      lamf = v.y;
    } else {
      const float2 cx = cxy[ij];
      const float2 t = k < cnzp ? ct[k] : make_float2(ct[nzp - k].x, -ct[nzp - k].y);
      sf = fabsf(cx.x * t.x - cx.y * t.y);
      lamf = fabsf(cx.x);
    }
    {
      double2 L[NT * (NT + 1) / 2];
      double inv[NT], cond = 0.0;
      build_sd<double, NT>(kt, (double)sf, (double)lamf, L);
      const bool ok = chol_std<double, NT>(L, inv, cond);
      const int b = ok ? min(max((int)floor(log10(cond)), 0), nb - 2) : nb - 1;
      atomicAdd(&h[b], 1u);
    }
    if (info && sf > 0.0f) {
      const ITab &it = itab[k];
      const float is = 1.0f / sf;
      float q00 = ia.s0i[0] * is, q11 = ia.s0i[1] * is, q22 = ia.s0i[2] * is;
      float2 q01 = make_float2(ia.s0i[3] * is, 0.0f), q02 = make_float2(ia.s0i[4] * is, 0.0f),
             q12 = make_float2(ia.s0i[5] * is, 0.0f);
#pragma unroll
      for (int m = 0; m < NT; m++) {
        const float w = 1.0f / (lamf * it.mu[m] + 1.0f);
        const float *P = it.P[m];
        q00 += w * P[0]; q11 += w * P[1]; q22 += w * P[2];
        q01.x += w * P[3]; q01.y += w * P[4];
        q02.x += w * P[5]; q02.y += w * P[6];
        q12.x += w * P[7]; q12.y += w * P[8];
      }
      bool ok = q00 > 0.0f;
      const float r0 = rsqrtf(q00), l00 = q00 * r0;
      const float2 l10 = make_float2(q01.x * r0, -q01.y * r0), l20 = make_float2(q02.x * r0, -q02.y * r0);
      const float p1 = q11 - (l10.x * l10.x + l10.y * l10.y);
      ok = ok && p1 > 0.0f;
      const float r1 = rsqrtf(p1), l11 = p1 * r1;
      const float2 t21 = csub<float>(make_float2(q12.x, -q12.y), cmulc<float>(l20, l10));
      const float2 l21 = make_float2(t21.x * r1, t21.y * r1);
      const float p2 = q22 - (l20.x * l20.x + l20.y * l20.y) - (l21.x * l21.x + l21.y * l21.y);
      ok = ok && p2 > 0.0f;
      const float l22 = p2 * rsqrtf(p2);
      const float dmax = fmaxf(l00, fmaxf(l11, l22)), dmin = fminf(l00, fminf(l11, l22));
      const float cond = (dmax / dmin) * (dmax / dmin);
      const int b = ok ? min(max((int)floorf(log10f(cond)), 0), nb - 2) : nb - 1;
      atomicAdd(&h[nb + b], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * nb; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], (unsigned long long)h[i]);
}

}  // namespace cg

extern "C" int cg_condition_histogram(cg_workspace w, unsigned long long *hist_chol, unsigned long long *hist_info,
                                      int nbuckets, void *stream)
{
  int rc = check_ws(w);
  if (rc) return rc;
  if (!hist_chol || !hist_info) { set_error("null histogram"); return CG_ERR_ARG; }
  if (nbuckets < 2 || nbuckets > kCondBucketsMax) { set_error("nbuckets %d outside 2..%d", nbuckets, kCondBucketsMax); return CG_ERR_ARG; }
  if (w->is4d) { set_error("the condition histogram covers the fused form's 3D model"); return CG_ERR_UNSUPPORTED; }
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long *d = nullptr;
  CG_CUDA(scratch_alloc((void **)&d, sizeof(unsigned long long) * 2 * nbuckets, st));
  cudaError_t e = cudaMemsetAsync(d, 0, sizeof(unsigned long long) * 2 * nbuckets, st);
  InfoArgs ia;
  for (int q = 0; q < 6; q++) ia.s0i[q] = w->sig0inv[q];
  const int plane = (w->nxp / 2 + 1) * w->nyp;
  const dim3 grid(ceil_div(plane, 128), w->nzp);
  if (e == cudaSuccess) {
    rc = dispatch_nt(w->ntheta, [&](auto NTc) -> int {
      constexpr int NT = decltype(NTc)::value;
      k_cond_hist<NT><<<grid, 128, 0, st>>>((const float2 *)w->cxy_f, (const float2 *)w->ct_f,
                                            w->sl_on ? (const float2 *)w->sl_f : nullptr, w->ktab_d, w->itab,
                                            ia, plane, w->nzp, w->info_ok, d, nbuckets);
      return CG_OK;
    });
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(hist_chol, d, sizeof(unsigned long long) * nbuckets, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(hist_info, d + nbuckets, sizeof(unsigned long long) * nbuckets, cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "cg_condition_histogram");
  return rc;
}
