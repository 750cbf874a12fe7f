// One vintage of the 4D time-lapse inversion in one pass over the bins.
//
// The reference updates the 6-parameter state (static and dynamic Vp, Vs, rho)
// vintage by vintage (src/doinversion.cpp:96-135, src/crava.cpp:1028-1040):
// State4D::merge folds it to the 3-parameter current state, the bin loop
// inverts the vintage's data with the 4D branch of findParameterVariances
// (src/seismicparametersholder.cpp:366-373), and State4D::split conditions
// the 6-parameter state on the current state's posterior.  Here one thread
// does all three for its bin: it reads the 21 prior spectra (twice, the
// second time from L1/L2), the 6 means, the data and the error correlation,
// and writes the updated state, the residuals and the current state's
// posterior mean (the vintage's output before its inverse transform).  With
// the FP32 reference-order arithmetic the result is bit for bit that of the
// three separate passes (the same device functions: plain_bin.cuh,
// state4d.cuh), at about half their HBM traffic.
//
// CG_PREC_MIXED flags a bin whose data-covariance Cholesky fails or whose
// pivot-ratio condition estimate exceeds the workspace threshold: the FP32
// pass leaves it untouched and queues it, and k_vintage4d_fix64 redoes its
// merge, solve and split in FP64 from the untouched inputs.  The MIXED FP32
// pass divides by reciprocal multiplication (one division per pivot instead
// of one per element: the reference-order IEEE divisions were about a third
// of the kernel's instructions), so unlike the FP32 form it is not bit for bit
// the three passes; the FP64 redo keeps the reference's operations.
#include <cstring>

#include "common.cuh"
#include "fused_bins.cuh"
#include "plain_bin.cuh"
#include "posterior.cuh"
#include "state4d.cuh"
#include "trace.cuh"

namespace cg {

struct V4Args {
  float2 *mu_s[3], *mu_d[3];
  float2 *ss[6], *sd[9], *dd[6];
  float2 *data[kMaxTheta];  // data spectra in, residual spectra out
  float2 *post_mean[3];     // out: the current state's posterior mean
  const float2 *errcorr;
  const float2 *K, *em1, *em2, *em3;
  const unsigned char *band;
  float c0[kMaxTheta * kMaxTheta];  // float(0.5*(1-wnc)*errThetaCov[l][m])
  float cw[kMaxTheta];              // float(wnc*errThetaCov[l][l])
  int plane;
  long csize;
  int *counters;  // [0] bins queued for FP64, [1] failed bin Cholesky, [2] queue overflow
  int *nsplit;    // bins whose split kept the prior
  int *queue;
  int queue_cap;
  float cond_thr;
};

template <typename T>
__device__ __forceinline__ T vabs(C2<T> v)
{
  if constexpr (sizeof(T) == 4) return sqrtf(v.x * v.x + v.y * v.y);
  else return sqrt(v.x * v.x + v.y * v.y);
}

// MODE 0: FP32; 1: FP32 with the FP64 guard (returns false for a queued bin, which is left untouched);
// 2: FP64
template <typename T, int NT, int MODE>
__device__ __forceinline__ bool vintage_bin(const V4Args &a, long b)
{
  const int k = (int)(b / a.plane);
  // State4D::merge: the current state's mean and covariance (merge order 00 01 02 11 12 22)
  C2<T> mu[3], c6m[6];
#pragma unroll
  for (int l = 0; l < 3; l++) {
    const float2 s = a.mu_s[l][b], d = a.mu_d[l][b];
    if constexpr (sizeof(T) == 4) mu[l] = make_float2(s.x + d.x, s.y + d.y);
    else mu[l] = mk<T>((T)s.x + (T)d.x, (T)s.y + (T)d.y);
  }
  {
    C2<T> F[6][6];
    load_full6<T>(a.ss, a.sd, a.dd, b, F);
    merge_cov<T>(F, c6m);
  }
  // findParameterVariances, 4D branch: |.| on the diagonal, off-diagonal entries as they are
  C2<T> S[3][3];
  S[0][0] = mk<T>(vabs<T>(c6m[0]), (T)0);
  S[1][1] = mk<T>(vabs<T>(c6m[3]), (T)0);
  S[2][2] = mk<T>(vabs<T>(c6m[5]), (T)0);
  S[0][1] = c6m[1]; S[1][0] = mk<T>(c6m[1].x, -c6m[1].y);
  S[0][2] = c6m[2]; S[2][0] = mk<T>(c6m[2].x, -c6m[2].y);
  S[1][2] = c6m[4]; S[2][1] = mk<T>(c6m[4].x, -c6m[4].y);
  C2<T> res[NT];
#pragma unroll
  for (int l = 0; l < NT; l++) {
    const float2 v = a.data[l][b];
    res[l] = mk<T>((T)v.x, (T)v.y);
  }
  if (a.band[k]) {
    const float2 ec = a.errcorr[b];
    T lam;
    if constexpr (sizeof(T) == 4) lam = sqrtf(ec.x * ec.x);
    else lam = sqrt((T)ec.x * (T)ec.x);
    T cond = (T)0;
    const bool ok = plain_solve<T, NT, MODE == 1>(a.K + (long)k * NT * 3, a.em1 + (long)k * NT, a.em2 + (long)k * NT,
                                       a.em3 + (long)k * NT, a.c0, a.cw, lam, S, mu, res, &cond);
    if (MODE == 1 && (!ok || cond > (T)a.cond_thr)) {
      const int pos = atomicAdd(&a.counters[0], 1);
      if (pos < a.queue_cap) {
        a.queue[pos] = (int)b;
        return false;
      }
      atomicAdd(&a.counters[2], 1);  // queue full: keep the FP32 answer
    }
    if (!ok) atomicAdd(&a.counters[1], 1);
  }
#pragma unroll
  for (int l = 0; l < NT; l++) a.data[l][b] = make_float2((float)res[l].x, (float)res[l].y);
#pragma unroll
  for (int p = 0; p < 3; p++) a.post_mean[p][b] = make_float2((float)mu[p].x, (float)mu[p].y);
  // State4D::split on the current state's posterior: S's upper triangle, its lower one by conjugation
  C2<T> Cpost[3][3];
  Cpost[0][0] = S[0][0]; Cpost[0][1] = S[0][1]; Cpost[0][2] = S[0][2];
  Cpost[1][1] = S[1][1]; Cpost[1][2] = S[1][2]; Cpost[2][2] = S[2][2];
  Cpost[1][0] = mk<T>(S[0][1].x, -S[0][1].y);
  Cpost[2][0] = mk<T>(S[0][2].x, -S[0][2].y);
  Cpost[2][1] = mk<T>(S[1][2].x, -S[1][2].y);
  C2<T> muF[6];
#pragma unroll
  for (int l = 0; l < 3; l++) {
    const float2 s = a.mu_s[l][b], d = a.mu_d[l][b];
    muF[l] = mk<T>((T)s.x, (T)s.y);
    muF[l + 3] = mk<T>((T)d.x, (T)d.y);
  }
  if (!split_bin<T, MODE == 1>(a.mu_s, a.mu_d, a.ss, a.sd, a.dd, b, muF, mu, Cpost) && a.nsplit) atomicAdd(a.nsplit, 1);
  return true;
}

template <int NT, int MODE>
__global__ void __launch_bounds__(128, 4) k_vintage4d(const __grid_constant__ V4Args a)
{
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.csize) return;
  vintage_bin<float, NT, MODE>(a, b);
}

// FP64 redo of the bins the MIXED pass queued (their inputs are untouched)
template <int NT>
__global__ void __launch_bounds__(128) k_vintage4d_fix64(const __grid_constant__ V4Args a)
{
  const int nq = min(*((volatile int *)&a.counters[0]), a.queue_cap);
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x)
    vintage_bin<double, NT, 2>(a, (long)a.queue[q]);
}

}  // namespace cg

using namespace cg;

extern "C" int cg_vintage4d(cg_workspace w, float *const *mu_s, float *const *mu_d, float *const *ss,
                            float *const *sd, float *const *dd, float *const *data, const float *errcorr,
                            float *const *post_mean, int precision, int *nsplit_dev, void *stream)
{
  int rc = check_ws(w);
  if (rc) return rc;
  if (!w->is4d) { set_error("cg_vintage4d needs a workspace whose model was set with is4d = 1"); return CG_ERR_STATE; }
  if (precision != CG_PREC_FP32 && precision != CG_PREC_MIXED) { set_error("precision %d not valid", precision); return CG_ERR_ARG; }
  if (!mu_s || !mu_d || !ss || !sd || !dd || !data || !errcorr || !post_mean) { set_error("null argument"); return CG_ERR_ARG; }
  const int nt = w->ntheta;
  V4Args a;
  memset(&a, 0, sizeof(a));
  for (int t = 0; t < 3; t++) {
    a.mu_s[t] = (float2 *)mu_s[t]; a.mu_d[t] = (float2 *)mu_d[t]; a.post_mean[t] = (float2 *)post_mean[t];
    if (!a.mu_s[t] || !a.mu_d[t] || !a.post_mean[t]) { set_error("null mean grid"); return CG_ERR_ARG; }
  }
  for (int t = 0; t < 6; t++) {
    a.ss[t] = (float2 *)ss[t]; a.dd[t] = (float2 *)dd[t];
    if (!a.ss[t] || !a.dd[t]) { set_error("null covariance grid"); return CG_ERR_ARG; }
  }
  for (int t = 0; t < 9; t++) {
    a.sd[t] = (float2 *)sd[t];
    if (!a.sd[t]) { set_error("null static-dynamic grid"); return CG_ERR_ARG; }
  }
  for (int l = 0; l < nt; l++) {
    a.data[l] = (float2 *)data[l];
    if (!a.data[l]) { set_error("null data[%d]", l); return CG_ERR_ARG; }
  }
  a.errcorr = (const float2 *)errcorr;
  a.K = w->K; a.em1 = w->em1; a.em2 = w->em2; a.em3 = w->em3; a.band = w->band;
  for (int l = 0; l < nt; l++) {
    for (int m = 0; m < nt; m++) a.c0[l * nt + m] = (float)(0.5 * (1.0 - w->wnc) * w->etc_host[l * nt + m]);
    a.cw[l] = (float)(w->wnc * w->etc_host[l * nt + l]);
  }
  a.plane = (w->nxp / 2 + 1) * w->nyp;
  a.csize = (long)a.plane * w->nzp;
  a.counters = w->counters;
  a.nsplit = nsplit_dev;
  a.queue = w->queue;
  a.queue_cap = w->queue_cap;
  a.cond_thr = (float)w->cond_threshold;
  cudaStream_t st = (cudaStream_t)stream;
  const int threads = 128;
  const unsigned blocks = (unsigned)((a.csize + threads - 1) / threads);
  // algorithmic bytes: 27 state spectra + n data + the error correlation in, 27 + n + 3 out
  const double bytes = 8.0 * (double)a.csize * ((27 + nt + 1) + (27 + nt + 3));
  if (precision == CG_PREC_MIXED) CG_CUDA(cudaMemsetAsync(w->counters, 0, sizeof(int), st));
  return dispatch_nt(nt, [&](auto NTc) -> int {
    constexpr int NT = decltype(NTc)::value;
    if (precision == CG_PREC_MIXED) {
      {
        TraceScope ts("k_vintage4d_mixed", st, bytes);
        k_vintage4d<NT, 1><<<blocks, threads, 0, st>>>(a);
      }
      CG_CHECK_LAUNCH("k_vintage4d");
      int nsm = 0;
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, w->device);
      TraceScope ts("k_vintage4d_fix64", st, 0.0);
      k_vintage4d_fix64<NT><<<nsm * 4, 128, 0, st>>>(a);
    } else {
      TraceScope ts("k_vintage4d_fp32", st, bytes);
      k_vintage4d<NT, 0><<<blocks, threads, 0, st>>>(a);
    }
    CG_CHECK_LAUNCH("k_vintage4d");
    return CG_OK;
  });
}
