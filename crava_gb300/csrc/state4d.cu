// 4D time-lapse state: fold of the 6-parameter (static + dynamic) prior to
// the 3-parameter current state, and the Gaussian conditional split of the
// current-state posterior back to 6 parameters -- State4D::merge / mergeCov /
// split (src/state4d.cpp:140-580), one thread per frequency bin; the per-bin
// arithmetic is in state4d.cuh.
#include <cstring>

#include "common.cuh"
#include "state4d.cuh"
#include "trace.cuh"

namespace cg {

struct S4Args {
  float2 *mu_s[3], *mu_d[3];
  float2 *ss[6], *sd[9], *dd[6];
  float2 *mu_cur[3];   // merge: out; split: posterior of the current state (in)
  float2 *cov_cur[6];  // merge: out; split: posterior of the current state (in)
  long csize;
  int *nfail;
};

__global__ void k_state4d_merge(const __grid_constant__ S4Args a)
{
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.csize) return;
#pragma unroll
  for (int l = 0; l < 3; l++) {
    const float2 s = a.mu_s[l][b], d = a.mu_d[l][b];
    a.mu_cur[l][b] = make_float2(s.x + d.x, s.y + d.y);
  }
  float2 F[6][6], c6[6];
  load_full6<float>(a.ss, a.sd, a.dd, b, F);
  merge_cov<float>(F, c6);
#pragma unroll
  for (int t = 0; t < 6; t++) a.cov_cur[t][b] = c6[t];
}

__global__ void __launch_bounds__(128, 4) k_state4d_split(const __grid_constant__ S4Args a)
{
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.csize) return;
  float2 muF[6], muCpost[3];
#pragma unroll
  for (int l = 0; l < 3; l++) { muF[l] = a.mu_s[l][b]; muF[l + 3] = a.mu_d[l][b]; muCpost[l] = a.mu_cur[l][b]; }
  float2 Cpost[3][3];
  Cpost[0][0] = a.cov_cur[0][b]; Cpost[0][1] = a.cov_cur[1][b]; Cpost[0][2] = a.cov_cur[2][b];
  Cpost[1][1] = a.cov_cur[3][b]; Cpost[1][2] = a.cov_cur[4][b]; Cpost[2][2] = a.cov_cur[5][b];
  Cpost[1][0] = make_float2(Cpost[0][1].x, -Cpost[0][1].y);
  Cpost[2][0] = make_float2(Cpost[0][2].x, -Cpost[0][2].y);
  Cpost[2][1] = make_float2(Cpost[1][2].x, -Cpost[1][2].y);
  if (!split_bin<float>(a.mu_s, a.mu_d, a.ss, a.sd, a.dd, b, muF, muCpost, Cpost) && a.nfail) atomicAdd(a.nfail, 1);
}

static int fill_args(S4Args &a, float *const *mu_s, float *const *mu_d, float *const *ss, float *const *sd,
                     float *const *dd, float *const *mu_cur, float *const *cov_cur, int nxp, int nyp, int nzp,
                     int *nfail)
{
  memset(&a, 0, sizeof(a));
  if (!mu_s || !mu_d || !ss || !sd || !dd || !mu_cur || !cov_cur || nxp < 1 || nyp < 1 || nzp < 1) {
    set_error("state4d: bad argument");
    return CG_ERR_ARG;
  }
  for (int t = 0; t < 3; t++) {
    a.mu_s[t] = (float2 *)mu_s[t]; a.mu_d[t] = (float2 *)mu_d[t]; a.mu_cur[t] = (float2 *)mu_cur[t];
    if (!a.mu_s[t] || !a.mu_d[t] || !a.mu_cur[t]) { set_error("state4d: null mean grid"); return CG_ERR_ARG; }
  }
  for (int t = 0; t < 6; t++) {
    a.ss[t] = (float2 *)ss[t]; a.dd[t] = (float2 *)dd[t]; a.cov_cur[t] = (float2 *)cov_cur[t];
    if (!a.ss[t] || !a.dd[t] || !a.cov_cur[t]) { set_error("state4d: null covariance grid"); return CG_ERR_ARG; }
  }
  for (int t = 0; t < 9; t++) {
    a.sd[t] = (float2 *)sd[t];
    if (!a.sd[t]) { set_error("state4d: null static-dynamic grid"); return CG_ERR_ARG; }
  }
  a.csize = (long)(nxp / 2 + 1) * nyp * nzp;
  a.nfail = nfail;
  return CG_OK;
}

}  // namespace cg

using namespace cg;

extern "C" int cg_state4d_merge(float *const *mu_s, float *const *mu_d, float *const *ss, float *const *sd,
                                float *const *dd, float *const *mu_cur, float *const *cov_cur, int nxp, int nyp,
                                int nzp, void *stream)
{
  S4Args a;
  int rc = fill_args(a, mu_s, mu_d, ss, sd, dd, mu_cur, cov_cur, nxp, nyp, nzp, nullptr);
  if (rc) return rc;
  TraceScope ts("k_state4d_merge", (cudaStream_t)stream, 8.0 * a.csize * (27 + 9));
  k_state4d_merge<<<ceil_div(a.csize, 128), 128, 0, (cudaStream_t)stream>>>(a);
  CG_CHECK_LAUNCH("k_state4d_merge");
  return CG_OK;
}

extern "C" int cg_state4d_split(float *const *mu_s, float *const *mu_d, float *const *ss, float *const *sd,
                                float *const *dd, float *const *mu_post, float *const *cov_post, int nxp, int nyp,
                                int nzp, int *nfail_dev, void *stream)
{
  S4Args a;
  int rc = fill_args(a, mu_s, mu_d, ss, sd, dd, mu_post, cov_post, nxp, nyp, nzp, nfail_dev);
  if (rc) return rc;
  TraceScope ts("k_state4d_split", (cudaStream_t)stream, 8.0 * a.csize * (27 + 9 + 27));
  k_state4d_split<<<ceil_div(a.csize, 128), 128, 0, (cudaStream_t)stream>>>(a);
  CG_CHECK_LAUNCH("k_state4d_split");
  return CG_OK;
}
