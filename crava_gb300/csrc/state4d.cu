// 4D time-lapse state: fold of the 6-parameter (static + dynamic) prior to
// the 3-parameter current state, and the Gaussian conditional split of the
// current-state posterior back to 6 parameters -- State4D::merge / mergeCov /
// split (src/state4d.cpp:140-580), one thread per frequency bin, in the
// reference's operation order (lib_matr.c products, Cholesky and solve).
//
// Grid layout of the 6x6 prior (upper triangle), as State4D keeps it:
//   ss[6]  static-static   (0,0)(0,1)(0,2)(1,1)(1,2)(2,2)
//   sd[9]  static-dynamic  (0,3)(0,4)(0,5)(1,3)(1,4)(1,5)(2,3)(2,4)(2,5)
//   dd[6]  dynamic-dynamic (3,3)(3,4)(3,5)(4,4)(4,5)(5,5)
// current-state covariance order: 00 01 02 11 12 22 (the sigma[] vector of
// State4D::mergeCov).
#include <cstring>

#include "common.cuh"
#include "linalg.cuh"
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

// (row, column) of stored entry t of each block as compile-time functions: in
// unrolled loops they fold to constants, so the 6x6 matrices stay in registers
// (a table in memory would force them to local memory)
__host__ __device__ constexpr int tri_r(int t) { return t < 3 ? 0 : t < 5 ? 1 : 2; }   // 00 01 02 11 12 22
__host__ __device__ constexpr int tri_c(int t) { return t < 3 ? t : t < 5 ? t - 2 : 2; }
__host__ __device__ constexpr int sd_r(int t) { return t / 3; }                        // (0,3) (0,4) ... (2,5)
__host__ __device__ constexpr int sd_c(int t) { return 3 + t % 3; }

__device__ __forceinline__ void load_full6(const S4Args &a, long b, float2 (*F)[6])
{
#pragma unroll
  for (int t = 0; t < 6; t++) F[tri_r(t)][tri_c(t)] = a.ss[t][b];
#pragma unroll
  for (int t = 0; t < 9; t++) F[sd_r(t)][sd_c(t)] = a.sd[t][b];
#pragma unroll
  for (int t = 0; t < 6; t++) F[3 + tri_r(t)][3 + tri_c(t)] = a.dd[t][b];
#pragma unroll
  for (int l = 0; l < 6; l++)
#pragma unroll
    for (int m = l + 1; m < 6; m++) F[m][l] = make_float2(F[l][m].x, -F[l][m].y);
}

__global__ void k_state4d_merge(S4Args a)
{
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.csize) return;
#pragma unroll
  for (int l = 0; l < 3; l++) {
    const float2 s = a.mu_s[l][b], d = a.mu_d[l][b];
    a.mu_cur[l][b] = make_float2(s.x + d.x, s.y + d.y);
  }
  float2 F[6][6];
  load_full6(a, b, F);
#pragma unroll
  for (int t = 0; t < 6; t++) {
    const int l = tri_r(t), m = tri_c(t);
    float re = F[l][m].x;
    re += F[l + 3][m + 3].x;
    re += F[l + 3][m].x;
    re += F[l][m + 3].x;
    float im = F[l][m].y;
    im += F[l + 3][m + 3].y;
    im += F[l + 3][m].y;
    im += F[l][m + 3].y;
    a.cov_cur[t][b] = make_float2(re, im);
  }
}

__global__ void __launch_bounds__(128, 3) k_state4d_split(S4Args a)
{
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.csize) return;
  float2 F[6][6];
  load_full6(a, b, F);
  float2 muF[6], muCpost[3], muC[3];
#pragma unroll
  for (int l = 0; l < 3; l++) { muF[l] = a.mu_s[l][b]; muF[l + 3] = a.mu_d[l][b]; muCpost[l] = a.mu_cur[l][b]; }
  float2 Cpost[3][3];
  Cpost[0][0] = a.cov_cur[0][b]; Cpost[0][1] = a.cov_cur[1][b]; Cpost[0][2] = a.cov_cur[2][b];
  Cpost[1][1] = a.cov_cur[3][b]; Cpost[1][2] = a.cov_cur[4][b]; Cpost[2][2] = a.cov_cur[5][b];
  Cpost[1][0] = make_float2(Cpost[0][1].x, -Cpost[0][1].y);
  Cpost[2][0] = make_float2(Cpost[0][2].x, -Cpost[0][2].y);
  Cpost[2][1] = make_float2(Cpost[1][2].x, -Cpost[1][2].y);
#pragma unroll
  for (int l = 0; l < 3; l++) muC[l] = make_float2(muF[l].x + muF[l + 3].x, muF[l].y + muF[l + 3].y);
  float2 FvC[6][3];
#pragma unroll
  for (int l = 0; l < 6; l++)
#pragma unroll
    for (int m = 0; m < 3; m++) FvC[l][m] = make_float2(F[l][m].x + F[l][m + 3].x, F[l][m].y + F[l][m + 3].y);
  float2 Cp[3][3];
#pragma unroll
  for (int l = 0; l < 3; l++)
#pragma unroll
    for (int m = 0; m < 3; m++) Cp[l][m] = make_float2(FvC[l][m].x + FvC[l + 3][m].x, FvC[l][m].y + FvC[l + 3][m].y);
  float2 L[6];
#pragma unroll
  for (int l = 0; l < 3; l++)
#pragma unroll
    for (int m = 0; m <= l; m++) L[ltri(l, m)] = Cp[l][m];
  float2 sand[3][6];
#pragma unroll
  for (int i = 0; i < 6; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) sand[j][i] = make_float2(FvC[i][j].x, -FvC[i][j].y);
  float2 out[6][6], muFpost[6];
  if (chol_ref<float, 3>(L)) {
    axeqb_ref<float, 3, 6>(L, sand);
#pragma unroll
    for (int l = 0; l < 3; l++)
#pragma unroll
      for (int m = 0; m < 3; m++) { Cpost[l][m].x -= Cp[l][m].x; Cpost[l][m].y -= Cp[l][m].y; }
    float2 helper[3][6];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 6; j++) {
        float xr = 0, xi = 0;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          xr += Cpost[i][k].x * sand[k][j].x - Cpost[i][k].y * sand[k][j].y;
          xi += Cpost[i][k].y * sand[k][j].x + Cpost[i][k].x * sand[k][j].y;
        }
        helper[i][j] = make_float2(xr, xi);
      }
    // out = adjoint(sand) * helper + F (only the upper triangle is stored)
#pragma unroll
    for (int i = 0; i < 6; i++)
#pragma unroll
      for (int j = i; j < 6; j++) {
        float xr = 0, xi = 0;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          const float2 ad = make_float2(sand[k][i].x, -sand[k][i].y);
          xr += ad.x * helper[k][j].x - ad.y * helper[k][j].y;
          xi += ad.y * helper[k][j].x + ad.x * helper[k][j].y;
        }
        out[i][j] = make_float2(xr + F[i][j].x, xi + F[i][j].y);
      }
#pragma unroll
    for (int l = 0; l < 3; l++) { muCpost[l].x -= muC[l].x; muCpost[l].y -= muC[l].y; }
#pragma unroll
    for (int i = 0; i < 6; i++) {
      float xr = 0, xi = 0;
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const float2 ad = make_float2(sand[j][i].x, -sand[j][i].y);
        xr += ad.x * muCpost[j].x - ad.y * muCpost[j].y;
        xi += ad.y * muCpost[j].x + ad.x * muCpost[j].y;
      }
      muFpost[i] = make_float2(xr + muF[i].x, xi + muF[i].y);
    }
  } else {
#pragma unroll
    for (int i = 0; i < 6; i++)
#pragma unroll
      for (int j = i; j < 6; j++) out[i][j] = F[i][j];
#pragma unroll
    for (int i = 0; i < 6; i++) muFpost[i] = muF[i];
    if (a.nfail) atomicAdd(a.nfail, 1);
  }
#pragma unroll
  for (int t = 0; t < 6; t++) a.ss[t][b] = out[tri_r(t)][tri_c(t)];
#pragma unroll
  for (int t = 0; t < 9; t++) a.sd[t][b] = out[sd_r(t)][sd_c(t)];
#pragma unroll
  for (int t = 0; t < 6; t++) a.dd[t][b] = out[3 + tri_r(t)][3 + tri_c(t)];
#pragma unroll
  for (int l = 0; l < 3; l++) { a.mu_s[l][b] = muFpost[l]; a.mu_d[l][b] = muFpost[l + 3]; }
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
