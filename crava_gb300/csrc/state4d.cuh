// 4D time-lapse state arithmetic of one frequency bin, shared by the State4D
// kernels (state4d.cu) and the fused per-vintage kernel (vintage4d.cu):
// State4D::merge / mergeCov and State4D::split (src/state4d.cpp:140-580) in
// the reference's operation order (lib_matr.c products, Cholesky and solve).
// T = float is the reference's arithmetic, T = double the FP64 redo.
//
// Grid layout of the 6x6 prior (upper triangle), as State4D keeps it:
//   ss[6]  static-static   (0,0)(0,1)(0,2)(1,1)(1,2)(2,2)
//   sd[9]  static-dynamic  (0,3)(0,4)(0,5)(1,3)(1,4)(1,5)(2,3)(2,4)(2,5)
//   dd[6]  dynamic-dynamic (3,3)(3,4)(3,5)(4,4)(4,5)(5,5)
// current-state covariance order: 00 01 02 11 12 22 (the sigma[] vector of
// State4D::mergeCov).
#pragma once

#include "common.cuh"
#include "linalg.cuh"

namespace cg {

// (row, column) of stored entry t of each block as compile-time functions: in
// unrolled loops they fold to constants, so the 6x6 matrices stay in registers
// (a table in memory would force them to local memory)
__host__ __device__ constexpr int tri_r(int t) { return t < 3 ? 0 : t < 5 ? 1 : 2; }   // 00 01 02 11 12 22
__host__ __device__ constexpr int tri_c(int t) { return t < 3 ? t : t < 5 ? t - 2 : 2; }
__host__ __device__ constexpr int sd_r(int t) { return t / 3; }                        // (0,3) (0,4) ... (2,5)
__host__ __device__ constexpr int sd_c(int t) { return 3 + t % 3; }

// the full Hermitian 6x6 prior of bin b from the 21 stored spectra
template <typename T>
__device__ __forceinline__ void load_full6(float2 *const *ss, float2 *const *sd, float2 *const *dd, long b,
                                           C2<T> (*F)[6])
{
#pragma unroll
  for (int t = 0; t < 6; t++) { const float2 v = ss[t][b]; F[tri_r(t)][tri_c(t)] = mk<T>((T)v.x, (T)v.y); }
#pragma unroll
  for (int t = 0; t < 9; t++) { const float2 v = sd[t][b]; F[sd_r(t)][sd_c(t)] = mk<T>((T)v.x, (T)v.y); }
#pragma unroll
  for (int t = 0; t < 6; t++) { const float2 v = dd[t][b]; F[3 + tri_r(t)][3 + tri_c(t)] = mk<T>((T)v.x, (T)v.y); }
#pragma unroll
  for (int l = 0; l < 6; l++)
#pragma unroll
    for (int m = l + 1; m < 6; m++) F[m][l] = mk<T>(F[l][m].x, -F[l][m].y);
}

// State4D::mergeCov: the current state's covariance (merge order) from the full prior
template <typename T>
__device__ __forceinline__ void merge_cov(const C2<T> (*F)[6], C2<T> *cov6)
{
#pragma unroll
  for (int t = 0; t < 6; t++) {
    const int l = tri_r(t), m = tri_c(t);
    T re = F[l][m].x;
    re += F[l + 3][m + 3].x;
    re += F[l + 3][m].x;
    re += F[l][m + 3].x;
    T im = F[l][m].y;
    im += F[l + 3][m + 3].y;
    im += F[l + 3][m].y;
    im += F[l][m + 3].y;
    cov6[t] = mk<T>(re, im);
  }
}

// entry (i, j) of the full Hermitian 6x6 prior of bin b, read from the stored upper triangle (i, j
// compile-time after unrolling)
__host__ __device__ constexpr int tri_t(int i, int j) { return i * (5 - i) / 2 + j; }  // 00 01 02 11 12 22
template <typename T>
__device__ __forceinline__ C2<T> state_entry(float2 *const *ss, float2 *const *sd, float2 *const *dd, long b, int i,
                                             int j)
{
  const int r = i < j ? i : j, c = i < j ? j : i;
  const float2 v = c < 3 ? ss[tri_t(r, c)][b] : (r < 3 ? sd[r * 3 + c - 3][b] : dd[tri_t(r - 3, c - 3)][b]);
  return i <= j ? mk<T>((T)v.x, (T)v.y) : mk<T>((T)v.x, -(T)v.y);
}

// State4D::split of bin b, in place on the 27 stored spectra.  muF is the bin's full prior mean; muCpost,
// Cpost (Hermitian, all nine entries) the current state's posterior (both consumed).  The prior covariance
// F is read from the grids twice (for the sums F(:, m) + F(:, m+3) at the start and for the final
// F + sand^H * helper), so it is never held in registers as a whole; every posterior entry is stored as
// soon as it is formed.  Returns false when the Cholesky of the current prior fails: the grids then keep
// the prior, as the reference keeps it.
template <typename T, bool FAST = false>
__device__ __forceinline__ bool split_bin(float2 *const *mu_s, float2 *const *mu_d, float2 *const *ss,
                                          float2 *const *sd, float2 *const *dd, long b, const C2<T> *muF,
                                          C2<T> *muCpost, C2<T> (*Cpost)[3])
{
  C2<T> muC[3];
#pragma unroll
  for (int l = 0; l < 3; l++) muC[l] = mk<T>(muF[l].x + muF[l + 3].x, muF[l].y + muF[l + 3].y);
  C2<T> FvC[6][3];
#pragma unroll
  for (int l = 0; l < 6; l++)
#pragma unroll
    for (int m = 0; m < 3; m++) {
      const C2<T> a = state_entry<T>(ss, sd, dd, b, l, m), c = state_entry<T>(ss, sd, dd, b, l, m + 3);
      FvC[l][m] = mk<T>(a.x + c.x, a.y + c.y);
    }
  C2<T> Cp[3][3];
#pragma unroll
  for (int l = 0; l < 3; l++)
#pragma unroll
    for (int m = 0; m < 3; m++) Cp[l][m] = mk<T>(FvC[l][m].x + FvC[l + 3][m].x, FvC[l][m].y + FvC[l + 3][m].y);
  C2<T> L[6];
#pragma unroll
  for (int l = 0; l < 3; l++)
#pragma unroll
    for (int m = 0; m <= l; m++) L[ltri(l, m)] = Cp[l][m];
  C2<T> sand[3][6];
#pragma unroll
  for (int i = 0; i < 6; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) sand[j][i] = mk<T>(FvC[i][j].x, -FvC[i][j].y);
  if (!chol_ref<T, 3, FAST>(L)) return false;
  axeqb_ref<T, 3, 6, FAST>(L, sand);
#pragma unroll
  for (int l = 0; l < 3; l++)
#pragma unroll
    for (int m = 0; m < 3; m++) { Cpost[l][m].x -= Cp[l][m].x; Cpost[l][m].y -= Cp[l][m].y; }
  // F + adjoint(sand) * helper, helper = Cpost * sand, upper triangle; one column of helper at a time (the
  // sums keep their order), each entry stored as it is formed
#pragma unroll
  for (int j = 0; j < 6; j++) {
    C2<T> hj[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      T xr = 0, xi = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        xr += Cpost[i][k].x * sand[k][j].x - Cpost[i][k].y * sand[k][j].y;
        xi += Cpost[i][k].y * sand[k][j].x + Cpost[i][k].x * sand[k][j].y;
      }
      hj[i] = mk<T>(xr, xi);
    }
#pragma unroll
    for (int i = 0; i <= j; i++) {
      T xr = 0, xi = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const C2<T> ad = mk<T>(sand[k][i].x, -sand[k][i].y);
        xr += ad.x * hj[k].x - ad.y * hj[k].y;
        xi += ad.y * hj[k].x + ad.x * hj[k].y;
      }
      const C2<T> f = state_entry<T>(ss, sd, dd, b, i, j);
      const float2 o = make_float2((float)(xr + f.x), (float)(xi + f.y));
      if (j < 3) ss[tri_t(i, j)][b] = o;
      else if (i < 3) sd[i * 3 + j - 3][b] = o;
      else dd[tri_t(i - 3, j - 3)][b] = o;
    }
  }
#pragma unroll
  for (int l = 0; l < 3; l++) { muCpost[l].x -= muC[l].x; muCpost[l].y -= muC[l].y; }
#pragma unroll
  for (int i = 0; i < 6; i++) {
    T xr = 0, xi = 0;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const C2<T> ad = mk<T>(sand[j][i].x, -sand[j][i].y);
      xr += ad.x * muCpost[j].x - ad.y * muCpost[j].y;
      xi += ad.y * muCpost[j].x + ad.x * muCpost[j].y;
    }
    const float2 o = make_float2((float)(xr + muF[i].x), (float)(xi + muF[i].y));
    if (i < 3) mu_s[i][b] = o;
    else mu_d[i - 3][b] = o;
  }
  return true;
}

}  // namespace cg
