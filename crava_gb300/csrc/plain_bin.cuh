// The reference-order solve of one in-band bin (Crava::invertSeismicData with
// getNextErrorVariance, src/crava.cpp:1389-1469, lib_matr.c's products,
// Cholesky and triangular solves), shared by the plain bin kernel and the
// fused 4D vintage kernel.  T = float is the reference's arithmetic; T =
// double is the FP64 redo of guarded bins.
#pragma once

#include "common.cuh"
#include "linalg.cuh"
#include "posterior.cuh"

namespace cg {

// S (3x3 prior, all nine entries) in, posterior out; mu prior mean in,
// posterior mean out; res data in, residual out.  Kk, e1k, e2k, e3k: the
// plane's tables (NT x 3, NT, NT, NT); c0 = float(0.5 (1-wnc) errThetaCov),
// cw = float(wnc errThetaCov_ll); lam = |Re errCorr| of the bin.  Returns
// false when the Cholesky of the data covariance fails (S, mu and res are
// then left as they came in, as the reference keeps the prior); *cond
// receives the squared ratio of the largest to the smallest Cholesky pivot.
// FAST: reciprocal-multiply divisions (chol_ref); false keeps the reference's operations.
template <typename T, int NT, bool FAST = false>
__device__ __forceinline__ bool plain_solve(const float2 *__restrict__ Kk, const float2 *__restrict__ e1k,
                                            const float2 *__restrict__ e2k, const float2 *__restrict__ e3k,
                                            const float *c0t, const float *cwt, T lam, C2<T> (*S)[3], C2<T> *mu,
                                            C2<T> *res, T *cond)
{
  C2<T> d[NT], K[NT][3], KS[NT][3], KScc[3][NT], Sd[NT * (NT + 1) / 2];
#pragma unroll
  for (int l = 0; l < NT; l++) d[l] = res[l];
#pragma unroll
  for (int l = 0; l < NT; l++)
#pragma unroll
    for (int p = 0; p < 3; p++) {
      const float2 v = __ldg(&Kk[l * 3 + p]);
      K[l][p] = mk<T>((T)v.x, (T)v.y);
    }
  // KS = K S (lib_matrProdCpx)
#pragma unroll
  for (int l = 0; l < NT; l++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      T xr = 0, xi = 0;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        xr += K[l][q].x * S[q][j].x - K[l][q].y * S[q][j].y;
        xi += K[l][q].y * S[q][j].x + K[l][q].x * S[q][j].y;
      }
      KS[l][j] = mk<T>(xr, xi);
    }
  // Sd = KS K^H + errVar (lower triangle; lib_matrProdAdjointCpx + getNextErrorVariance)
#pragma unroll
  for (int l = 0; l < NT; l++) {
    const float2 e1l = __ldg(&e1k[l]);
    const float2 e2l = __ldg(&e2k[l]);
#pragma unroll
    for (int m = 0; m <= l; m++) {
      T xr = 0, xi = 0;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        xr += KS[l][q].x * K[m][q].x + KS[l][q].y * K[m][q].y;
        xi += KS[l][q].y * K[m][q].x - KS[l][q].x * K[m][q].y;
      }
      const float2 e1m = __ldg(&e1k[m]);
      const float2 e2m = __ldg(&e2k[m]);
      const T c0 = (T)c0t[l * NT + m] * lam;
      T er = c0 * ((T)e1l.x * (T)e1m.x + (T)e1l.y * (T)e1m.y);
      er += c0 * ((T)e2l.x * (T)e2m.x + (T)e2l.y * (T)e2m.y);
      T ei;
      if (l == m) {
        const float2 e3 = __ldg(&e3k[l]);
        er += (T)cwt[l] * (T)e3.x * (T)e3.x;
        ei = (T)0;
      } else {
        ei = c0 * (-(T)e1l.x * (T)e1m.y + (T)e1l.y * (T)e1m.x);
        ei += c0 * (-(T)e2l.x * (T)e2m.y + (T)e2l.y * (T)e2m.x);
      }
      Sd[tri(l, m)] = mk<T>(xr + er, xi + ei);
    }
  }
  if (!chol_ref<T, NT, FAST>(Sd)) return false;
  {
    T dmax = Sd[0].x, dmin = Sd[0].x;
#pragma unroll
    for (int i = 1; i < NT; i++) {
      dmax = Sd[tri(i, i)].x > dmax ? Sd[tri(i, i)].x : dmax;
      dmin = Sd[tri(i, i)].x < dmin ? Sd[tri(i, i)].x : dmin;
    }
    *cond = (dmax / dmin) * (dmax / dmin);
  }
#pragma unroll
  for (int l = 0; l < NT; l++)
#pragma unroll
    for (int p = 0; p < 3; p++) KScc[p][l] = mk<T>(KS[l][p].x, -KS[l][p].y);
  // lib_matrAXeqBMatCpx: KS <- Sd^-1 KS
  T rh[NT];
  if constexpr (FAST) diag_rcp<T, NT>(Sd, rh);
#pragma unroll
  for (int c = 0; c < 3; c++) {
#pragma unroll
    for (int i = 0; i < NT; i++) {
      T xr = KS[i][c].x, xi = KS[i][c].y;
#pragma unroll
      for (int j = 0; j < i; j++) {
        xr -= (KS[j][c].x * Sd[tri(i, j)].x - KS[j][c].y * Sd[tri(i, j)].y);
        xi -= (KS[j][c].y * Sd[tri(i, j)].x + KS[j][c].x * Sd[tri(i, j)].y);
      }
      const C2<T> lii = Sd[tri(i, i)];
      if constexpr (FAST) {
        KS[i][c] = mk<T>((xr * lii.x + xi * lii.y) * rh[i], (xi * lii.x - xr * lii.y) * rh[i]);
      } else {
        const T help = lii.x * lii.x + lii.y * lii.y;
        KS[i][c] = mk<T>((xr * lii.x + xi * lii.y) / help, (xi * lii.x - xr * lii.y) / help);
      }
    }
#pragma unroll
    for (int i = NT - 1; i >= 0; i--) {
      T xr = KS[i][c].x, xi = KS[i][c].y;
#pragma unroll
      for (int j = NT - 1; j > i; j--) {
        xr = xr - (KS[j][c].x * Sd[tri(j, i)].x + KS[j][c].y * Sd[tri(j, i)].y);
        xi = xi - (-KS[j][c].x * Sd[tri(j, i)].y + KS[j][c].y * Sd[tri(j, i)].x);
      }
      const C2<T> lii = Sd[tri(i, i)];
      if constexpr (FAST) {
        KS[i][c] = mk<T>((xr * lii.x - xi * lii.y) * rh[i], (xi * lii.x + xr * lii.y) * rh[i]);
      } else {
        const T help = lii.x * lii.x + lii.y * lii.y;
        KS[i][c] = mk<T>((xr * lii.x - xi * lii.y) / help, (xi * lii.x + xr * lii.y) / help);
      }
    }
  }
  // S -= KScc KS
#pragma unroll
  for (int p = 0; p < 3; p++)
#pragma unroll
    for (int q = 0; q < 3; q++) {
      T xr = 0, xi = 0;
#pragma unroll
      for (int l = 0; l < NT; l++) {
        xr += KScc[p][l].x * KS[l][q].x - KScc[p][l].y * KS[l][q].y;
        xi += KScc[p][l].y * KS[l][q].x + KScc[p][l].x * KS[l][q].y;
      }
      S[p][q].x -= xr;
      S[p][q].y -= xi;
    }
  // d -= K mu; ans = KS^H d; mu += ans; res -= K mu (K read again from the table, an L1 hit, so that it need
  // not stay in registers through the solve)
  auto kat = [&](int l, int p) -> C2<T> {
    const float2 v = __ldg(&Kk[l * 3 + p]);
    return mk<T>((T)v.x, (T)v.y);
  };
#pragma unroll
  for (int l = 0; l < NT; l++) {
    T xr = 0, xi = 0;
#pragma unroll
    for (int p = 0; p < 3; p++) {
      const C2<T> k = kat(l, p);
      xr += k.x * mu[p].x - k.y * mu[p].y;
      xi += k.y * mu[p].x + k.x * mu[p].y;
    }
    d[l].x -= xr;
    d[l].y -= xi;
  }
#pragma unroll
  for (int p = 0; p < 3; p++) {
    T xr = 0, xi = 0;
#pragma unroll
    for (int l = 0; l < NT; l++) {
      xr += KS[l][p].x * d[l].x + KS[l][p].y * d[l].y;
      xi += -KS[l][p].y * d[l].x + KS[l][p].x * d[l].y;
    }
    mu[p].x += xr;
    mu[p].y += xi;
  }
#pragma unroll
  for (int l = 0; l < NT; l++) {
    T xr = 0, xi = 0;
#pragma unroll
    for (int p = 0; p < 3; p++) {
      const C2<T> k = kat(l, p);
      xr += k.x * mu[p].x - k.y * mu[p].y;
      xi += k.y * mu[p].x + k.x * mu[p].y;
    }
    res[l].x -= xr;
    res[l].y -= xi;
  }
  return true;
}

}  // namespace cg
