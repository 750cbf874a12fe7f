// Reference-order small complex linear algebra on packed lower triangles
// (libs/lib/lib_matr.c), shared by the per-bin kernels.
#pragma once

#include "common.cuh"

namespace cg {

constexpr double kLibMatrTol = 1e-20;  // lib_matr.c:19

__host__ __device__ constexpr int ltri(int l, int m) { return l * (l + 1) / 2 + m; }  // l >= m

// lib_matrCholCpx (libs/lib/lib_matr.c:78-168) on a packed lower triangle.
// FAST = false: the reference's operations, IEEE divisions included (bit for
// bit the reference in FP32).  FAST = true: the same steps with each divisor's
// reciprocal formed once and multiplied (one division per pivot instead of one
// per element; results differ from the reference by rounding only).
template <typename T, int N, bool FAST = false>
__device__ __forceinline__ bool chol_ref(C2<T> *L)
{
  const T factor = L[0].x;
  if (!(factor > (T)0)) return false;
  if constexpr (FAST) {
    const T rf = (T)1 / factor;
#pragma unroll
    for (int t = 0; t < N * (N + 1) / 2; t++) { L[t].x *= rf; L[t].y *= rf; }
  } else {
#pragma unroll
    for (int t = 0; t < N * (N + 1) / 2; t++) { L[t].x = L[t].x / factor; L[t].y = L[t].y / factor; }
  }
#pragma unroll
  for (int i = 0; i < N; i++) {
    if (L[ltri(i, i)].x <= (T)kLibMatrTol) return false;
#pragma unroll
    for (int j = 0; j < i; j++) {
      T lr = 0, li = 0;
#pragma unroll
      for (int k = 0; k < j; k++) {
        lr += (L[ltri(i, k)].x * L[ltri(j, k)].x) + (L[ltri(i, k)].y * L[ltri(j, k)].y);
        li += -(L[ltri(i, k)].x * L[ltri(j, k)].y) + (L[ltri(i, k)].y * L[ltri(j, k)].x);
      }
      const C2<T> ljj = L[ltri(j, j)];
      const T help = ljj.x * ljj.x + ljj.y * ljj.y;
      const C2<T> lij = L[ltri(i, j)];
      if constexpr (FAST) {
        const T rh = (T)1 / help;
        L[ltri(i, j)].x = ((lij.x - lr) * ljj.x + (lij.y - li) * ljj.y) * rh;
        L[ltri(i, j)].y = ((lij.y - li) * ljj.x - (lij.x - lr) * ljj.y) * rh;
      } else {
        L[ltri(i, j)].x = ((lij.x - lr) * ljj.x + (lij.y - li) * ljj.y) / help;
        L[ltri(i, j)].y = ((lij.y - li) * ljj.x - (lij.x - lr) * ljj.y) / help;
      }
    }
    T lr = 0;
#pragma unroll
    for (int k = 0; k < i; k++) lr += (L[ltri(i, k)].x * L[ltri(i, k)].x) + (L[ltri(i, k)].y * L[ltri(i, k)].y);
    lr = L[ltri(i, i)].x - lr;
    if (lr <= (T)kLibMatrTol) return false;
    L[ltri(i, i)] = mk<T>(sqrt(lr), (T)0);
  }
  const T sf = sqrt(factor);
#pragma unroll
  for (int t = 0; t < N * (N + 1) / 2; t++) { L[t].x *= sf; L[t].y *= sf; }
  return true;
}

// the reciprocals 1/|L_ii|^2 of a factor's diagonal (FAST solves)
template <typename T, int N>
__device__ __forceinline__ void diag_rcp(const C2<T> *L, T *r)
{
#pragma unroll
  for (int i = 0; i < N; i++) {
    const C2<T> lii = L[ltri(i, i)];
    r[i] = (T)1 / (lii.x * lii.x + lii.y * lii.y);
  }
}

// lib_matrAXeqBMatCpx (libs/lib/lib_matr.c:330-367): X <- (L L^H)^-1 X for the
// M columns of X (row-major N x M), L from chol_ref.  FAST as chol_ref.
template <typename T, int N, int M, bool FAST = false>
__device__ __forceinline__ void axeqb_ref(const C2<T> *L, C2<T> (*X)[M])
{
  T rh[N];
  if constexpr (FAST) diag_rcp<T, N>(L, rh);
#pragma unroll
  for (int c = 0; c < M; c++) {
#pragma unroll
    for (int i = 0; i < N; i++) {
      T xr = X[i][c].x, xi = X[i][c].y;
#pragma unroll
      for (int j = 0; j < i; j++) {
        xr -= (X[j][c].x * L[ltri(i, j)].x - X[j][c].y * L[ltri(i, j)].y);
        xi -= (X[j][c].y * L[ltri(i, j)].x + X[j][c].x * L[ltri(i, j)].y);
      }
      const C2<T> lii = L[ltri(i, i)];
      if constexpr (FAST) {
        X[i][c] = mk<T>((xr * lii.x + xi * lii.y) * rh[i], (xi * lii.x - xr * lii.y) * rh[i]);
      } else {
        const T help = lii.x * lii.x + lii.y * lii.y;
        X[i][c] = mk<T>((xr * lii.x + xi * lii.y) / help, (xi * lii.x - xr * lii.y) / help);
      }
    }
#pragma unroll
    for (int i = N - 1; i >= 0; i--) {
      T xr = X[i][c].x, xi = X[i][c].y;
#pragma unroll
      for (int j = N - 1; j > i; j--) {
        xr = xr - (X[j][c].x * L[ltri(j, i)].x + X[j][c].y * L[ltri(j, i)].y);
        xi = xi - (-X[j][c].x * L[ltri(j, i)].y + X[j][c].y * L[ltri(j, i)].x);
      }
      const C2<T> lii = L[ltri(i, i)];
      if constexpr (FAST) {
        X[i][c] = mk<T>((xr * lii.x - xi * lii.y) * rh[i], (xi * lii.x + xr * lii.y) * rh[i]);
      } else {
        const T help = lii.x * lii.x + lii.y * lii.y;
        X[i][c] = mk<T>((xr * lii.x - xi * lii.y) / help, (xi * lii.x + xr * lii.y) / help);
      }
    }
  }
}

}  // namespace cg
