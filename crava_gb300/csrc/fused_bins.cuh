// Per-bin arithmetic of the fused posterior (shared by k_invert_fused in
// posterior.cu and the fused y-transform kernel in fused_ybin.cu).
//
// For every in-band bin, with the separable prior S = s*Sigma0 and the
// per-k tables (posterior.cuh, KTab):
//   Sd = s M + lam E + D, L = chol(Sd), Y = L^-1 K S0, v = L^-1 (d - K mu),
//   mu+ = mu + s Y^H v, S+ = s Sigma0 - s^2 Y^H Y, residual = d - K mu+.
#pragma once

#include <type_traits>

#include "common.cuh"
#include "posterior.cuh"

namespace cg {

// calls f(std::integral_constant<int, NT>) for the model's stack count
template <typename F>
int dispatch_nt(int nt, F &&f)
{
  switch (nt) {
    case 1: return f(std::integral_constant<int, 1>());
    case 2: return f(std::integral_constant<int, 2>());
    case 3: return f(std::integral_constant<int, 3>());
    case 4: return f(std::integral_constant<int, 4>());
    case 5: return f(std::integral_constant<int, 5>());
    case 6: return f(std::integral_constant<int, 6>());
    case 7: return f(std::integral_constant<int, 7>());
    case 8: return f(std::integral_constant<int, 8>());
    default: set_error("ntheta %d outside 1..%d", nt, kMaxTheta); return CG_ERR_ARG;
  }
}


// ---------------------------------------------------------------------------
// fused kernels
// ---------------------------------------------------------------------------
template <typename T>
struct FusedArgs {
  C2<T> *data[kMaxTheta];
  C2<T> *mean[3];
  C2<T> *cov[6];
  const float2 *cxy;      // cnxp*nyp  (FP32 tables)
  const float2 *ct;       // nzp/2+1
  const double2 *cxy_d;   // FP64 tables (FP64 mode)
  const double2 *ct_d;
  // per-bin (s, lam) table of a prior with nonzero correlation gradients
  // (cg_prior_spectra_grad), bin order; null for the separable prior
  const float2 *sl;
  const double2 *sl_d;
  const KTab<T> *ktab;
  T sig0[6];
  int cnxp, nyp, nzp, plane;
  float cond_thr;
  int *queue;
  int queue_cap;
  int *counters;
  int k0;       // first z-plane of the launch (a launch covers planes k0 .. k0 + grid.y - 1)
  int chunked;  // MIXED fix-up of one z-chunk: queue entries from counters[3] on
};

// prior scale s = |Re(Cxy Ct)| and error eigenvalue lam = |Re Cxy| of one bin
// (separable prior); TAB: s = |Re P|, lam = |Re E| read from the per-bin
// table of a prior made non-separable by correlation gradients (a separate
// instantiation, so the separable kernels carry no table code)
template <typename T, bool TAB = false>
__device__ __forceinline__ void bin_scales(const FusedArgs<T> &a, int ij, int k, T &s, T &lam)
{
  if constexpr (TAB) {
    const long b = (long)k * a.plane + ij;
    if (sizeof(T) == 8 && a.sl_d) {
      const double2 v = a.sl_d[b];
      s = (T)v.x;
      lam = (T)v.y;
    } else {
      const float2 v = __ldg(&a.sl[b]);
      s = (T)v.x;
      lam = (T)v.y;
    }
    return;
  }
  const int cnzp = a.nzp / 2 + 1;
  if (sizeof(T) == 8) {
    const double2 cx = a.cxy_d[ij];
    double2 t = k < cnzp ? a.ct_d[k] : make_double2(a.ct_d[a.nzp - k].x, -a.ct_d[a.nzp - k].y);
    s = (T)fabs(cx.x * t.x - cx.y * t.y);
    lam = (T)fabs(cx.x);
  } else {
    const float2 cx = __ldg(&a.cxy[ij]);
    float2 t = k < cnzp ? __ldg(&a.ct[k]) : make_float2(a.ct[a.nzp - k].x, -a.ct[a.nzp - k].y);
    s = (T)fabsf(cx.x * t.x - cx.y * t.y);
    lam = (T)fabsf(cx.x);
  }
}

// Plain lower Cholesky (no pre-scaling) with the reference's failure rule:
// fail when A00 <= 0 or any pivot <= 1e-20 * A00 (lib_matr.c:78-168 scales by
// A00 first).  inv[i] receives 1/L_ii (FP32: from one rsqrt per pivot), and
// cond the squared ratio of the largest to the smallest pivot of L, a cheap
// lower bound on the condition number.
template <typename T>
__device__ __forceinline__ T inv_sqrt(T x)
{
  if constexpr (sizeof(T) == 4) return rsqrtf(x);
  else return 1.0 / sqrt(x);
}

template <typename T, int N>
__device__ __forceinline__ bool chol_std(C2<T> *L, T *inv, T &cond)
{
  const T a00 = L[0].x;
  if (!(a00 > (T)0)) return false;
  const T tol = (T)kCholTol * a00;
  T dmax = 0, dmin = 0;
#pragma unroll
  for (int i = 0; i < N; i++) {
#pragma unroll
    for (int j = 0; j < i; j++) {
      C2<T> acc = L[tri(i, j)];
#pragma unroll
      for (int k = 0; k < j; k++) acc = csub<T>(acc, cmulc<T>(L[tri(i, k)], L[tri(j, k)]));
      L[tri(i, j)] = mk<T>(acc.x * inv[j], acc.y * inv[j]);
    }
    T piv = L[tri(i, i)].x;
#pragma unroll
    for (int k = 0; k < i; k++) piv -= L[tri(i, k)].x * L[tri(i, k)].x + L[tri(i, k)].y * L[tri(i, k)].y;
    if (!(piv > tol)) return false;
    const T r = inv_sqrt<T>(piv);
    const T di = piv * r;
    inv[i] = r;
    L[tri(i, i)] = mk<T>(di, (T)0);
    dmax = i == 0 ? di : (di > dmax ? di : dmax);
    dmin = i == 0 ? di : (di < dmin ? di : dmin);
  }
  const T q = dmax / dmin;
  cond = q * q;
  return true;
}

// forward substitution L x = b in place
template <typename T, int N>
__device__ __forceinline__ void lsolve(const C2<T> *L, const T *inv, C2<T> *x)
{
#pragma unroll
  for (int i = 0; i < N; i++) {
    C2<T> acc = x[i];
#pragma unroll
    for (int j = 0; j < i; j++) acc = csub<T>(acc, cmul<T>(L[tri(i, j)], x[j]));
    x[i] = mk<T>(acc.x * inv[i], acc.y * inv[i]);
  }
}

// backward substitution L^H x = b in place
template <typename T, int N>
__device__ __forceinline__ void lhsolve(const C2<T> *L, const T *inv, C2<T> *x)
{
#pragma unroll
  for (int i = N - 1; i >= 0; i--) {
    C2<T> acc = x[i];
#pragma unroll
    for (int j = i + 1; j < N; j++) acc = csub<T>(acc, cmulc<T>(x[j], L[tri(j, i)]));
    x[i] = mk<T>(acc.x * inv[i], acc.y * inv[i]);
  }
}

template <typename T, int N>
__device__ __forceinline__ void build_sd(const KTab<T> &kt, T s, T lam, C2<T> *Sd)
{
#pragma unroll
  for (int l = 0; l < N; l++)
#pragma unroll
    for (int m = 0; m <= l; m++) {
      const int t = tri(l, m);
      C2<T> v = mk<T>(s * kt.M[t].x + lam * kt.E[t].x, s * kt.M[t].y + lam * kt.E[t].y);
      if (l == m) v = mk<T>(v.x + kt.D[l], (T)0);
      Sd[t] = v;
    }
}

// Posterior of one in-band bin from the Cholesky factor L of Sd.  d[] holds
// the data on entry and the residual on exit; mu the prior/posterior mean.
// refine: solve Sd u = r with one step of iterative refinement (FP64 paths).
template <typename T, int N>
__device__ __forceinline__ void posterior_from_chol(const KTab<T> &kt, const T *sig0, T s, T lam, const C2<T> *L,
                                                    const T *inv, C2<T> *d, C2<T> *mu, C2<T> *cov, bool refine)
{
  C2<T> r[N];
#pragma unroll
  for (int l = 0; l < N; l++) {
    C2<T> km = mk<T>(0, 0);
#pragma unroll
    for (int p = 0; p < 3; p++) km = cadd<T>(km, cmul<T>(kt.K[l][p], mu[p]));
    r[l] = csub<T>(d[l], km);
  }
  // covariance: S+ = s S0 - s^2 Y^H Y with Y = L^-1 K S0
  C2<T> Y[3][N];
#pragma unroll
  for (int p = 0; p < 3; p++) {
#pragma unroll
    for (int l = 0; l < N; l++) Y[p][l] = kt.KS0[l][p];
    lsolve<T, N>(L, inv, Y[p]);
  }
  const int pq[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
#pragma unroll
  for (int t = 0; t < 6; t++) {
    C2<T> acc = mk<T>(0, 0);
#pragma unroll
    for (int l = 0; l < N; l++) acc = cadd<T>(acc, cmulc<T>(Y[pq[t][1]][l], Y[pq[t][0]][l]));
    cov[t] = mk<T>(s * sig0[t] - s * s * acc.x, t < 3 ? (T)0 : -s * s * acc.y);
  }
  C2<T> up[3];
  if (!refine) {
    // mean: mu+ = mu + s Y^H v, v = L^-1 r
    C2<T> v[N];
#pragma unroll
    for (int l = 0; l < N; l++) v[l] = r[l];
    lsolve<T, N>(L, inv, v);
#pragma unroll
    for (int p = 0; p < 3; p++) {
      C2<T> acc = mk<T>(0, 0);
#pragma unroll
      for (int l = 0; l < N; l++) acc = cadd<T>(acc, cmulc<T>(v[l], Y[p][l]));
      up[p] = acc;
    }
  } else {
    // u = Sd^-1 r, one refinement step u += Sd^-1 (r - Sd u), mu+ = mu + s (K S0)^H u
    C2<T> u[N], rho[N], Sd[N * (N + 1) / 2];
#pragma unroll
    for (int l = 0; l < N; l++) u[l] = r[l];
    lsolve<T, N>(L, inv, u);
    lhsolve<T, N>(L, inv, u);
    build_sd<T, N>(kt, s, lam, Sd);
#pragma unroll
    for (int l = 0; l < N; l++) {
      C2<T> acc = r[l];
#pragma unroll
      for (int m = 0; m < N; m++) {
        C2<T> a = l >= m ? Sd[tri(l, m)] : cconj<T>(Sd[tri(m, l)]);
        acc = csub<T>(acc, cmul<T>(a, u[m]));
      }
      rho[l] = acc;
    }
    lsolve<T, N>(L, inv, rho);
    lhsolve<T, N>(L, inv, rho);
#pragma unroll
    for (int l = 0; l < N; l++) u[l] = cadd<T>(u[l], rho[l]);
#pragma unroll
    for (int p = 0; p < 3; p++) {
      C2<T> acc = mk<T>(0, 0);
#pragma unroll
      for (int l = 0; l < N; l++) acc = cadd<T>(acc, cmulc<T>(u[l], kt.KS0[l][p]));
      up[p] = acc;
    }
  }
#pragma unroll
  for (int p = 0; p < 3; p++) mu[p] = mk<T>(mu[p].x + s * up[p].x, mu[p].y + s * up[p].y);
#pragma unroll
  for (int l = 0; l < N; l++) {
    C2<T> km = mk<T>(0, 0);
#pragma unroll
    for (int p = 0; p < 3; p++) km = cadd<T>(km, cmul<T>(kt.K[l][p], mu[p]));
    d[l] = csub<T>(d[l], km);
  }
}

template <typename T>
__device__ __forceinline__ void write_prior_cov(const FusedArgs<T> &a, long b, T s)
{
#pragma unroll
  for (int t = 0; t < 6; t++) a.cov[t][b] = mk<T>(s * a.sig0[t], (T)0);
}

int check_ws(Workspace *w);
// the fused bin kernel (and, MIXED, the FP64 fix-up) over z-planes k0 .. k0 + nk - 1 (posterior.cu)
int fused_bins_range(Workspace *w, void *const *data, void *const *mean, void *const *cov, int precision, int k0,
                     int nk, bool chunked, cudaStream_t st);
template <typename T>
int fill_fused_args(Workspace *w, void *const *data, void *const *mean, void *const *cov, FusedArgs<T> *out);

}  // namespace cg
