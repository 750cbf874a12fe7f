// Split y transform of the posterior-mean cubes in the fused inversion.
//
// The length-256 y transform is the four-step product 16 x 16: with y = 16 n1
// + n2 and k = k1 + 16 k2,
//   X[k1 + 16 k2] = sum_n2 w16^(n2 k2) [ w256^(n2 k1) sum_n1 w16^(n1 k1) x[16 n1 + n2] ].
// Stage 1 (the bracket, stored at row 16 k1 + n2) reads and writes the same
// set of 16 rows {16 m + n2}, so it runs in the x-row kernel: a CTA that
// transforms the 32 x rows of two values of n2 finishes their stage 1 in
// shared memory.  Stage 2 reads the 16 contiguous rows 16 k1 .. 16 k1 + 15 and
// produces the natural-order rows k1 + 16 k2, which differ from the rows it
// read: done in place by independent CTAs that would race, so it runs inside
// the bin kernel, whose CTA holds those 16 rows of a 16-column tile of the
// three means (the data cubes take the ordinary y pass, since their residual
// spectra are written in natural order).  The inverse mirrors this: stage 2
// inverse in the bin kernel, stage 1 inverse in the C2R row kernel.  The
// means thus skip the forward and inverse y passes (6 of the 33 cube passes
// of a five-stack inversion).
#pragma once

#include "fft_4step.cuh"
#include "fused_ybin.cuh"
#include "trace.cuh"

namespace cg {

constexpr int kYsNY = 256, kYsN1 = 16, kYsN2 = 16;  // y length and its four-step factors

// x R2C of the 32 rows {16 n1 + n2 : n2 = 2 blockIdx.x + g, g = 0, 1} of
// z-plane blockIdx.y, then stage 1 of the y transform of those rows
template <int M>
__global__ void __launch_bounds__(kFFTThreads) k_r2c_ys(const __grid_constant__ CubeSet cs, const float2 *__restrict__ twg, float prescale)
{
  constexpr int XN1 = fs_n1_rows(M), XN2 = M / XN1, NI = fs_r2c_items(M);
  constexpr int RPC = fs_rows_per_cta(M), P = fs_row_pitch(M), Q = XN1 + 1;
  constexpr int NX = 2 * M, CN = M + 1, OP = CN + 1;
  static_assert(RPC == 2 * kYsN1 && NX == kYsNY, "two stage-1 row groups per CTA, x and y tables alike");
  constexpr int P1 = RPC * XN2, P2 = RPC * NI, P3 = 2 * CN;
  constexpr int B1 = (P1 + kFFTThreads - 1) / kFFTThreads, B2 = (P2 + kFFTThreads - 1) / kFFTThreads;
  constexpr int B3 = (P3 + kFFTThreads - 1) / kFFTThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf = (float2 *)smem_raw;
  float2 *tw = buf + RPC * P;
  float2 *ob = tw + NX;  // x spectra of the 32 rows, [row][k]
  const int z = blockIdx.y, n2b = 2 * blockIdx.x;
  float2 *cube = (float2 *)cs.ptr[blockIdx.z];
  auto row_ptr = [&](int r) -> float2 * {
    const int y = kYsN2 * (r % kYsN1) + n2b + r / kYsN1;
    return cube + ((long)z * kYsNY + y) * CN;
  };
  for (int t = threadIdx.x; t < NX; t += kFFTThreads) tw[t] = twg[t];
  auto load1 = [&](int q, float2 *v) {
    const int t = q * kFFTThreads + threadIdx.x;
    const int n2 = t % XN2, row = t / XN2;
    const bool ok = P1 % kFFTThreads == 0 || t < P1;
    const float2 *rp = row_ptr(ok ? row : 0);
#pragma unroll
    for (int n1 = 0; n1 < XN1; n1++) v[n1] = ok ? rp[XN2 * n1 + n2] : make_float2(0.f, 0.f);
  };
  float2 v[XN1];
  load1(0, v);
  __syncthreads();
#pragma unroll
  for (int q = 0; q < B1; q++) {
    if (q > 0) load1(q, v);
    const int t = q * kFFTThreads + threadIdx.x;
    if (P1 % kFFTThreads == 0 || t < P1) {
      const int n2 = t % XN2, row = t / XN2;
      reg_fft<float, XN1, 2 * XN2>(v, -1, tw);
#pragma unroll
      for (int k1 = 1; k1 < XN1; k1++) v[k1] = cmul<float>(v[k1], tw[2 * n2 * k1]);
#pragma unroll
      for (int k1 = 0; k1 < XN1; k1++) buf[row * P + n2 * Q + k1] = v[k1];
    }
  }
  __syncthreads();
  // x half-length unpack, as k_r2c_rows_4s, into ob
#pragma unroll
  for (int q = 0; q < B2; q++) {
    const int t = q * kFFTThreads + threadIdx.x;
    if (P2 % kFFTThreads == 0 || t < P2) {
      const int ka = t % NI, row = t / NI;
      const bool has_b = ka != 0 || XN1 % 2 == 0;
      const int kb = ka == 0 ? (XN1 % 2 == 0 ? XN1 / 2 : 0) : XN1 - ka;
      float2 a[XN2], b[XN2];
#pragma unroll
      for (int n2 = 0; n2 < XN2; n2++) {
        a[n2] = buf[row * P + n2 * Q + ka];
        b[n2] = buf[row * P + n2 * Q + kb];
      }
      reg_fft<float, XN2, 2 * XN1>(a, -1, tw);
      if (has_b) reg_fft<float, XN2, 2 * XN1>(b, -1, tw);
      float2 *op = ob + row * OP;
#pragma unroll
      for (int k2 = 0; k2 < XN2; k2++) {
        {
          const int k = ka + XN1 * k2;
          const float2 A = a[k2];
          const float2 Bc = ka == 0 ? a[(XN2 - k2) % XN2] : b[XN2 - 1 - k2];
          const float2 B = make_float2(Bc.x, -Bc.y);
          const float2 E = make_float2((A.x + B.x) * 0.5f, (A.y + B.y) * 0.5f);
          const float2 O = make_float2((A.y - B.y) * 0.5f, -(A.x - B.x) * 0.5f);
          const float2 X = cadd<float>(E, cmul<float>(tw[k], O));
          op[k] = make_float2(X.x * prescale, X.y * prescale);
        }
        if (has_b) {
          const int k = kb + XN1 * k2;
          const float2 A = b[k2];
          const float2 Bc = ka == 0 ? b[XN2 - 1 - k2] : a[XN2 - 1 - k2];
          const float2 B = make_float2(Bc.x, -Bc.y);
          const float2 E = make_float2((A.x + B.x) * 0.5f, (A.y + B.y) * 0.5f);
          const float2 O = make_float2((A.y - B.y) * 0.5f, -(A.x - B.x) * 0.5f);
          const float2 X = cadd<float>(E, cmul<float>(tw[k], O));
          op[k] = make_float2(X.x * prescale, X.y * prescale);
        }
      }
      if (ka == 0) {
        const float2 A = a[0];
        op[M] = make_float2((A.x - A.y) * prescale, 0.f);
      }
    }
  }
  __syncthreads();
  // y stage 1: DFT16 over n1 of column k of group g, twiddle w256^(n2 k1), row 16 k1 + n2
#pragma unroll
  for (int q = 0; q < B3; q++) {
    const int t = q * kFFTThreads + threadIdx.x;
    if (t < P3) {
      const int k = t % CN, g = t / CN;
      const int n2 = n2b + g;
      float2 u[kYsN1];
#pragma unroll
      for (int n1 = 0; n1 < kYsN1; n1++) u[n1] = ob[(g * kYsN1 + n1) * OP + k];
      reg_fft<float, kYsN1, kYsNY / kYsN1>(u, -1, tw);
#pragma unroll
      for (int k1 = 1; k1 < kYsN1; k1++) u[k1] = cmul<float>(u[k1], tw[n2 * k1]);
      float2 *dst = cube + ((long)z * kYsNY + n2) * CN + k;
#pragma unroll
      for (int k1 = 0; k1 < kYsN1; k1++) dst[(long)(kYsN2 * k1) * CN] = u[k1];
    }
  }
}

// inverse of k_r2c_ys: y stage 1 inverse of the 32 rows, then the x C2R with postscale
template <int M>
__global__ void __launch_bounds__(kFFTThreads) k_c2r_ys(const __grid_constant__ CubeSet cs, const float2 *__restrict__ twg, float postscale)
{
  constexpr int XN1 = fs_n1_rows(M), XN2 = M / XN1;
  constexpr int RPC = fs_rows_per_cta(M), P = fs_row_pitch(M), Q = XN1 + 1;
  constexpr int NX = 2 * M, CN = M + 1, OP = CN + 1;
  static_assert(RPC == 2 * kYsN1 && NX == kYsNY, "two stage-1 row groups per CTA, x and y tables alike");
  constexpr int P0 = 2 * CN, P1 = RPC * XN2, P2 = RPC * XN1;
  constexpr int B0 = (P0 + kFFTThreads - 1) / kFFTThreads, B1 = (P1 + kFFTThreads - 1) / kFFTThreads;
  constexpr int B2 = (P2 + kFFTThreads - 1) / kFFTThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf = (float2 *)smem_raw;
  float2 *tw = buf + RPC * P;
  float2 *ib = tw + NX;  // x spectra of the 32 rows after the y stage 1 inverse, [row][k]
  const int z = blockIdx.y, n2b = 2 * blockIdx.x;
  float2 *cube = (float2 *)cs.ptr[blockIdx.z];
  for (int t = threadIdx.x; t < NX; t += kFFTThreads) tw[t] = twg[t];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < B0; q++) {
    const int t = q * kFFTThreads + threadIdx.x;
    if (t < P0) {
      const int k = t % CN, g = t / CN;
      const int n2 = n2b + g;
      const float2 *src = cube + ((long)z * kYsNY + n2) * CN + k;
      float2 u[kYsN1];
#pragma unroll
      for (int k1 = 0; k1 < kYsN1; k1++) u[k1] = src[(long)(kYsN2 * k1) * CN];
#pragma unroll
      for (int k1 = 1; k1 < kYsN1; k1++) u[k1] = cmul<float>(u[k1], tw_at<float>(tw, n2 * k1, +1));
      reg_fft<float, kYsN1, kYsNY / kYsN1>(u, +1, tw);
#pragma unroll
      for (int n1 = 0; n1 < kYsN1; n1++) ib[(g * kYsN1 + n1) * OP + k] = u[n1];
    }
  }
  __syncthreads();
  auto row_ptr = [&](int r) -> float2 * {
    const int y = kYsN2 * (r % kYsN1) + n2b + r / kYsN1;
    return cube + ((long)z * kYsNY + y) * CN;
  };
#pragma unroll
  for (int q = 0; q < B1; q++) {
    const int t = q * kFFTThreads + threadIdx.x;
    if (P1 % kFFTThreads == 0 || t < P1) {
      const int n2 = t % XN2, row = t / XN2;
      float2 v[XN1];
#pragma unroll
      for (int n1 = 0; n1 < XN1; n1++) {
        const int k = XN2 * n1 + n2;
        float2 Xk = ib[row * OP + k], Xm = ib[row * OP + (M - k)];
        if (k == 0) { Xk.y = 0.f; Xm.y = 0.f; }  // the C2R keeps only Re of DC and Nyquist
        Xm.y = -Xm.y;
        const float2 E = cadd<float>(Xk, Xm);
        const float2 O = cmulc<float>(csub<float>(Xk, Xm), tw[k]);
        v[n1] = make_float2(E.x - O.y, E.y + O.x);
      }
      reg_fft<float, XN1, 2 * XN2>(v, +1, tw);
#pragma unroll
      for (int k1 = 1; k1 < XN1; k1++) v[k1] = cmul<float>(v[k1], tw_at<float>(tw, 2 * n2 * k1, +1));
#pragma unroll
      for (int k1 = 0; k1 < XN1; k1++) buf[row * P + n2 * Q + k1] = v[k1];
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < B2; q++) {
    const int t = q * kFFTThreads + threadIdx.x;
    if (P2 % kFFTThreads == 0 || t < P2) {
      const int k1 = t % XN1, row = t / XN1;
      float2 u[XN2];
#pragma unroll
      for (int n2 = 0; n2 < XN2; n2++) u[n2] = buf[row * P + n2 * Q + k1];
      reg_fft<float, XN2, 2 * XN1>(u, +1, tw);
      float2 *op = row_ptr(row);
#pragma unroll
      for (int k2 = 0; k2 < XN2; k2++) op[k1 + XN1 * k2] = make_float2(u[k2].x * postscale, u[k2].y * postscale);
      if (k1 == 0) op[M] = make_float2(0.f, 0.f);  // the row's padding pair
    }
  }
}

// The bin loop with y stage 2 of the means: CTA (x tile, k1, z) holds the
// stage-1 rows 16 k1 .. 16 k1 + 15 of a 16-column tile of the 3 means,
// transforms them to the bins (x, k1 + 16 k2, z), runs the posterior of those
// 256 bins (data and residual, covariance: natural order, straight to HBM),
// and transforms the posterior means back to the stage-1 rows (normalised:
// stage 2 then its inverse is the identity, the factor 16 of the unnormalised
// pair moves into the C2R postscale).  Planes outside the band keep the prior
// means (stage-1 rows untouched) and get the prior covariance.  MIXED: guarded bins are redone in FP64 in place.
template <int NT, bool MIXED, int MINB>
__global__ void __launch_bounds__(kFFTThreads, MINB) k_bins_ys(const __grid_constant__ YBinArgs a)
{
  constexpr int W = 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *ms = (float2 *)smem_raw;  // [3][16 rows][W]
  float2 *tw = ms + 3 * kYsN2 * W;
  KTab<float> *ktp = (KTab<float> *)(tw + kYsNY);
  const int k1 = blockIdx.y, z = blockIdx.z;
  const int i0 = blockIdx.x * W;
  const int cnxp = a.f.cnxp;
  const int wv = min(W, cnxp - i0);
  const long plane = (long)cnxp * kYsNY;
  const int t = threadIdx.x, c = t % W, r = t / W;
  for (int q = t; q < kYsNY; q += kFFTThreads) tw[q] = a.tw[q];
  {
    const int *src = (const int *)&a.f.ktab[z];
    int *dst = (int *)ktp;
    for (int q = t; q < (int)(sizeof(KTab<float>) / sizeof(int)); q += kFFTThreads) dst[q] = src[q];
  }
  const bool cv = c < wv;
  const long mrow = (long)z * plane + (long)(kYsN2 * k1 + r) * cnxp + i0 + c;  // this thread's stage-1 element
  __syncthreads();
  const KTab<float> &kt = *ktp;
  const int y = k1 + kYsN1 * r;
  const int ij = y * cnxp + i0 + c;
  const long b = (long)z * plane + ij;
  if (!kt.band) {
    if (cv) {
      float s, lam;
      bin_scales<float>(a.f, ij, z, s, lam);
#pragma unroll
      for (int q = 0; q < 6; q++) a.f.cov[q][b] = make_float2(s * a.f.sig0[q], 0.0f);
    }
    return;  // the band flag is per plane: the whole CTA leaves here
  }
#pragma unroll
  for (int p = 0; p < 3; p++) ms[(p * kYsN2 + r) * W + c] = cv ? a.f.mean[p][mrow] : make_float2(0.f, 0.f);
  __syncthreads();
  if (t < 3 * W) {  // stage 2 over n2 of (mean p, column cc)
    const int p = t / W, cc = t % W;
    float2 u[kYsN2];
#pragma unroll
    for (int n2 = 0; n2 < kYsN2; n2++) u[n2] = ms[(p * kYsN2 + n2) * W + cc];
    reg_fft<float, kYsN2, kYsNY / kYsN2>(u, -1, tw);
#pragma unroll
    for (int k2 = 0; k2 < kYsN2; k2++) ms[(p * kYsN2 + k2) * W + cc] = u[k2];
  }
  __syncthreads();
  if (cv) {
    float s, lam;
    bin_scales<float>(a.f, ij, z, s, lam);
    float2 d[NT], mu[3], cov[6];
#pragma unroll
    for (int l = 0; l < NT; l++) d[l] = a.f.data[l][b];
#pragma unroll
    for (int p = 0; p < 3; p++) mu[p] = ms[(p * kYsN2 + r) * W + c];
    float2 L[NT * (NT + 1) / 2];
    float inv[NT], cond = 0.0f;
    build_sd<float, NT>(kt, s, lam, L);
    const bool ok = chol_std<float, NT>(L, inv, cond);
    bool queued = false;
    if constexpr (MIXED) {
      if (!ok || cond > a.f.cond_thr) {
        // queued for k_ys_fixup64: data untouched, the prior mean stashed in the
        // first three covariance slots, the tile keeps the prior mean
        const int pos = atomicAdd(&a.f.counters[0], 1);
        if (pos < a.f.queue_cap) {
          a.f.queue[pos] = (int)b;
#pragma unroll
          for (int p = 0; p < 3; p++) a.f.cov[p][b] = mu[p];
          queued = true;
        } else {
          atomicAdd(&a.f.counters[2], 1);  // queue full: keep the FP32 answer
        }
      }
    }
    if (!queued) {
      if (!ok) {
        atomicAdd(&a.f.counters[1], 1);
#pragma unroll
        for (int q = 0; q < 6; q++) cov[q] = make_float2(s * a.f.sig0[q], 0.0f);
      } else {
        posterior_from_chol<float, NT>(kt, a.f.sig0, s, lam, L, inv, d, mu, cov, false);
      }
#pragma unroll
      for (int l = 0; l < NT; l++) a.f.data[l][b] = d[l];
#pragma unroll
      for (int q = 0; q < 6; q++) a.f.cov[q][b] = cov[q];
#pragma unroll
      for (int p = 0; p < 3; p++) ms[(p * kYsN2 + r) * W + c] = mu[p];
    }
  }
  __syncthreads();
  if (t < 3 * W) {  // stage 2 inverse over k2, normalised (1/16: exact) so that planes it skips match
    const int p = t / W, cc = t % W;
    float2 u[kYsN2];
#pragma unroll
    for (int k2 = 0; k2 < kYsN2; k2++) u[k2] = ms[(p * kYsN2 + k2) * W + cc];
    reg_fft<float, kYsN2, kYsNY / kYsN2>(u, +1, tw);
    constexpr float inv_n2 = 1.0f / kYsN2;
#pragma unroll
    for (int n2 = 0; n2 < kYsN2; n2++) ms[(p * kYsN2 + n2) * W + cc] = make_float2(u[n2].x * inv_n2, u[n2].y * inv_n2);
  }
  __syncthreads();
  if (cv) {
#pragma unroll
    for (int p = 0; p < 3; p++) a.f.mean[p][mrow] = ms[(p * kYsN2 + r) * W + c];
  }
}

// FP64 redo of the bins k_bins_ys queued: posterior from the untouched data
// and the stashed prior mean, residual and covariance written in place, and
// the change of the posterior mean added to the 16 stage-1 rows it reaches
// through the normalised stage 2 inverse: row 16 k1 + n2 gets
// (mu+ - mu) w16^(-n2 k2) / 16 for the bin k1 + 16 k2 (atomically: bins of
// one row group may share rows).
template <int NT>
__global__ void __launch_bounds__(128) k_ys_fixup64(const __grid_constant__ YBinArgs a)
{
  const int nq = min(*((volatile int *)&a.f.counters[0]), a.f.queue_cap);
  const int cnxp = a.f.cnxp;
  const long plane = (long)cnxp * kYsNY;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
    const long b = a.f.queue[q];
    const int z = (int)(b / plane);
    const int ij = (int)(b - (long)z * plane);
    const int y = ij / cnxp, x = ij - y * cnxp;
    float s, lam;
    bin_scales<float>(a.f, ij, z, s, lam);
    float2 d[NT], mu[3], mu0[3], cov[6];
#pragma unroll
    for (int l = 0; l < NT; l++) d[l] = a.f.data[l][b];
#pragma unroll
    for (int p = 0; p < 3; p++) mu0[p] = mu[p] = a.f.cov[p][b];
    double s0[6];
#pragma unroll
    for (int t = 0; t < 6; t++) s0[t] = a.sig0d[t];
    if (!bin_fp64_t<NT>(a.ktab_d, s0, z, s, lam, d, mu, cov)) atomicAdd(&a.f.counters[1], 1);
#pragma unroll
    for (int l = 0; l < NT; l++) a.f.data[l][b] = d[l];
#pragma unroll
    for (int t = 0; t < 6; t++) a.f.cov[t][b] = cov[t];
    const int k1 = y % kYsN1, k2 = y / kYsN1;
#pragma unroll
    for (int p = 0; p < 3; p++) {
      const float2 dm = make_float2(mu[p].x - mu0[p].x, mu[p].y - mu0[p].y);
      if (dm.x == 0.0f && dm.y == 0.0f) continue;
      float2 *col = a.f.mean[p] + (long)z * plane + (long)(kYsN2 * k1) * cnxp + x;
      for (int n2 = 0; n2 < kYsN2; n2++) {
        const float2 w = tw_at<float>(a.tw, (kYsNY / kYsN2) * ((n2 * k2) % kYsN2), +1);
        const float2 v = cmul<float>(dm, w);
        atomicAdd(&col[(long)n2 * cnxp].x, v.x * (1.0f / kYsN2));
        atomicAdd(&col[(long)n2 * cnxp].y, v.y * (1.0f / kYsN2));
      }
    }
  }
}

}  // namespace cg
