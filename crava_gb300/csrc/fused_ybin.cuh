// The fused form of Crava::computePostMeanResidAndFFTCov with the y
// transforms folded into the bin loop.
//
// The 3D transforms are separable, so the forward transform may run its axes
// in the order x, z, y and the inverse in the order y, z, x.  Done that way,
// the last forward pass and the first inverse pass both work on y columns,
// and a tile of y columns lies in ONE z-plane: one CTA can
//   1. load W x-adjacent y columns of the n data and 3 prior-mean cubes of
//      z-plane k, transform them (four-step, in registers and shared memory),
//   2. run the bin loop on those W*nyp bins with the per-k tables of plane k
//      staged once (residual and posterior covariance spectra go straight to
//      HBM, the posterior means stay in shared memory),
//   3. inverse-transform the 3 posterior-mean columns and write them back,
// which removes one HBM round trip of the n+3 input cubes (forward y pass)
// and of the 3 posterior means (inverse y pass) per inversion.
//
// MIXED precision: bins whose Cholesky fails in FP32 or whose pivot-ratio
// condition estimate exceeds the threshold are redone in FP64 in place (one
// refinement step), since their posterior mean must be final before the
// inverse y transform.
#pragma once

#include "fft.cuh"
#include "fft_4step.cuh"
#include "fused_bins.cuh"
#include "trace.cuh"

namespace cg {

constexpr int kYW = 4;  // x columns per CTA (32-byte row segments)

struct YBinArgs {
  FusedArgs<float> f;
  const KTab<double> *ktab_d;
  double sig0d[6];
  const float2 *tw;  // forward table of the y length
  int mixed;
};

// FP64 redo of one bin (rare: kept out of line so it costs the FP32 path no
// registers); sig0d: the 6 entries of Sigma0 in bin-loop order
template <int NT>
__device__ __noinline__ int bin_fp64_t(const KTab<double> *__restrict__ ktd, const double *sig0d, int k, float sf,
                                       float lamf, float2 *d, float2 *mu, float2 *cov)
{
  const KTab<double> &kt = ktd[k];
  const double s = sf, lam = lamf;
  double2 dd[NT], md[3], cd[6], L[NT * (NT + 1) / 2];
#pragma unroll
  for (int l = 0; l < NT; l++) dd[l] = make_double2(d[l].x, d[l].y);
#pragma unroll
  for (int p = 0; p < 3; p++) md[p] = make_double2(mu[p].x, mu[p].y);
  build_sd<double, NT>(kt, s, lam, L);
  double cond, invr[NT];
  if (!chol_std<double, NT>(L, invr, cond)) {
#pragma unroll
    for (int t = 0; t < 6; t++) cov[t] = make_float2((float)(s * sig0d[t]), 0.0f);
    return 0;
  }
  posterior_from_chol<double, NT>(kt, sig0d, s, lam, L, invr, dd, md, cd, true);
#pragma unroll
  for (int l = 0; l < NT; l++) d[l] = make_float2((float)dd[l].x, (float)dd[l].y);
#pragma unroll
  for (int p = 0; p < 3; p++) mu[p] = make_float2((float)md[p].x, (float)md[p].y);
#pragma unroll
  for (int t = 0; t < 6; t++) cov[t] = make_float2((float)cd[t].x, (float)cd[t].y);
  return 1;
}

template <int NT>
__device__ __forceinline__ int bin_fp64(const YBinArgs &a, int k, float sf, float lamf, float2 *d, float2 *mu,
                                        float2 *cov)
{
  double s0[6];
#pragma unroll
  for (int t = 0; t < 6; t++) s0[t] = a.sig0d[t];
  return bin_fp64_t<NT>(a.ktab_d, s0, k, sf, lamf, d, mu, cov);
}

template <int N, int NT, int MINB>
__global__ void __launch_bounds__(kFFTThreads, MINB) k_ybin(const __grid_constant__ YBinArgs a)
{
  constexpr int W = kYW;
  constexpr int N1 = fs_n1(N), N2 = N / N1;
  constexpr int NC = NT + 3;  // cubes held: data 0..NT-1, means NT..NT+2
  constexpr int NXM = N1 > N2 ? N1 : N2;
  constexpr int PER = W * NXM;                // thread slots per cube and round
  constexpr int CPR = kFFTThreads / PER;      // cubes per round
  static_assert(CPR >= 1, "a y column tile must fit one round");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *spec = (float2 *)smem_raw;          // NC cubes x (N x W), [j][c]
  float2 *tw = spec + NC * N * W;             // N
  KTab<float> *ktp = (KTab<float> *)(tw + N);
  const int k = blockIdx.y;
  const int i0 = blockIdx.x * W;
  const int cnxp = a.f.cnxp;
  const int wv = min(W, cnxp - i0);
  const long plane = (long)cnxp * N;
  const int t = threadIdx.x;
  for (int q = t; q < N; q += kFFTThreads) tw[q] = a.tw[q];
  {
    const int *src = (const int *)&a.f.ktab[k];
    int *dst = (int *)ktp;
    for (int q = t; q < (int)(sizeof(KTab<float>) / sizeof(int)); q += kFFTThreads) dst[q] = src[q];
  }
  __syncthreads();
  const KTab<float> &kt = *ktp;
  auto cube_in = [&](int cb) -> const float2 * {
    return cb < NT ? (const float2 *)a.f.data[cb] : (const float2 *)a.f.mean[cb - NT];
  };

  // 1. forward y transforms of the NC column tiles
  for (int c0 = 0; c0 < NC; c0 += CPR) {
    const int cb = c0 + t / PER, r = t % PER;
    const bool live = t < CPR * PER && cb < NC;  // slots past the round's cubes idle
    const bool act1 = live && r < W * N2, act2 = live && r < W * N1;
    float2 *sp = spec + (long)(cb < NC ? cb : 0) * N * W;
    if (act1) {
      const int c = r % W, n2 = r / W;
      float2 v[N1];
      const float2 *src = cube_in(cb) + (long)k * plane + i0 + c;
#pragma unroll
      for (int n1 = 0; n1 < N1; n1++) v[n1] = c < wv ? src[(long)(N2 * n1 + n2) * cnxp] : make_float2(0.f, 0.f);
      reg_fft<float, N1, N2>(v, -1, tw);
#pragma unroll
      for (int k1 = 1; k1 < N1; k1++) v[k1] = cmul<float>(v[k1], tw_at<float>(tw, n2 * k1, -1));
#pragma unroll
      for (int k1 = 0; k1 < N1; k1++) sp[(k1 * N2 + n2) * W + c] = v[k1];
    }
    __syncthreads();
    float2 u[N2];
    const int c = r % W, k1 = r / W;
    if (act2) {
#pragma unroll
      for (int n2 = 0; n2 < N2; n2++) u[n2] = sp[(k1 * N2 + n2) * W + c];
      reg_fft<float, N2, N1>(u, -1, tw);
    }
    __syncthreads();  // every exchange value read before the outputs overwrite the tile
    if (act2) {
#pragma unroll
      for (int k2 = 0; k2 < N2; k2++) sp[(k1 + N1 * k2) * W + c] = u[k2];
    }
  }
  __syncthreads();

  // 2. bin loop over the W x N bins of the tile (all in z-plane k)
  for (int bi = t; bi < W * N; bi += kFFTThreads) {
    const int c = bi % W, j = bi / W;
    if (c >= wv) continue;
    const int ij = i0 + c + j * cnxp;
    const long b = (long)k * plane + ij;
    float s, lam;
    bin_scales<float>(a.f, ij, k, s, lam);
    float2 d[NT], mu[3], cov[6];
#pragma unroll
    for (int l = 0; l < NT; l++) d[l] = spec[(long)l * N * W + j * W + c];
#pragma unroll
    for (int p = 0; p < 3; p++) mu[p] = spec[(long)(NT + p) * N * W + j * W + c];
    if (!kt.band) {
#pragma unroll
      for (int q = 0; q < 6; q++) cov[q] = make_float2(s * a.f.sig0[q], 0.0f);
    } else {
      float2 L[NT * (NT + 1) / 2];
      float inv[NT], cond = 0.0f;
      build_sd<float, NT>(kt, s, lam, L);
      const bool ok = chol_std<float, NT>(L, inv, cond);
      if (a.mixed && (!ok || cond > a.f.cond_thr)) {
        atomicAdd(&a.f.counters[0], 1);
        float2 dl[NT], ml[3], cl[6];
#pragma unroll
        for (int l = 0; l < NT; l++) dl[l] = d[l];
#pragma unroll
        for (int p = 0; p < 3; p++) ml[p] = mu[p];
        if (!bin_fp64<NT>(a, k, s, lam, dl, ml, cl)) atomicAdd(&a.f.counters[1], 1);
#pragma unroll
        for (int l = 0; l < NT; l++) d[l] = dl[l];
#pragma unroll
        for (int p = 0; p < 3; p++) mu[p] = ml[p];
#pragma unroll
        for (int q = 0; q < 6; q++) cov[q] = cl[q];
      } else if (!ok) {
        atomicAdd(&a.f.counters[1], 1);
#pragma unroll
        for (int q = 0; q < 6; q++) cov[q] = make_float2(s * a.f.sig0[q], 0.0f);
      } else {
        posterior_from_chol<float, NT>(kt, a.f.sig0, s, lam, L, inv, d, mu, cov, false);
      }
    }
#pragma unroll
    for (int l = 0; l < NT; l++) a.f.data[l][b] = d[l];
#pragma unroll
    for (int q = 0; q < 6; q++) a.f.cov[q][b] = cov[q];
#pragma unroll
    for (int p = 0; p < 3; p++) spec[(long)(NT + p) * N * W + j * W + c] = mu[p];
  }
  __syncthreads();

  // 3. inverse y transforms of the 3 posterior means (CPR >= 1 cubes per round)
  for (int c0 = 0; c0 < 3; c0 += CPR) {
    const int m = c0 + t / PER, r = t % PER;
    const bool live = t < CPR * PER && m < 3;
    const bool act1 = live && r < W * N2, act2 = live && r < W * N1;
    float2 *sp = spec + (long)(NT + (m < 3 ? m : 0)) * N * W;
    float2 v[N1];
    const int c1 = r % W, n2 = r / W;
    if (act1) {
#pragma unroll
      for (int n1 = 0; n1 < N1; n1++) v[n1] = sp[(N2 * n1 + n2) * W + c1];
      reg_fft<float, N1, N2>(v, +1, tw);
#pragma unroll
      for (int k1 = 1; k1 < N1; k1++) v[k1] = cmul<float>(v[k1], tw_at<float>(tw, n2 * k1, +1));
    }
    __syncthreads();  // every natural-order value read before the exchange overwrites the tile
    if (act1) {
#pragma unroll
      for (int k1 = 0; k1 < N1; k1++) sp[(k1 * N2 + n2) * W + c1] = v[k1];
    }
    __syncthreads();
    if (act2) {
      const int c = r % W, k1 = r / W;
      float2 u[N2];
#pragma unroll
      for (int q = 0; q < N2; q++) u[q] = sp[(k1 * N2 + q) * W + c];
      reg_fft<float, N2, N1>(u, +1, tw);
      if (c < wv) {
        float2 *dst = a.f.mean[m] + (long)k * plane + i0 + c;
#pragma unroll
        for (int k2 = 0; k2 < N2; k2++) dst[(long)(k1 + N1 * k2) * cnxp] = u[k2];
      }
    }
    __syncthreads();
  }
}

// launch for one y length, dispatched on the stack count.  Two resident CTAs
// of 256 threads (128 registers): the 85-register build spills in the bin
// loop and measured 1.4x slower.
template <int N>
int launch_ybin_n(const YBinArgs &a, int nt, int ncols_tiles, int nzp, double bytes, cudaStream_t st)
{
  return dispatch_nt(nt, [&](auto NTc) -> int {
    constexpr int NT = decltype(NTc)::value;
    const size_t smem = ((size_t)(NT + 3) * N * kYW + N) * sizeof(float2) + sizeof(KTab<float>);
    static bool attr_set[64] = {};
    cudaError_t e = smem_limit_once(k_ybin<N, NT, 2>, smem, attr_set);
    if (e != cudaSuccess) return cuda_status(e, "k_ybin attribute");
    TraceScope ts("k_ybin", st, bytes);
    k_ybin<N, NT, 2><<<dim3(ncols_tiles, nzp), kFFTThreads, smem, st>>>(a);
    CG_CHECK_LAUNCH("k_ybin");
    return CG_OK;
  });
}

// instantiated in fused_ybin_<N>.cu
int launch_ybin_256(const YBinArgs &a, int nt, int tiles, int nzp, double bytes, cudaStream_t st);
int launch_ybin_200(const YBinArgs &a, int nt, int tiles, int nzp, double bytes, cudaStream_t st);
int launch_ybin_128(const YBinArgs &a, int nt, int tiles, int nzp, double bytes, cudaStream_t st);

}  // namespace cg

