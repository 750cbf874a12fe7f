// The fused inversion with the split y transform of the means (ysplit.cuh):
//   data cubes: x pass, y pass;  means: x pass + y stage 1 (k_r2c_ys);
//   z pass of all n + 3 cubes;  k_bins_ys (y stage 2 of the means, bin loop,
//   stage 2 inverse);  inverse z pass of the means;  y stage 1 inverse + x C2R
//   of the means (k_c2r_ys).
#include <cmath>
#include <cstring>

#include "tuning.cuh"
#include "ysplit.cuh"

namespace cg {

namespace {

template <int NT, bool MIXED, int MINB>
int launch_bins_ys_t(const YBinArgs &a, int cnxp, int nzp, cudaStream_t st, double bytes)
{
  const size_t smem = (3 * kYsN2 * 16 + kYsNY) * sizeof(float2) + sizeof(KTab<float>);
  static bool attr[64] = {};
  cudaError_t e = smem_limit_once(k_bins_ys<NT, MIXED, MINB>, smem, attr);
  if (e != cudaSuccess) return cuda_status(e, "k_bins_ys attribute");
  dim3 grid(ceil_div(cnxp, 16), kYsN1, nzp);
  TraceScope ts(MIXED ? "k_bins_ys_mixed" : "k_bins_ys_fp32", st, bytes);
  k_bins_ys<NT, MIXED, MINB><<<grid, kFFTThreads, smem, st>>>(a);
  CG_CHECK_LAUNCH("k_bins_ys");
  return CG_OK;
}

// CG_TUNE_BIN_MINB 6 (the 85-register build of the 128-thread bin kernel) maps
// to 3 resident 256-thread CTAs here, anything else to 2 (128 registers)
template <int NT>
int launch_bins_ys(const YBinArgs &a, int cnxp, int nzp, cudaStream_t st, double bytes)
{
  const bool tight = cg_tune_get(CG_TUNE_BIN_MINB, NT) == 6;
  if (a.mixed) {
    if (tight) return launch_bins_ys_t<NT, true, 3>(a, cnxp, nzp, st, bytes);
    return launch_bins_ys_t<NT, true, 2>(a, cnxp, nzp, st, bytes);
  }
  if (tight) return launch_bins_ys_t<NT, false, 3>(a, cnxp, nzp, st, bytes);
  return launch_bins_ys_t<NT, false, 2>(a, cnxp, nzp, st, bytes);
}

int rows_ys(bool forward, void *const *cubes, int n, int nzp, float scale, cudaStream_t st)
{
  constexpr int M = kYsNY / 2;
  constexpr int RPC = fs_rows_per_cta(M), P = fs_row_pitch(M);
  const size_t smem = ((size_t)RPC * P + 2 * M + (size_t)RPC * (M + 2)) * sizeof(float2);
  CubeSet cs;
  for (int i = 0; i < kMaxBatch; i++) cs.ptr[i] = i < n ? cubes[i] : nullptr;
  const float2 *tw = (const float2 *)twiddle_table<float>(2 * M);
  if (!tw) return cuda_status(cudaGetLastError(), "twiddle table");
  dim3 grid(kYsN2 / 2, nzp, n);
  const double bytes = (double)n * kYsNY * nzp * (2.0 * M * sizeof(float) + (M + 1.0) * sizeof(float2));
  cudaError_t e;
  if (forward) {
    static bool attr[64] = {};
    if ((e = smem_limit_once(k_r2c_ys<M>, smem, attr)) != cudaSuccess) return cuda_status(e, "k_r2c_ys attribute");
    TraceScope ts("k_r2c_ys", st, bytes);
    k_r2c_ys<M><<<grid, kFFTThreads, smem, st>>>(cs, tw, scale);
  } else {
    static bool attr[64] = {};
    if ((e = smem_limit_once(k_c2r_ys<M>, smem, attr)) != cudaSuccess) return cuda_status(e, "k_c2r_ys attribute");
    TraceScope ts("k_c2r_ys", st, bytes);
    k_c2r_ys<M><<<grid, kFFTThreads, smem, st>>>(cs, tw, scale);
  }
  CG_CHECK_LAUNCH(forward ? "k_r2c_ys" : "k_c2r_ys");
  return CG_OK;
}

}  // namespace

// nxp = nyp = 256 (the kernels' compile-time lengths); returns 0 when the
// sizes do not fit, a status otherwise
bool ysplit_fits(const Workspace *w) { return w->nxp == kYsNY && w->nyp == kYsNY && w->ntheta + 3 <= kMaxBatch; }

int invert_cubes_ysplit(Workspace *w, float *const *data, float *const *mean, float *const *cov, int precision,
                        cudaStream_t st, cudaEvent_t bins_done)
{
  const int nt = w->ntheta, nxp = w->nxp, nyp = w->nyp, nzp = w->nzp;
  const int cnxp = nxp / 2 + 1;
  const long plane = (long)cnxp * nyp;
  const float pre = (float)(1.0 / sqrt((double)nxp * nyp * nzp));
  void *dcubes[kMaxTheta], *mcubes[3], *all[kMaxTheta + 3];
  for (int l = 0; l < nt; l++) all[l] = dcubes[l] = data[l];
  for (int p = 0; p < 3; p++) all[nt + p] = mcubes[p] = mean[p];
  int rc;
  if ((rc = fft_x_pass<float>(dcubes, nt, nxp, nyp, nzp, true, pre, st))) return rc;
  if ((rc = fft_cols<float>(dcubes, nt, nyp, cnxp, cnxp, plane, nzp, -1, st))) return rc;
  if ((rc = rows_ys(true, mcubes, 3, nzp, pre, st))) return rc;
  if ((rc = fft_cols<float>(all, nt + 3, nzp, cnxp, plane, cnxp, nyp, -1, st))) return rc;
  YBinArgs a;
  memset(&a, 0, sizeof(a));
  if ((rc = fill_fused_args(w, (void *const *)data, (void *const *)mean, (void *const *)cov, &a.f))) return rc;
  a.ktab_d = w->ktab_d;
  const int pq[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  for (int t = 0; t < 6; t++) a.sig0d[t] = (double)w->sigma0f[pq[t][0] * 3 + pq[t][1]];
  a.tw = (const float2 *)twiddle_table<float>(nyp);
  if (!a.tw) return cuda_status(cudaGetLastError(), "twiddle table");
  a.mixed = precision == CG_PREC_MIXED;
  CG_CUDA(cudaMemsetAsync(w->counters, 0, sizeof(int), st));
  const long outband = plane * nzp - w->inband_bins;
  const double bytes = 8.0 * (w->inband_bins * (double)((nt + 3) + (nt + 3 + 6)) + outband * 6.0);
  rc = dispatch_nt(nt, [&](auto NTc) -> int {
    constexpr int NT = decltype(NTc)::value;
    int r = launch_bins_ys<NT>(a, cnxp, nzp, st, bytes);
    if (r || !a.mixed) return r;
    int dev = 0, nsm = 0;
    CG_CUDA(cudaGetDevice(&dev));
    CG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    TraceScope ts("k_ys_fixup64", st, 0.0);
    k_ys_fixup64<NT><<<nsm * 4, 128, 0, st>>>(a);
    CG_CHECK_LAUNCH("k_ys_fixup64");
    return CG_OK;
  });
  if (rc) return rc;
  if (bins_done) CG_CUDA(cudaEventRecord(bins_done, st));
  if ((rc = fft_cols<float>(mcubes, 3, nzp, cnxp, plane, cnxp, nyp, +1, st))) return rc;
  // the bin kernel's stage 2 pair is normalised: its factor 16 (a power of two) goes into the postscale
  return rows_ys(false, mcubes, 3, nzp, pre * (float)kYsN2, st);
}

}  // namespace cg
