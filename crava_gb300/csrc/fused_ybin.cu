// The fused inversion entry point (cg_invert_cubes_fused); kernel in fused_ybin.cuh.
#include <cstring>

#include "fused_ybin.cuh"
#include "fused_entry.h"

namespace cg {

// y lengths with a fused kernel, and whether the tuning table selects it
// (CG_TUNE_FUSED_Y; off by default: measured slower than the three passes
// around the stand-alone bin kernel at 256^3, see cg_tune_set)
static bool ybin_length(int n)
{
  return (n == 256 || n == 128 || n == 200) && cg_tune_get(CG_TUNE_FUSED_Y, n) == 1;
}

// Forward y pass, bins and inverse y pass per chunk of zc z-planes after one
// batched x + z pass: a chunk of the n + 3 spectra (zc * cnxp * nyp complex
// values each) is written by the y pass, read by the bin kernel and, for the
// three means, read again by the inverse y pass while it is still in L2.  An
// even zc keeps every chunk's first element 16-byte aligned.
static int chunked_y(cg_workspace w, float *const *data, float *const *mean, float *const *cov, int precision, int zc,
                     cudaStream_t st, cudaEvent_t bins_done)
{
  const int nt = w->ntheta, nxp = w->nxp, nyp = w->nyp, nzp = w->nzp;
  const int cnxp = nxp / 2 + 1;
  const long plane = (long)cnxp * nyp;  // complex values per z-plane
  int rc;
  void *fwd[kMaxTheta + 3];
  for (int l = 0; l < nt; l++) fwd[l] = data[l];
  for (int p = 0; p < 3; p++) fwd[nt + p] = mean[p];
  if ((rc = fft3d_xz<float>(fwd, nt + 3, nxp, nyp, nzp, CG_DATA, true, st))) return rc;
  if (precision == CG_PREC_MIXED) CG_CUDA(cudaMemsetAsync(w->counters, 0, sizeof(int), st));
  for (int k0 = 0; k0 < nzp; k0 += zc) {
    const int nk = nzp - k0 < zc ? nzp - k0 : zc;
    void *cf[kMaxTheta + 3], *cm[3];
    for (int i = 0; i < nt + 3; i++) cf[i] = (float2 *)fwd[i] + k0 * plane;
    for (int p = 0; p < 3; p++) cm[p] = (float2 *)mean[p] + k0 * plane;
    if ((rc = fft_cols<float>(cf, nt + 3, nyp, cnxp, cnxp, plane, nk, -1, st))) return rc;
    if ((rc = fused_bins_range(w, (void *const *)data, (void *const *)mean, (void *const *)cov, precision, k0, nk, true,
                               st)))
      return rc;
    if ((rc = fft_cols<float>(cm, 3, nyp, cnxp, cnxp, plane, nk, +1, st))) return rc;
  }
  if (bins_done) CG_CUDA(cudaEventRecord(bins_done, st));
  return fft3d_xz<float>((void *const *)mean, 3, nxp, nyp, nzp, CG_PARAMETER, false, st);
}

bool ysplit_fits(const Workspace *w);
int invert_cubes_ysplit(Workspace *w, float *const *data, float *const *mean, float *const *cov, int precision,
                        cudaStream_t st, cudaEvent_t bins_done);

}  // namespace cg

using namespace cg;

int cg::invert_cubes_fused(cg_workspace w, float *const *data, float *const *mean, float *const *cov, int precision,
                           void *stream, cudaEvent_t bins_done)
{
  int rc = check_ws(w);
  if (rc) return rc;
  if (!data || !mean || !cov) { set_error("null buffer argument"); return CG_ERR_ARG; }
  if (w->is4d) { set_error("the fused form needs a separable 3-parameter prior; use cg_invert_bins_plain for 4D"); return CG_ERR_UNSUPPORTED; }
  if (precision != CG_PREC_FP32 && precision != CG_PREC_MIXED) { set_error("precision %d not valid for FP32 buffers", precision); return CG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  const int nt = w->ntheta, nxp = w->nxp, nyp = w->nyp, nzp = w->nzp;
  void *fwd[kMaxTheta + 3];
  for (int l = 0; l < nt; l++) { if (!data[l]) { set_error("null data[%d]", l); return CG_ERR_ARG; } fwd[l] = data[l]; }
  for (int p = 0; p < 3; p++) { if (!mean[p]) { set_error("null mean[%d]", p); return CG_ERR_ARG; } fwd[nt + p] = mean[p]; }
  for (int t = 0; t < 6; t++) if (!cov[t]) { set_error("null cov[%d]", t); return CG_ERR_ARG; }
  const int zc = cg_tune_get(CG_TUNE_FUSED_Y, nyp);
  // the y-fused and y-split kernels take the separable prior only; a per-bin prior table (correlation
  // gradients) goes through the stand-alone bin kernels
  if (zc == 2 && ysplit_fits(w) && !w->sl_on) return invert_cubes_ysplit(w, data, mean, cov, precision, st, bins_done);
  if (zc >= 4 && nt + 3 <= kMaxBatch) return chunked_y(w, data, mean, cov, precision, zc, st, bins_done);
  if (!ybin_length(nyp) || w->sl_on) {
    // no fused kernel for this y length: three-pass transforms around the bin kernel
    if ((rc = fft3d<float>(fwd, nt + 3, nxp, nyp, nzp, CG_DATA, true, st))) return rc;
    if ((rc = cg_invert_bins_fused(w, data, mean, cov, precision, stream))) return rc;
    if (bins_done) CG_CUDA(cudaEventRecord(bins_done, st));
    return fft3d<float>((void *const *)mean, 3, nxp, nyp, nzp, CG_PARAMETER, false, st);
  }
  // DATA and PARAMETER share the 1/sqrt(N) forward scaling: one batched x + z pass over the n+3 cubes
  if ((rc = fft3d_xz<float>(fwd, nt + 3, nxp, nyp, nzp, CG_DATA, true, st))) return rc;
  YBinArgs a;
  memset(&a, 0, sizeof(a));
  rc = fill_fused_args(w, (void *const *)data, (void *const *)mean, (void *const *)cov, &a.f);
  if (rc) return rc;
  a.ktab_d = w->ktab_d;
  const int pq[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  for (int t = 0; t < 6; t++) a.sig0d[t] = (double)w->sigma0f[pq[t][0] * 3 + pq[t][1]];
  a.tw = (const float2 *)twiddle_table<float>(nyp);
  if (!a.tw) return cuda_status(cudaGetLastError(), "twiddle table");
  a.mixed = precision == CG_PREC_MIXED;
  CG_CUDA(cudaMemsetAsync(w->counters, 0, sizeof(int), st));
  const int tiles = ceil_div(a.f.cnxp, kYW);
  const double bytes = 8.0 * (double)a.f.plane * nzp * ((nt + 3) + (nt + 3 + 6));
  switch (nyp) {
    case 256: rc = launch_ybin_256(a, nt, tiles, nzp, bytes, st); break;
    case 200: rc = launch_ybin_200(a, nt, tiles, nzp, bytes, st); break;
    default: rc = launch_ybin_128(a, nt, tiles, nzp, bytes, st); break;
  }
  if (rc) return rc;
  if (bins_done) CG_CUDA(cudaEventRecord(bins_done, st));
  return fft3d_xz<float>((void *const *)mean, 3, nxp, nyp, nzp, CG_PARAMETER, false, st);
}

extern "C" int cg_invert_cubes_fused(cg_workspace w, float *const *data, float *const *mean, float *const *cov,
                                     int precision, void *stream)
{
  return cg::invert_cubes_fused(w, data, mean, cov, precision, stream, nullptr);
}
