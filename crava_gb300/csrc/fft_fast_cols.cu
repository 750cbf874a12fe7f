// Specialised strided-column FFT passes (see fft_fast.cuh).
#include <cstdlib>

#include "fft_fast.cuh"
#include "tuning.cuh"
#include "trace.cuh"

namespace cg {

namespace {
constexpr int kW = 16;

// Resident-CTA target per length (tuning key CG_TUNE_COLS_MINB): 3 for lengths
// up to 256 (measured faster at 256 despite a small spill), 2 above.
int minb_for(int n) { return cg_tune_get(CG_TUNE_COLS_MINB, n); }

template <int N, int MINB>
int launch_v(const CubeSet &cs, int ncubes, int ncols, long axis_stride, long batch_stride, int nbatch, int sign,
             const float2 *tw, cudaStream_t st)
{
  const size_t smem = ((size_t)N * kW + N) * sizeof(float2);
  static bool attr_set[64] = {};
  cudaError_t e = smem_limit_once(k_fft_cols_fast<N, kW, MINB>, smem, attr_set);
  if (e != cudaSuccess) return cuda_status(e, "k_fft_cols_fast attribute");
  ColsGeom g;
  g.axis_stride = axis_stride;
  g.batch_stride = batch_stride;
  g.nfull = ncols / kW;
  g.ntail = ncols - g.nfull * kW;
  g.nbatch = nbatch;
  g.trows = 1;
  const int groups = ceil_div(nbatch, kW);
  const int tail_cols = g.ntail > 0 ? ceil_div((long)g.ntail * groups, nbatch) : 0;
  dim3 grid(g.nfull + tail_cols, nbatch, ncubes);
  TraceScope ts("k_fft_cols_fast", st, 2.0 * ncubes * nbatch * (double)ncols * N * sizeof(float2));
  k_fft_cols_fast<N, kW, MINB><<<grid, kFFTThreads, smem, st>>>(cs, tw, g, sign);
  CG_CHECK_LAUNCH("k_fft_cols_fast");
  return 1;
}

// persistent double-buffered variant: one CTA per resident slot, each walking
// the tile list (tuning key CG_TUNE_COLS_PIPE).  Off by default: on GB300 it
// measured 25-30 % slower than one CTA per tile at lengths 200 and 256.
bool use_pipe(int n) { return cg_tune_get(CG_TUNE_COLS_PIPE, n) == 1; }

template <int N, int MINB>
int launch_pipe(const CubeSet &cs, int ncubes, int ncols, long axis_stride, long batch_stride, int nbatch, int sign,
                const float2 *tw, cudaStream_t st)
{
  const size_t smem = (2 * (size_t)N * kW + N) * sizeof(float2);
  static bool attr_set[64] = {};
  static int slots[64] = {};
  cudaError_t e = smem_limit_once(k_fft_cols_pipe<N, kW, MINB>, smem, attr_set);
  if (e != cudaSuccess) return cuda_status(e, "k_fft_cols_pipe attribute");
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  int &nslots = slots[dev < 64 ? dev : 0];
  if (nslots == 0) {
    int per_sm = 0, nsm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fft_cols_pipe<N, kW, MINB>, kFFTThreads,
                                                           smem)) != cudaSuccess)
      return cuda_status(e, "occupancy");
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
      return cuda_status(e, "SM count");
    nslots = (per_sm > 0 ? per_sm : 1) * nsm;
  }
  ColsGeom g;
  g.axis_stride = axis_stride;
  g.batch_stride = batch_stride;
  g.nfull = ncols / kW;
  g.ntail = ncols - g.nfull * kW;
  g.nbatch = nbatch;
  g.trows = 1;
  const long groups = ceil_div(nbatch, kW);
  const long ntiles = (long)ncubes * ((long)nbatch * g.nfull + (long)g.ntail * groups);
  if (ntiles > 0x7fffffffL) { set_error("too many column tiles"); return CG_ERR_UNSUPPORTED; }
  const int grid = (int)(ntiles < nslots ? ntiles : nslots);
  TraceScope ts("k_fft_cols_pipe", st, 2.0 * ncubes * nbatch * (double)ncols * N * sizeof(float2));
  k_fft_cols_pipe<N, kW, MINB><<<grid, kFFTThreads, smem, st>>>(cs, tw, g, (int)ntiles, sign);
  CG_CHECK_LAUNCH("k_fft_cols_pipe");
  return 1;
}

// register-direct first and last stages (tuning: CG_TUNE_COLS_PIPE value 2)
template <int N, int MINB>
int launch_rd(const CubeSet &cs, int ncubes, int ncols, long axis_stride, long batch_stride, int nbatch, int sign,
              const float2 *tw, cudaStream_t st)
{
  const size_t smem = ((size_t)N * kW + N) * sizeof(float2);
  static bool attr_set[64] = {};
  cudaError_t e = smem_limit_once(k_fft_cols_rd<N, kW, MINB>, smem, attr_set);
  if (e != cudaSuccess) return cuda_status(e, "k_fft_cols_rd attribute");
  ColsGeom g;
  g.axis_stride = axis_stride;
  g.batch_stride = batch_stride;
  g.nfull = ncols / kW;
  g.ntail = ncols - g.nfull * kW;
  g.nbatch = nbatch;
  g.trows = 1;
  const int groups = ceil_div(nbatch, kW);
  const int tail_cols = g.ntail > 0 ? ceil_div((long)g.ntail * groups, nbatch) : 0;
  dim3 grid(g.nfull + tail_cols, nbatch, ncubes);
  TraceScope ts("k_fft_cols_rd", st, 2.0 * ncubes * nbatch * (double)ncols * N * sizeof(float2));
  k_fft_cols_rd<N, kW, MINB><<<grid, kFFTThreads, smem, st>>>(cs, tw, g, sign);
  CG_CHECK_LAUNCH("k_fft_cols_rd");
  return 1;
}

// register-direct on persistent CTAs with the next tile's loads in flight (tuning value 4)
template <int N, int MINB>
int launch_rdp(const CubeSet &cs, int ncubes, int ncols, long axis_stride, long batch_stride, int nbatch, int sign,
               const float2 *tw, cudaStream_t st)
{
  const size_t smem = ((size_t)N * kW + N) * sizeof(float2);
  static bool attr_set[64] = {};
  static int slots[64] = {};
  cudaError_t e = smem_limit_once(k_fft_cols_rdp<N, kW, MINB>, smem, attr_set);
  if (e != cudaSuccess) return cuda_status(e, "k_fft_cols_rdp attribute");
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  int &nslots = slots[dev < 64 ? dev : 0];
  if (nslots == 0) {
    int per_sm = 0, nsm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fft_cols_rdp<N, kW, MINB>, kFFTThreads, smem)) !=
        cudaSuccess)
      return cuda_status(e, "occupancy");
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
      return cuda_status(e, "SM count");
    nslots = (per_sm > 0 ? per_sm : 1) * nsm;
  }
  ColsGeom g;
  g.axis_stride = axis_stride;
  g.batch_stride = batch_stride;
  g.nfull = ncols / kW;
  g.ntail = ncols - g.nfull * kW;
  g.nbatch = nbatch;
  g.trows = 1;
  const long groups = ceil_div(nbatch, kW);
  const long ntiles = (long)ncubes * ((long)nbatch * g.nfull + (long)g.ntail * groups);
  if (ntiles > 0x7fffffffL) { set_error("too many column tiles"); return CG_ERR_UNSUPPORTED; }
  const int grid = (int)(ntiles < nslots ? ntiles : nslots);
  TraceScope ts("k_fft_cols_rdp", st, 2.0 * ncubes * nbatch * (double)ncols * N * sizeof(float2));
  k_fft_cols_rdp<N, kW, MINB><<<grid, kFFTThreads, smem, st>>>(cs, tw, g, (int)ntiles, sign);
  CG_CHECK_LAUNCH("k_fft_cols_rdp");
  return 1;
}

template <int N>
int launch(const CubeSet &cs, int ncubes, int ncols, long axis_stride, long batch_stride, int nbatch, int sign,
           const float2 *tw, cudaStream_t st, bool no_alloc)
{
  int kind = cg_tune_get(CG_TUNE_COLS_PIPE, N);
  if (kind == 5 && no_alloc) kind = 2;  // the TMA pass allocates its fault word on first use
  if (kind == 5) {
    // TMA-fed persistent pass (length 256 along y or z); the register-direct
    // kernel wherever its geometry or alignment does not fit
    if constexpr (N == 256) {
      const int rc = tma_cols(cs, ncubes, N, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
      if (rc != 0) return rc;
    }
    kind = 2;
  }
  if (kind == 4) {
    if (minb_for(N) == 3) return launch_rdp<N, 3>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    return launch_rdp<N, 2>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
  }
  if (kind == 3) return four_step_cols(minb_for(N), cs, ncubes, N, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
  if (kind == 2) {
    if constexpr (N <= 256)
      if (minb_for(N) == 4) return launch_rd<N, 4>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    if (minb_for(N) == 3) return launch_rd<N, 3>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    return launch_rd<N, 2>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
  }
  if (use_pipe(N)) {
    if (minb_for(N) == 3) return launch_pipe<N, 3>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    return launch_pipe<N, 2>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
  }
  if (minb_for(N) == 3) return launch_v<N, 3>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
  return launch_v<N, 2>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
}
}  // namespace

// Runs a whole column pass when the length has a specialisation; *done_cols
// receives how many columns were handled (all of them, or 0).
int fast_cols(const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride, long batch_stride, int nbatch,
              int sign, const float2 *tw, cudaStream_t st, int *done_cols, bool no_alloc)
{
  *done_cols = 0;
  if (ncols < 1) return 0;
  int rc = 0;
  switch (n) {
#define CG_COLS(NN) case NN: rc = launch<NN>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st, no_alloc); break;
    CG_COLS(64) CG_COLS(80) CG_COLS(96) CG_COLS(100) CG_COLS(120) CG_COLS(128) CG_COLS(160) CG_COLS(192)
    CG_COLS(200) CG_COLS(240) CG_COLS(256) CG_COLS(320) CG_COLS(384) CG_COLS(400) CG_COLS(480) CG_COLS(512)
#undef CG_COLS
    default:  // further lengths exist only as four-step kernels
      rc = four_step_cols(minb_for(n), cs, ncubes, n, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
      break;
  }
  if (rc == 1) *done_cols = ncols;
  return rc;
}

}  // namespace cg
