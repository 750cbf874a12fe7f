// Four-step strided-column passes (see fft_4step.cuh).
#include "fft_4step.cuh"
#include "trace.cuh"

namespace cg {

namespace {
template <int N, int MINB>
int launch(const CubeSet &cs, int ncubes, int ncols, long axis_stride, long batch_stride, int nbatch, int sign,
           const float2 *tw, cudaStream_t st)
{
  constexpr int W = fs_cols_w(N);
  const size_t smem = ((size_t)N * W + N) * sizeof(float2);
  static bool attr_set[64] = {};
  cudaError_t e = smem_limit_once(k_fft_cols_4s<N, W, MINB>, smem, attr_set);
  if (e != cudaSuccess) return cuda_status(e, "k_fft_cols_4s attribute");
  ColsGeom g;
  g.axis_stride = axis_stride;
  g.batch_stride = batch_stride;
  g.nfull = ncols / W;
  g.ntail = ncols - g.nfull * W;
  g.nbatch = nbatch;
  const int groups = ceil_div(nbatch, W);
  const int tail_cols = g.ntail > 0 ? ceil_div((long)g.ntail * groups, nbatch) : 0;
  dim3 grid(g.nfull + tail_cols, nbatch, ncubes);
  TraceScope ts("k_fft_cols_4s", st, 2.0 * ncubes * nbatch * (double)ncols * N * sizeof(float2));
  k_fft_cols_4s<N, W, MINB><<<grid, kFFTThreads, smem, st>>>(cs, tw, g, sign);
  CG_CHECK_LAUNCH("k_fft_cols_4s");
  return 1;
}

template <int N>
int launch_minb(int minb, const CubeSet &cs, int ncubes, int ncols, long axis_stride, long batch_stride, int nbatch,
                int sign, const float2 *tw, cudaStream_t st)
{
  if (minb == 3) return launch<N, 3>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
  return launch<N, 2>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
}
}  // namespace

// the whole column pass with the four-step kernel, or 0 when n has no specialisation
int four_step_cols(int minb, const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride, long batch_stride,
                   int nbatch, int sign, const float2 *tw, cudaStream_t st)
{
  switch (n) {
#define CG_COLS(NN) \
  case NN: return launch_minb<NN>(minb, cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    CG_COLS(64) CG_COLS(80) CG_COLS(96) CG_COLS(100) CG_COLS(120) CG_COLS(128) CG_COLS(160) CG_COLS(192)
    CG_COLS(200) CG_COLS(240) CG_COLS(256) CG_COLS(320) CG_COLS(384) CG_COLS(400) CG_COLS(480) CG_COLS(512)
#undef CG_COLS
    default: return 0;
  }
}

}  // namespace cg
