// Launch helpers of the four-step kernels (fft_4step.cuh), shared by the
// translation units that instantiate them for different lengths.
#pragma once

#include "fft_4step.cuh"
#include "trace.cuh"
#include "tuning.cuh"

namespace cg {

template <int N, int MINB, int SHAPE>
int launch_cols_4s_shape(const CubeSet &cs, int ncubes, int ncols, long axis_stride, long batch_stride, int nbatch,
                         int sign, const float2 *tw, cudaStream_t st)
{
  constexpr int W = fs_shape_w(N, SHAPE), N1 = fs_shape_n1(N, SHAPE);
  const size_t smem = ((size_t)N * W + N) * sizeof(float2);
  static bool attr_set[64] = {};
  cudaError_t e = smem_limit_once(k_fft_cols_4s<N, W, N1, MINB>, smem, attr_set);
  if (e != cudaSuccess) return cuda_status(e, "k_fft_cols_4s attribute");
  ColsGeom g;
  g.axis_stride = axis_stride;
  g.batch_stride = batch_stride;
  g.nfull = ncols / W;
  g.ntail = ncols - g.nfull * W;
  g.nbatch = nbatch;
  g.trows = 1;
  const long tail_tiles = ceil_div((long)g.ntail * nbatch, (long)W);
  const int tail_cols = (int)ceil_div(tail_tiles, (long)nbatch);
  dim3 grid(g.nfull + tail_cols, nbatch, ncubes);
  TraceScope ts("k_fft_cols_4s", st, 2.0 * ncubes * nbatch * (double)ncols * N * sizeof(float2));
  k_fft_cols_4s<N, W, N1, MINB><<<grid, kFFTThreads, smem, st>>>(cs, tw, g, sign);
  CG_CHECK_LAUNCH("k_fft_cols_4s");
  return 1;
}

// the tile shape the tuning table names for this length (0 when unset); a swap of equal factors is the default
template <int N, int MINB>
int launch_cols_4s(const CubeSet &cs, int ncubes, int ncols, long axis_stride, long batch_stride, int nbatch, int sign,
                   const float2 *tw, cudaStream_t st)
{
  int shape = cg_tune_get(CG_TUNE_COLS_SHAPE, N);
  if (fs_n1(N) * fs_n1(N) == N) shape &= 2;
  switch (shape) {
    case 1: return launch_cols_4s_shape<N, MINB, 1>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    case 2: return launch_cols_4s_shape<N, MINB, 2>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    case 3: return launch_cols_4s_shape<N, MINB, 3>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    default: return launch_cols_4s_shape<N, MINB, 0>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
  }
}

template <int M>
int launch_rows_4s(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nrows, float scale,
                   const float2 *tw, cudaStream_t st, int epi)
{
  constexpr int RPC = fs_rows_per_cta(M), P = fs_row_pitch(M);
  const size_t smem = ((size_t)RPC * P + 3 * M) * sizeof(float2);  // exchange, twiddles, pass-1 twiddles
  dim3 grid(ceil_div(nrows, RPC), 1, ncubes);
  const double bytes = (double)ncubes * nrows * (2.0 * M * sizeof(float) + (M + 1.0) * sizeof(float2));
  static bool attr_fwd[64] = {}, attr_inv[64] = {};
  cudaError_t e;
  if (forward) {
    e = smem_limit_once(k_r2c_rows_4s<M>, smem, attr_fwd);
    if (e != cudaSuccess) return cuda_status(e, "k_r2c_rows_4s attribute");
    TraceScope ts("k_r2c_rows_4s", st, bytes);
    k_r2c_rows_4s<M><<<grid, kFFTThreads, smem, st>>>(cs, tw, nrows, scale);
  } else {
    bool any_add = false;
    for (int i = 0; i < ncubes; i++) any_add = any_add || addend.ptr[i] != nullptr;
    if (any_add) {
      static bool attr_add[64] = {};
      e = smem_limit_once(k_c2r_rows_4s<M, true>, smem, attr_add);
      if (e != cudaSuccess) return cuda_status(e, "k_c2r_rows_4s attribute");
      // the addend is one more read of a row's 2(M+1) floats
      TraceScope ts("k_c2r_rows_4s", st, bytes + (double)ncubes * nrows * (M + 1.0) * sizeof(float2));
      k_c2r_rows_4s<M, true><<<grid, kFFTThreads, smem, st>>>(cs, addend, tw, nrows, scale, epi);
    } else {
      e = smem_limit_once(k_c2r_rows_4s<M, false>, smem, attr_inv);
      if (e != cudaSuccess) return cuda_status(e, "k_c2r_rows_4s attribute");
      TraceScope ts("k_c2r_rows_4s", st, bytes);
      k_c2r_rows_4s<M, false><<<grid, kFFTThreads, smem, st>>>(cs, addend, tw, nrows, scale, epi);
    }
  }
  CG_CHECK_LAUNCH(forward ? "k_r2c_rows_4s" : "k_c2r_rows_4s");
  return 1;
}

template <int NX>
int launch_rows_odd(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nrows, float scale,
                    const float2 *tw, cudaStream_t st, int epi)
{
  constexpr int RPC = fs_odd_rows_per_cta(NX), P = fs_odd_row_pitch(NX);
  const size_t smem = ((size_t)RPC * P + NX) * sizeof(float2);
  dim3 grid(ceil_div(nrows, RPC), 1, ncubes);
  const double bytes = (double)ncubes * nrows * (NX * sizeof(float) + (NX + 1) / 2 * sizeof(float2));
  static bool attr_fwd[64] = {}, attr_inv[64] = {};
  cudaError_t e;
  if (forward) {
    e = smem_limit_once(k_r2c_rows_odd<NX>, smem, attr_fwd);
    if (e != cudaSuccess) return cuda_status(e, "k_r2c_rows_odd attribute");
    TraceScope ts("k_r2c_rows_odd", st, bytes);
    k_r2c_rows_odd<NX><<<grid, kFFTThreads, smem, st>>>(cs, tw, nrows, scale);
  } else {
    e = smem_limit_once(k_c2r_rows_odd<NX>, smem, attr_inv);
    if (e != cudaSuccess) return cuda_status(e, "k_c2r_rows_odd attribute");
    TraceScope ts("k_c2r_rows_odd", st, bytes);
    k_c2r_rows_odd<NX><<<grid, kFFTThreads, smem, st>>>(cs, addend, tw, nrows, scale, epi);
  }
  CG_CHECK_LAUNCH(forward ? "k_r2c_rows_odd" : "k_c2r_rows_odd");
  return 1;
}

// the four-step column pass of a tuned length with the resident-CTA target minb
template <int N>
int launch_minb(int minb, const CubeSet &cs, int ncubes, int ncols, long axis_stride, long batch_stride, int nbatch,
                int sign, const float2 *tw, cudaStream_t st)
{
  if constexpr (N <= 256)
    if (minb == 4) return launch_cols_4s<N, 4>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
  if (minb == 3) return launch_cols_4s<N, 3>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
  return launch_cols_4s<N, 2>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
}

// tuned lengths 200..512 (fft_4step_cols_main2.cu): 0 when not handled
int four_step_cols_main2(int minb, const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride,
                         long batch_stride, int nbatch, int sign, const float2 *tw, cudaStream_t st);

// odd x lengths (fft_4step_rows_odd.cu): 0 when not handled
int four_step_rows_odd(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nxp, int nrows,
                       float scale, const float2 *tw, cudaStream_t st, int epi);

// further lengths (fft_4step_cols_ext*.cu, fft_4step_rows_ext*.cu): 0 when not handled
int four_step_cols_ext0(const CubeSet &, int, int, int, long, long, int, int, const float2 *, cudaStream_t);
int four_step_cols_ext1(const CubeSet &, int, int, int, long, long, int, int, const float2 *, cudaStream_t);
int four_step_cols_ext2(const CubeSet &, int, int, int, long, long, int, int, const float2 *, cudaStream_t);
int four_step_cols_ext3(const CubeSet &, int, int, int, long, long, int, int, const float2 *, cudaStream_t);
int four_step_rows_ext0(bool, const CubeSet &, const CubeSet &, int, int, int, float, const float2 *, cudaStream_t, int);
int four_step_rows_ext1(bool, const CubeSet &, const CubeSet &, int, int, int, float, const float2 *, cudaStream_t, int);
int four_step_rows_ext2(bool, const CubeSet &, const CubeSet &, int, int, int, float, const float2 *, cudaStream_t, int);

}  // namespace cg
