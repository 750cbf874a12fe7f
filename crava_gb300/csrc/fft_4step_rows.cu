// Four-step x-row R2C / C2R passes (see fft_4step.cuh).
#include "fft_4step.cuh"
#include "trace.cuh"

namespace cg {

namespace {
template <int M>
int launch(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nrows, float scale,
           const float2 *tw, cudaStream_t st, int epi)
{
  constexpr int RPC = fs_rows_per_cta(M), P = fs_row_pitch(M);
  const size_t smem = ((size_t)RPC * P + 2 * M) * sizeof(float2);
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
    e = smem_limit_once(k_c2r_rows_4s<M>, smem, attr_inv);
    if (e != cudaSuccess) return cuda_status(e, "k_c2r_rows_4s attribute");
    TraceScope ts("k_c2r_rows_4s", st, bytes);
    k_c2r_rows_4s<M><<<grid, kFFTThreads, smem, st>>>(cs, addend, tw, nrows, scale, epi);
  }
  CG_CHECK_LAUNCH(forward ? "k_r2c_rows_4s" : "k_c2r_rows_4s");
  return 1;
}
}  // namespace

// the x-row pass with the four-step kernels, or 0 when nxp/2 has no specialisation
int four_step_rows(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nxp, int nrows, float scale,
                   const float2 *tw, cudaStream_t st, int epi)
{
  if (nxp % 2) return 0;
  switch (nxp / 2) {
#define CG_ROWS(MM) case MM: return launch<MM>(forward, cs, addend, ncubes, nrows, scale, tw, st, epi);
    CG_ROWS(32) CG_ROWS(40) CG_ROWS(48) CG_ROWS(50) CG_ROWS(60) CG_ROWS(64) CG_ROWS(80) CG_ROWS(96)
    CG_ROWS(100) CG_ROWS(120) CG_ROWS(128) CG_ROWS(160) CG_ROWS(192) CG_ROWS(200) CG_ROWS(240) CG_ROWS(256)
#undef CG_ROWS
    default: return 0;
  }
}

}  // namespace cg
