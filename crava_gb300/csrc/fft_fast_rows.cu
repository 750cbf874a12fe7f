// Specialised x-row R2C / C2R passes (see fft_fast.cuh).
#include "fft_fast.cuh"
#include "trace.cuh"
#include "tuning.cuh"
#include "cravagpu.h"

namespace cg {

namespace {
template <int M>
int launch(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nrows, float scale,
           const float2 *tw, cudaStream_t st, int epi)
{
  constexpr int LDW = kRows + 1;
  const size_t smem = ((size_t)M * LDW + 2 * M) * sizeof(float2);
  dim3 grid(ceil_div(nrows, kRows), 1, ncubes);
  const double bytes = (double)ncubes * nrows * (2.0 * M * sizeof(float) + (M + 1.0) * sizeof(float2));
  static bool attr_fwd[64] = {}, attr_inv[64] = {};
  cudaError_t e;
  if (forward) {
    e = smem_limit_once(k_r2c_rows_fast<M>, smem, attr_fwd);
    if (e != cudaSuccess) return cuda_status(e, "k_r2c_rows_fast attribute");
    TraceScope ts("k_r2c_rows_fast", st, bytes);
    k_r2c_rows_fast<M><<<grid, kFFTThreads, smem, st>>>(cs, tw, nrows, scale);
  } else {
    e = smem_limit_once(k_c2r_rows_fast<M>, smem, attr_inv);
    if (e != cudaSuccess) return cuda_status(e, "k_c2r_rows_fast attribute");
    TraceScope ts("k_c2r_rows_fast", st, bytes);
    k_c2r_rows_fast<M><<<grid, kFFTThreads, smem, st>>>(cs, addend, tw, nrows, scale, epi);
  }
  CG_CHECK_LAUNCH(forward ? "k_r2c_rows_fast" : "k_c2r_rows_fast");
  return 1;
}
}  // namespace

// Runs the x-row pass when nxp is even and nxp/2 has a specialisation.
int fast_rows(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nxp, int nrows, float scale,
              const float2 *tw, cudaStream_t st, int epi)
{
  if (nxp % 2)  // odd x lengths exist only as four-step kernels (tuning key n = nxp)
    return cg_tune_get(CG_TUNE_ROWS_KERNEL, nxp) == 1 ? four_step_rows(forward, cs, addend, ncubes, nxp, nrows, scale, tw, st, epi) : 0;
  if (cg_tune_get(CG_TUNE_ROWS_KERNEL, nxp / 2) == 1)
    return four_step_rows(forward, cs, addend, ncubes, nxp, nrows, scale, tw, st, epi);
  switch (nxp / 2) {
#define CG_ROWS(MM) case MM: return launch<MM>(forward, cs, addend, ncubes, nrows, scale, tw, st, epi);
    CG_ROWS(32) CG_ROWS(40) CG_ROWS(48) CG_ROWS(50) CG_ROWS(60) CG_ROWS(64) CG_ROWS(80) CG_ROWS(96)
    CG_ROWS(100) CG_ROWS(120) CG_ROWS(128) CG_ROWS(160) CG_ROWS(192) CG_ROWS(200) CG_ROWS(240) CG_ROWS(256)
#undef CG_ROWS
    default: return 0;
  }
}

}  // namespace cg
