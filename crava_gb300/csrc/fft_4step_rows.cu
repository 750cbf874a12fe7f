// Four-step x-row R2C / C2R passes (see fft_4step.cuh): the tuned half
// lengths and the dispatch to the further ones.
#include "fft_4step_launch.cuh"

namespace cg {

// the x-row pass with the four-step kernels, or 0 when nxp/2 has no specialisation
int four_step_rows(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nxp, int nrows, float scale,
                   const float2 *tw, cudaStream_t st, int epi)
{
  if (nxp % 2) return four_step_rows_odd(forward, cs, addend, ncubes, nxp, nrows, scale, tw, st, epi);
  const int m = nxp / 2;
  switch (m) {
#define CG_ROWS(MM) case MM: return launch_rows_4s<MM>(forward, cs, addend, ncubes, nrows, scale, tw, st, epi);
    CG_ROWS(32) CG_ROWS(40) CG_ROWS(48) CG_ROWS(50) CG_ROWS(60) CG_ROWS(64) CG_ROWS(80) CG_ROWS(96)
    CG_ROWS(100) CG_ROWS(120) CG_ROWS(128) CG_ROWS(160) CG_ROWS(192) CG_ROWS(200) CG_ROWS(240) CG_ROWS(256)
#undef CG_ROWS
    default: break;
  }
  int rc;
  if ((rc = four_step_rows_ext0(forward, cs, addend, ncubes, m, nrows, scale, tw, st, epi))) return rc;
  if ((rc = four_step_rows_ext1(forward, cs, addend, ncubes, m, nrows, scale, tw, st, epi))) return rc;
  return four_step_rows_ext2(forward, cs, addend, ncubes, m, nrows, scale, tw, st, epi);
}

}  // namespace cg
