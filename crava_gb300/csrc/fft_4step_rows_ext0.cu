// Four-step x-row passes for further half lengths, part 0 (see fft_4step.cuh).
#include "fft_4step_launch.cuh"

namespace cg {

int four_step_rows_ext0(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int m, int nrows,
                        float scale, const float2 *tw, cudaStream_t st, int epi)
{
  switch (m) {
#define CG_ROWS(MM) case MM: return launch_rows_4s<MM>(forward, cs, addend, ncubes, nrows, scale, tw, st, epi);
    CG_ROWS(20) CG_ROWS(27) CG_ROWS(30) CG_ROWS(42) CG_ROWS(49) CG_ROWS(72) CG_ROWS(84) CG_ROWS(90) CG_ROWS(125) CG_ROWS(126) CG_ROWS(144) CG_ROWS(175) CG_ROWS(180) CG_ROWS(210) CG_ROWS(252)
#undef CG_ROWS
    default: return 0;
  }
}

}  // namespace cg
