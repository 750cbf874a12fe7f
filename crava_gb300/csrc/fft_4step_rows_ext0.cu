// Four-step x-row passes for further even half lengths, part 0 (see fft_4step.cuh).
#include "fft_4step_launch.cuh"

namespace cg {

int four_step_rows_ext0(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int m, int nrows,
                        float scale, const float2 *tw, cudaStream_t st, int epi)
{
  switch (m) {
#define CG_ROWS(MM) case MM: return launch_rows_4s<MM>(forward, cs, addend, ncubes, nrows, scale, tw, st, epi);
    CG_ROWS(18) CG_ROWS(28) CG_ROWS(36) CG_ROWS(42) CG_ROWS(70) CG_ROWS(72) CG_ROWS(98) CG_ROWS(112) CG_ROWS(126) CG_ROWS(150) CG_ROWS(162) CG_ROWS(180) CG_ROWS(210) CG_ROWS(252)
#undef CG_ROWS
    default: return 0;
  }
}

}  // namespace cg
