// Four-step x-row passes for further half lengths, part 1 (see fft_4step.cuh).
#include "fft_4step_launch.cuh"

namespace cg {

int four_step_rows_ext1(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int m, int nrows,
                        float scale, const float2 *tw, cudaStream_t st, int epi)
{
  switch (m) {
#define CG_ROWS(MM) case MM: return launch_rows_4s<MM>(forward, cs, addend, ncubes, nrows, scale, tw, st, epi);
    CG_ROWS(16) CG_ROWS(18) CG_ROWS(24) CG_ROWS(35) CG_ROWS(36) CG_ROWS(54) CG_ROWS(70) CG_ROWS(81) CG_ROWS(98) CG_ROWS(108) CG_ROWS(140) CG_ROWS(150) CG_ROWS(162) CG_ROWS(189) CG_ROWS(216) CG_ROWS(243)
#undef CG_ROWS
    default: return 0;
  }
}

}  // namespace cg
