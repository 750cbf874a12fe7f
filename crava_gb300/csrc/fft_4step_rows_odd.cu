// Four-step x-row passes for odd x lengths (see fft_4step.cuh).
#include "fft_4step_launch.cuh"

namespace cg {

int four_step_rows_odd(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nxp, int nrows,
                       float scale, const float2 *tw, cudaStream_t st, int epi)
{
  switch (nxp) {
#define CG_ROWS(NN) case NN: return launch_rows_odd<NN>(forward, cs, addend, ncubes, nrows, scale, tw, st, epi);
    CG_ROWS(15) CG_ROWS(21) CG_ROWS(25) CG_ROWS(27) CG_ROWS(35) CG_ROWS(45) CG_ROWS(49) CG_ROWS(63) CG_ROWS(75)
    CG_ROWS(81) CG_ROWS(105) CG_ROWS(125) CG_ROWS(135) CG_ROWS(147) CG_ROWS(175) CG_ROWS(189) CG_ROWS(225)
    CG_ROWS(243)
#undef CG_ROWS
    default: return 0;
  }
}

}  // namespace cg
