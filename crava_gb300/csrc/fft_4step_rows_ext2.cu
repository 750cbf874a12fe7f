// Four-step x-row passes for further half lengths, part 2 (see fft_4step.cuh).
#include "fft_4step_launch.cuh"

namespace cg {

int four_step_rows_ext2(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int m, int nrows,
                        float scale, const float2 *tw, cudaStream_t st, int epi)
{
  switch (m) {
#define CG_ROWS(MM) case MM: return launch_rows_4s<MM>(forward, cs, addend, ncubes, nrows, scale, tw, st, epi);
    CG_ROWS(15) CG_ROWS(21) CG_ROWS(25) CG_ROWS(28) CG_ROWS(45) CG_ROWS(56) CG_ROWS(63) CG_ROWS(75) CG_ROWS(105) CG_ROWS(112) CG_ROWS(135) CG_ROWS(147) CG_ROWS(168) CG_ROWS(196) CG_ROWS(224) CG_ROWS(225)
#undef CG_ROWS
    default: return 0;
  }
}

}  // namespace cg
