// Four-step column passes for further 7-smooth lengths, part 2 (see fft_4step.cuh).
#include "fft_4step_launch.cuh"

namespace cg {

int four_step_cols_ext2(const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride, long batch_stride,
                        int nbatch, int sign, const float2 *tw, cudaStream_t st)
{
  switch (n) {
#define CG_COLS(NN) \
  case NN: return launch_cols_4s<NN, (NN <= 128 ? 3 : 2)>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    CG_COLS(16) CG_COLS(21) CG_COLS(28) CG_COLS(40) CG_COLS(50) CG_COLS(56) CG_COLS(75) CG_COLS(98) CG_COLS(112) CG_COLS(140) CG_COLS(168) CG_COLS(189) CG_COLS(224) CG_COLS(270) CG_COLS(294) CG_COLS(350) CG_COLS(378) CG_COLS(441) CG_COLS(486)
#undef CG_COLS
    default: return 0;
  }
}

}  // namespace cg
