// Four-step column passes for further 7-smooth lengths, part 0 (see fft_4step.cuh).
#include "fft_4step_launch.cuh"

namespace cg {

int four_step_cols_ext0(const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride, long batch_stride,
                        int nbatch, int sign, const float2 *tw, cudaStream_t st)
{
  switch (n) {
#define CG_COLS(NN) \
  case NN: return launch_cols_4s<NN, (NN <= 128 ? 3 : 2)>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    CG_COLS(25) CG_COLS(30) CG_COLS(36) CG_COLS(45) CG_COLS(63) CG_COLS(72) CG_COLS(90) CG_COLS(125) CG_COLS(147) CG_COLS(150) CG_COLS(210) CG_COLS(225) CG_COLS(250) CG_COLS(315) CG_COLS(324) CG_COLS(392) CG_COLS(420) CG_COLS(504)
#undef CG_COLS
    default: return 0;
  }
}

}  // namespace cg
