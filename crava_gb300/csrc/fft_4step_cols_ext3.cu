// Four-step column passes for further 7-smooth lengths, part 3 (see fft_4step.cuh).
#include "fft_4step_launch.cuh"

namespace cg {

int four_step_cols_ext3(const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride, long batch_stride,
                        int nbatch, int sign, const float2 *tw, cudaStream_t st)
{
  switch (n) {
#define CG_COLS(NN) \
  case NN: return launch_cols_4s<NN, (NN <= 128 ? 3 : 2)>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    CG_COLS(18) CG_COLS(20) CG_COLS(27) CG_COLS(42) CG_COLS(49) CG_COLS(54) CG_COLS(81) CG_COLS(84) CG_COLS(126) CG_COLS(135) CG_COLS(175) CG_COLS(180) CG_COLS(243) CG_COLS(252) CG_COLS(288) CG_COLS(360) CG_COLS(405) CG_COLS(448) CG_COLS(450)
#undef CG_COLS
    default: return 0;
  }
}

}  // namespace cg
