// Four-step column passes for further 7-smooth lengths, part 1 (see fft_4step.cuh).
#include "fft_4step_launch.cuh"

namespace cg {

int four_step_cols_ext1(const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride, long batch_stride,
                        int nbatch, int sign, const float2 *tw, cudaStream_t st)
{
  switch (n) {
#define CG_COLS(NN) \
  case NN: return launch_cols_4s<NN, (NN <= 128 ? 3 : 2)>(cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    CG_COLS(24) CG_COLS(32) CG_COLS(35) CG_COLS(48) CG_COLS(60) CG_COLS(70) CG_COLS(105) CG_COLS(108) CG_COLS(144) CG_COLS(162) CG_COLS(196) CG_COLS(216) CG_COLS(280) CG_COLS(300) CG_COLS(336) CG_COLS(375) CG_COLS(432) CG_COLS(500)
#undef CG_COLS
    default: return 0;
  }
}

}  // namespace cg
