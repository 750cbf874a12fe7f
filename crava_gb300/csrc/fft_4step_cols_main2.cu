// Four-step strided-column passes of the tuned lengths 200..512 (a second
// translation unit, compiled in parallel with fft_4step_cols.cu).
#include "fft_4step_launch.cuh"

namespace cg {

int four_step_cols_main2(int minb, const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride,
                         long batch_stride, int nbatch, int sign, const float2 *tw, cudaStream_t st)
{
  switch (n) {
#define CG_COLS(NN) \
  case NN: return launch_minb<NN>(minb, cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    CG_COLS(200) CG_COLS(240) CG_COLS(256) CG_COLS(320) CG_COLS(384) CG_COLS(400) CG_COLS(480) CG_COLS(512)
#undef CG_COLS
    default: return 0;
  }
}

}  // namespace cg
