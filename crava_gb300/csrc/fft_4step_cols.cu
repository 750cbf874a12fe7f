// Four-step strided-column passes (see fft_4step.cuh): the tuned lengths
// (both resident-CTA targets) and the dispatch to the further lengths.
#include "fft_4step_launch.cuh"

namespace cg {

// the whole column pass with the four-step kernel, or 0 when n has no specialisation
int four_step_cols(int minb, const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride, long batch_stride,
                   int nbatch, int sign, const float2 *tw, cudaStream_t st)
{
  switch (n) {
#define CG_COLS(NN) \
  case NN: return launch_minb<NN>(minb, cs, ncubes, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
    CG_COLS(64) CG_COLS(80) CG_COLS(96) CG_COLS(100) CG_COLS(120) CG_COLS(128) CG_COLS(160) CG_COLS(192)
#undef CG_COLS
    default: break;
  }
  int rc;
  if ((rc = four_step_cols_main2(minb, cs, ncubes, n, ncols, axis_stride, batch_stride, nbatch, sign, tw, st))) return rc;
  if ((rc = four_step_cols_ext0(cs, ncubes, n, ncols, axis_stride, batch_stride, nbatch, sign, tw, st))) return rc;
  if ((rc = four_step_cols_ext1(cs, ncubes, n, ncols, axis_stride, batch_stride, nbatch, sign, tw, st))) return rc;
  if ((rc = four_step_cols_ext2(cs, ncubes, n, ncols, axis_stride, batch_stride, nbatch, sign, tw, st))) return rc;
  return four_step_cols_ext3(cs, ncubes, n, ncols, axis_stride, batch_stride, nbatch, sign, tw, st);
}

}  // namespace cg
