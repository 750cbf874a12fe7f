// Correlation cube fills (fill.cu) at either precision, for callers inside
// the library: R = float is the C-ABI's cg_fill_param_corr / cg_fill_err_corr.
#pragma once

#include "common.cuh"

namespace cg {

template <typename R>
int fill_param_corr(R *buf, int nxp, int nyp, int nzp, const float *corr_xy, const float *circ_corr_t, float grad_i,
                    float grad_j, R scalar, cudaStream_t st);
template <typename R>
int fill_err_corr(R *buf, int nxp, int nyp, int nzp, const float *corr_xy, float grad_i, float grad_j,
                  cudaStream_t st);

}  // namespace cg
