// Library-internal entry of the fused inversion for the C++ host layer.
#pragma once

#include <cuda_runtime.h>

#include "cravagpu.h"

namespace cg {
// cg_invert_cubes_fused, recording bins_done (may be null) on the stream as soon
// as the residual and covariance spectra are final
int invert_cubes_fused(cg_workspace w, float *const *data, float *const *mean, float *const *cov, int precision,
                       void *stream, cudaEvent_t bins_done);
}  // namespace cg
