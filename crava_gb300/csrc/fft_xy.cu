// Plane kernels for the x and y passes (fft_xy.cuh): cluster launches and the
// lengths they are instantiated for.
#include "fft_xy.cuh"
#include "trace.cuh"
#include "tuning.cuh"

namespace cg {

namespace {

cudaLaunchConfig_t cluster_config(int cl, dim3 grid, size_t smem, cudaStream_t st, cudaLaunchAttribute *attr)
{
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(kXYThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

template <int M, int NY, int CL>
int launch_xy(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nzp, float scale,
              cudaStream_t st, int epi)
{
  using G = XYGeom<M, NY, CL>;
  const float2 *twx = (const float2 *)twiddle_table<float>(2 * M);
  const float2 *twy = (const float2 *)twiddle_table<float>(NY);
  if (!twx || !twy) return cuda_status(cudaGetLastError(), "twiddle table");
  dim3 grid(CL, nzp, ncubes);
  // one read of the real rows and one write of the half spectra (or the reverse)
  const double bytes = (double)ncubes * nzp * NY * (2.0 * M * sizeof(float) + (M + 1.0) * sizeof(float2));
  static bool attr_fwd[64] = {}, attr_inv[64] = {};
  cudaError_t e;
  cudaLaunchAttribute attr[1];
  const cudaLaunchConfig_t cfg = cluster_config(CL, grid, G::SMEM, st, attr);
  if (forward) {
    e = smem_limit_once(k_xy_r2c<M, NY, CL>, G::SMEM, attr_fwd);
    if (e != cudaSuccess) return cuda_status(e, "k_xy_r2c attribute");
    TraceScope ts("k_xy_r2c", st, bytes);
    e = cudaLaunchKernelEx(&cfg, k_xy_r2c<M, NY, CL>, cs, twx, twy, scale);
  } else {
    e = smem_limit_once(k_yx_c2r<M, NY, CL>, G::SMEM, attr_inv);
    if (e != cudaSuccess) return cuda_status(e, "k_yx_c2r attribute");
    TraceScope ts("k_yx_c2r", st, bytes);
    e = cudaLaunchKernelEx(&cfg, k_yx_c2r<M, NY, CL>, cs, addend, twx, twy, scale, epi);
  }
  if (e != cudaSuccess) return cuda_status(e, forward ? "k_xy_r2c" : "k_yx_c2r");
  return 1;
}

}  // namespace

// The x and y passes of ncubes cubes as plane kernels when (nxp, nyp) has one and the tuning table selects it
// (CG_TUNE_XY_PLANE per nxp); 0 otherwise (the caller runs the separate passes).
int xy_planes(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nxp, int nyp, int nzp,
              float scale, cudaStream_t st, int epi)
{
  if (cg_tune_get(CG_TUNE_XY_PLANE, nxp) != 1) return 0;
  if (nxp == 256 && nyp == 256) return launch_xy<128, 256, 2>(forward, cs, addend, ncubes, nzp, scale, st, epi);
  return 0;
}

}  // namespace cg
