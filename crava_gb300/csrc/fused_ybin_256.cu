// Fused y transform + bin loop kernels for y length 256 (see fused_ybin.cuh).
#include "fused_ybin.cuh"

namespace cg {

int launch_ybin_256(const YBinArgs &a, int nt, int tiles, int nzp, double bytes, cudaStream_t st)
{
  return launch_ybin_n<256>(a, nt, tiles, nzp, bytes, st);
}

}  // namespace cg
