// Host side of the TMA-fed column pass (kernel in fft_tma.cuh): tensor maps
// over the super-row view of each cube, the persistent grid, and the device
// word a kernel sets when one of its waits gives up (cg_device_faults).
#include <cstdint>
#include <cstring>
#include <mutex>

#include "fft_tma.cuh"
#include "trace.cuh"

namespace cg {

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  return fn;
}

// 8-byte elements, dims (2 cnxp, nyp/2, nzp), strides (16 cnxp, 8 cnxp nyp) bytes
bool encode_super_rows(EncodeTiledFn fn, CUtensorMap *map, void *base, long cnxp, int nyp, int nzp, unsigned bx,
                       unsigned by, unsigned bz)
{
  const cuuint64_t dims[3] = {(cuuint64_t)(2 * cnxp), (cuuint64_t)(nyp / 2), (cuuint64_t)nzp};
  const cuuint64_t strides[2] = {(cuuint64_t)(16 * cnxp), (cuuint64_t)(8 * cnxp * nyp)};
  const cuuint32_t box[3] = {bx, by, bz}, estr[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

std::mutex g_fault_mu;
int *g_fault[64] = {};

}  // namespace

// the current device's fault word (allocated and zeroed on first use)
int *device_fault_word()
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_fault_mu);
  if (!g_fault[dev]) {
    int *p = nullptr;
    count_alloc();
    if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, sizeof(int)) != cudaSuccess) { cudaFree(p); return nullptr; }
    g_fault[dev] = p;
  }
  return g_fault[dev];
}

// The column pass of length 256 along y or z through k_fft_cols_tma.  Returns
// 1 when launched, 0 when the geometry, alignment or driver does not allow it
// (the caller then uses the register-direct kernel), < 0 on a launch error.
int tma_cols(const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride, long batch_stride, int nbatch,
             int sign, const float2 *tw, cudaStream_t st)
{
  if (n != kTmaN || ncubes < 1 || ncubes > kMaxBatch || ncols < 1 || nbatch < 1) return 0;
  int axis, nyp, nzp;
  if (axis_stride == ncols && batch_stride == (long)ncols * n) {
    axis = 0, nyp = n, nzp = nbatch;
  } else if (batch_stride == ncols && axis_stride == (long)ncols * nbatch) {
    axis = 1, nyp = nbatch, nzp = n;
  } else {
    return 0;
  }
  if (nyp % 2) return 0;
  for (int i = 0; i < ncubes; i++)
    if (!cs.ptr[i] || (uintptr_t)cs.ptr[i] % 16) return 0;
  EncodeTiledFn fn = encode_fn();
  int *fault = device_fault_word();
  if (!fn || !fault) return 0;
  const long cnxp = ncols;
  const int sh = (int)(cnxp & 1);
  ColsTmaArgs a;  // copied into the launch's parameters
  memset(&a, 0, sizeof(a));
  for (int i = 0; i < ncubes; i++) {
    a.ptr[i] = (float2 *)cs.ptr[i];
    bool ok;
    if (axis == 0)
      ok = encode_super_rows(fn, &a.mapA[i], cs.ptr[i], cnxp, nyp, nzp, 16, nyp / 2, 1) &&
           encode_super_rows(fn, &a.mapB[i], cs.ptr[i], cnxp, nyp, nzp, 16 + 2 * sh, nyp / 2, 1);
    else
      ok = encode_super_rows(fn, &a.mapA[i], cs.ptr[i], cnxp, nyp, nzp, 16, 1, nzp);
    if (!ok) return 0;
  }
  a.plane = cnxp * nyp;
  a.cnxp = (int)cnxp;
  a.nyp = nyp;
  a.nbatch = nbatch;
  a.ngroups = (int)(axis == 0 ? (cnxp + 15) / 16 : (cnxp + sh + 15) / 16);
  const long ntiles = (long)ncubes * nbatch * a.ngroups;
  if (ntiles > (1L << 30)) return 0;
  a.ntiles = (int)ntiles;
  a.fault = fault;
  const size_t smem = (size_t)2 * kTmaBuf * sizeof(float2) + kTmaN * sizeof(float2) + 128;
  static bool attr0[64] = {}, attr1[64] = {};
  cudaError_t e = axis == 0 ? smem_limit_once(k_fft_cols_tma<0>, smem, attr0) : smem_limit_once(k_fft_cols_tma<1>, smem, attr1);
  if (e != cudaSuccess) return cuda_status(e, "k_fft_cols_tma attribute");
  int dev = 0, nsm = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess || (e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return cuda_status(e, "device query");
  e = axis == 0 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fft_cols_tma<0>, kFFTThreads, smem)
                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fft_cols_tma<1>, kFFTThreads, smem);
  if (e != cudaSuccess) return cuda_status(e, "occupancy");
  if (per_sm < 1) return 0;
  const long grid = ntiles < (long)per_sm * nsm ? ntiles : (long)per_sm * nsm;
  TraceScope ts("k_fft_cols_tma", st, 2.0 * ncubes * nbatch * (double)ncols * n * sizeof(float2));
  if (axis == 0) k_fft_cols_tma<0><<<(unsigned)grid, kFFTThreads, smem, st>>>(a, tw, sign);
  else k_fft_cols_tma<1><<<(unsigned)grid, kFFTThreads, smem, st>>>(a, tw, sign);
  CG_CHECK_LAUNCH("k_fft_cols_tma");
  return 1;
}

}  // namespace cg

using namespace cg;

extern "C" int cg_device_faults(int *flag)
{
  if (!flag) { set_error("null argument"); return CG_ERR_ARG; }
  int *w = device_fault_word();
  if (!w) { set_error("no device fault word"); return CG_ERR_CUDA; }
  cudaError_t e = cudaMemcpy(flag, w, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(w, 0, sizeof(int));
  return e == cudaSuccess ? CG_OK : cuda_status(e, "cg_device_faults");
}
