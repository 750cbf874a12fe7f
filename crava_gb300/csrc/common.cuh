// Shared device/host helpers for the GB300 AVO inversion library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cravagpu.h"

namespace cg {

// ---------------------------------------------------------------------------
// complex arithmetic on float2 / double2
// ---------------------------------------------------------------------------
template <typename T> struct cplx;
template <> struct cplx<float> { typedef float2 type; };
template <> struct cplx<double> { typedef double2 type; };

template <typename T> using C2 = typename cplx<T>::type;

template <typename T>
__host__ __device__ __forceinline__ C2<T> mk(T re, T im) { C2<T> r; r.x = re; r.y = im; return r; }
template <typename T>
__host__ __device__ __forceinline__ C2<T> cadd(C2<T> a, C2<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T>
__host__ __device__ __forceinline__ C2<T> csub(C2<T> a, C2<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T>
__host__ __device__ __forceinline__ C2<T> cmul(C2<T> a, C2<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T>
__host__ __device__ __forceinline__ C2<T> cmulc(C2<T> a, C2<T> b) {
  return mk<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename T>
__host__ __device__ __forceinline__ C2<T> cconj(C2<T> a) { return mk<T>(a.x, -a.y); }
template <typename T>
__host__ __device__ __forceinline__ C2<T> cscale(C2<T> a, T s) { return mk<T>(a.x * s, a.y * s); }

// Output epilogues of the inverse transform's last pass.  kEpiExp is
// FFTGrid::expTransf (src/fftgrid.cpp:1726-1743): every value but RMISSING
// becomes exp(value).
constexpr int kEpiNone = 0, kEpiExp = 1;
constexpr float kRMissing = -99999.0f;
template <typename T>
__device__ __forceinline__ T epilogue(T v, int epi)
{
  if (epi == kEpiExp && v != (T)kRMissing) {
    if constexpr (sizeof(T) == 4) return expf(v);
    else return exp(v);
  }
  return v;
}

// ---------------------------------------------------------------------------
// error plumbing for the C-ABI
// ---------------------------------------------------------------------------
void set_error(const char *fmt, ...);
int cuda_status(cudaError_t e, const char *where);
// stream-ordered allocation from the library's own per-device pool, which keeps its memory between calls
cudaError_t scratch_alloc(void **p, size_t bytes, cudaStream_t st);
// every memory allocation the library makes (device, pinned host, pools) calls this first (cg_alloc_calls)
void count_alloc();
cudaError_t dev_malloc(void **p, size_t bytes);  // cudaMalloc, counted

#define CG_CUDA(call)                                           \
  do {                                                          \
    cudaError_t e_ = (call);                                    \
    if (e_ != cudaSuccess) return ::cg::cuda_status(e_, #call); \
  } while (0)

#define CG_CHECK_LAUNCH(where)                                  \
  do {                                                          \
    cudaError_t e_ = cudaGetLastError();                        \
    if (e_ != cudaSuccess) return ::cg::cuda_status(e_, where); \
  } while (0)

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace cg
