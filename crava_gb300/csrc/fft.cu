// Mixed-radix (2/3/4/5/7/8) 3D real<->complex FFT for padded FFTGrid cubes.
//
// A 3D transform is three passes over HBM:
//   forward:  x rows R2C (prescale fused) -> y columns C2C -> z columns C2C
//   inverse:  z columns C2C -> y columns C2C -> x rows C2R (postscale fused)
// which is the order FFTW 2's rfftwnd uses (libs/fft/rfftw/rfftwnd.c:299-400),
// so the result of a C2R on a spectrum that is not Hermitian on the x=0 and
// x=nxp/2 planes matches the reference: only the real part of those bins
// survives the last (x) pass, as in rfftw_c2hc (libs/fft/rfftw/rexec2.c:214).
//
// Each pass stages a tile in shared memory and runs Stockham autosort stages
// on it (every butterfly reads stride n/R, writes the expanded index, two
// ping-pong buffers).  Tiles are laid out [axis index][column] so a warp's
// shared-memory accesses are conflict free, and global loads/stores are
// row segments of 16 complex (128 B) for the strided passes and whole rows
// for the x pass.  Twiddles come from a table computed in double on the host.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "fft.cuh"
#include "fft_fast.cuh"
#include "trace.cuh"

namespace cg {

// ---------------------------------------------------------------------------
// plans and twiddle tables
// ---------------------------------------------------------------------------
bool make_axis_plan(int n, AxisPlan *p)
{
  if (n < 1 || n > kMaxFFT) return false;
  p->n = n;
  p->nstages = 0;
  int m = n;
  while (m % 8 == 0) { p->radix[p->nstages++] = 8; m /= 8; }
  while (m % 4 == 0) { p->radix[p->nstages++] = 4; m /= 4; }
  while (m % 2 == 0) { p->radix[p->nstages++] = 2; m /= 2; }
  while (m % 3 == 0) { p->radix[p->nstages++] = 3; m /= 3; }
  while (m % 5 == 0) { p->radix[p->nstages++] = 5; m /= 5; }
  while (m % 7 == 0) { p->radix[p->nstages++] = 7; m /= 7; }
  return m == 1;
}

namespace {
std::mutex g_tw_mutex;
std::map<long, void *> g_tw_cache;  // key: (device, n, element size)
}

// Device table tw[t] = exp(-2*pi*i*t/n), t in [0, n), computed in double.
template <typename T>
const C2<T> *twiddle_table(int n)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  long key = ((long)dev << 40) | ((long)n << 8) | (long)sizeof(T);
  std::lock_guard<std::mutex> lk(g_tw_mutex);
  auto it = g_tw_cache.find(key);
  if (it != g_tw_cache.end()) return (const C2<T> *)it->second;
  std::vector<C2<T>> h(n);
  for (int t = 0; t < n; t++) {
    // reduce t/n to the first octant-free form: angle = 2*pi*t/n exactly in double
    double a = -2.0 * M_PI * (double)t / (double)n;
    h[t] = mk<T>((T)cos(a), (T)sin(a));
  }
  void *d = nullptr;
  count_alloc();
  if (cudaMalloc(&d, sizeof(C2<T>) * (size_t)n) != cudaSuccess) return nullptr;
  if (cudaMemcpy(d, h.data(), sizeof(C2<T>) * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    return nullptr;
  }
  g_tw_cache[key] = d;
  return (const C2<T> *)d;
}
template const C2<float> *twiddle_table<float>(int);
template const C2<double> *twiddle_table<double>(int);

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
// asynchronous global -> shared copy of one complex element (8 or 16 bytes)
template <typename T>
__device__ __forceinline__ void cp_async_elem(C2<T> *dst, const C2<T> *src)
{
  if constexpr (sizeof(T) == 4) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
  }
}

template <typename T>
__device__ __forceinline__ void cp_async_real(T *dst, const T *src)
{
  if constexpr (sizeof(T) == 4) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
  }
}

// the C2R row kernel stages kRows whole rows in bufB, so bufB holds
// max(m*(kRows+1), kRows*cnxp) elements
__host__ __device__ inline size_t c2r_bufb_elems(int m, int cnxp)
{
  size_t a = (size_t)m * (kRows + 1), b = (size_t)kRows * cnxp;
  return a > b ? a : b;
}

template <typename T>
__global__ void __launch_bounds__(kFFTThreads) k_fft_cols(const __grid_constant__ CubeSet cs, const __grid_constant__ AxisPlan p, const C2<T> *__restrict__ twg,
                                                          int col0, int ncols, int wfull, int ntiles,
                                                          long axis_stride, long batch_stride, int sign)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = p.n;
  const int wmax = wfull + 1;
  C2<T> *bufA = (C2<T> *)smem_raw;
  C2<T> *bufB = bufA + (size_t)n * wmax;
  C2<T> *tw = bufB + (size_t)n * wmax;
  const int tile = blockIdx.x;
  const int c0 = tile * wfull;
  const int width = (tile == ntiles - 1) ? (ncols - c0) : wfull;
  C2<T> *base = (C2<T> *)cs.ptr[blockIdx.z] + (long)blockIdx.y * batch_stride + col0 + c0;

  for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = twg[t];
  const int tot = n * width;
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    int e = t / width, c = t - e * width;
    cp_async_elem<T>(&bufA[e * width + c], &base[(long)e * axis_stride + c]);
  }
  cp_async_wait_all();
  __syncthreads();
  C2<T> *res = smem_fft<T>(bufA, bufB, p, width, width, tw, 1, sign);
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    int e = t / width, c = t - e * width;
    base[(long)e * axis_stride + c] = res[e * width + c];
  }
}

// x rows, real -> half spectrum, prescale fused into the load.
template <typename T>
__global__ void __launch_bounds__(kFFTThreads) k_r2c_rows(const __grid_constant__ CubeSet cs, const __grid_constant__ AxisPlan p, const C2<T> *__restrict__ twg,
                                                          int nxp, int nrows, T prescale)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int m = p.n;  // nxp/2 (even nxp) or nxp (odd)
  const int ldw = kRows + 1;
  const bool even = (nxp % 2) == 0;
  const int cnxp = nxp / 2 + 1, rnxp = 2 * cnxp;
  C2<T> *bufA = (C2<T> *)smem_raw;
  C2<T> *bufB = bufA + (size_t)m * ldw;
  C2<T> *tw = bufB + (size_t)m * ldw;
  const int r0 = blockIdx.x * kRows;
  const int nr = min(kRows, nrows - r0);
  T *base = (T *)cs.ptr[blockIdx.z] + (long)r0 * rnxp;

  for (int t = threadIdx.x; t < nxp; t += blockDim.x) tw[t] = twg[t];
  const int tot = kRows * m;
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    int row = t / m, e = t - row * m;
    if (row < nr) {
      if (even) {
        cp_async_elem<T>(&bufA[e * ldw + row], (const C2<T> *)(base + (long)row * rnxp) + e);
      } else {
        bufA[e * ldw + row].y = (T)0;
        cp_async_real<T>(&bufA[e * ldw + row].x, base + (long)row * rnxp + e);
      }
    } else {
      bufA[e * ldw + row] = mk<T>(0, 0);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  C2<T> *res = smem_fft<T>(bufA, bufB, p, kRows, ldw, tw, even ? 2 : 1, -1);
  const int tot2 = nr * cnxp;
  for (int t = threadIdx.x; t < tot2; t += blockDim.x) {
    int row = t / cnxp, k = t - row * cnxp;
    C2<T> X;
    if (even) {
      C2<T> A = res[(k == m ? 0 : k) * ldw + row];
      C2<T> B = cconj<T>(res[(k == 0 ? 0 : m - k) * ldw + row]);
      C2<T> E = mk<T>((A.x + B.x) * (T)0.5, (A.y + B.y) * (T)0.5);
      // O = -i (A - B) / 2
      C2<T> O = mk<T>((A.y - B.y) * (T)0.5, -(A.x - B.x) * (T)0.5);
      X = cadd<T>(E, cmul<T>(tw[k], O));
    } else {
      X = res[k * ldw + row];
    }
    X.x *= prescale;  // the transform is linear: scaling the output equals scaling the input
    X.y *= prescale;
    ((C2<T> *)(base + (long)row * rnxp))[k] = X;
  }
}

// x rows, half spectrum -> real, postscale fused into the store.
template <typename T>
__global__ void __launch_bounds__(kFFTThreads) k_c2r_rows(const __grid_constant__ CubeSet cs, const __grid_constant__ CubeSet addend, const __grid_constant__ AxisPlan p,
                                                          const C2<T> *__restrict__ twg, int nxp, int nrows,
                                                          T postscale, int epi)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int m = p.n;
  const int ldw = kRows + 1;
  const bool even = (nxp % 2) == 0;
  const int cnxp = nxp / 2 + 1, rnxp = 2 * cnxp;
  C2<T> *bufA = (C2<T> *)smem_raw;
  C2<T> *bufB = bufA + (size_t)m * ldw;
  C2<T> *tw = bufB + c2r_bufb_elems(m, cnxp);
  C2<T> *S = bufB;  // row staging (kRows x cnxp), dead once bufA is filled
  const int r0 = blockIdx.x * kRows;
  const int nr = min(kRows, nrows - r0);
  T *base = (T *)cs.ptr[blockIdx.z] + (long)r0 * rnxp;

  for (int t = threadIdx.x; t < nxp; t += blockDim.x) tw[t] = twg[t];
  for (int t = threadIdx.x; t < nr * cnxp; t += blockDim.x) {
    int row = t / cnxp, k = t - row * cnxp;
    cp_async_elem<T>(&S[row * cnxp + k], (const C2<T> *)(base + (long)row * rnxp) + k);
  }
  cp_async_wait_all();
  __syncthreads();
  // rfftw_c2hc keeps only the real part of the DC and (even nxp) Nyquist bins
  for (int row = threadIdx.x; row < nr; row += blockDim.x) {
    S[row * cnxp].y = (T)0;
    if (even) S[row * cnxp + cnxp - 1].y = (T)0;
  }
  __syncthreads();
  const int tot = kRows * m;
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    int row = t / m, k = t - row * m;
    C2<T> Z = mk<T>(0, 0);
    if (row < nr) {
      if (even) {
        C2<T> Xk = S[row * cnxp + k];
        C2<T> Xm = cconj<T>(S[row * cnxp + (m - k)]);
        C2<T> E = cadd<T>(Xk, Xm);
        C2<T> O = cmulc<T>(csub<T>(Xk, Xm), tw[k]);  // (Xk - conj X[m-k]) * W^-k
        Z = mk<T>(E.x - O.y, E.y + O.x);              // E + i O
      } else {
        Z = (k < cnxp) ? S[row * cnxp + k] : cconj<T>(S[row * cnxp + (m - k)]);
      }
    }
    bufA[k * ldw + row] = Z;
  }
  __syncthreads();
  C2<T> *res = smem_fft<T>(bufA, bufB, p, kRows, ldw, tw, even ? 2 : 1, +1);
  // optional fused FFTGrid::add of a real cube (src/fftgrid.cpp:1870-1891)
  const T *add = addend.ptr[blockIdx.z] ? (const T *)addend.ptr[blockIdx.z] + (long)r0 * rnxp : nullptr;
  if (even) {
    const int tot2 = nr * (m + 1);
    for (int t = threadIdx.x; t < tot2; t += blockDim.x) {
      int row = t / (m + 1), e = t - row * (m + 1);
      C2<T> z = (e < m) ? res[e * ldw + row] : mk<T>(0, 0);
      z = mk<T>(z.x * postscale, z.y * postscale);
      if (add) {
        const C2<T> a = ((const C2<T> *)(add + (long)row * rnxp))[e];
        z.x += a.x;
        z.y += a.y;
      }
      z.x = epilogue<T>(z.x, epi);
      z.y = epilogue<T>(z.y, epi);
      ((C2<T> *)(base + (long)row * rnxp))[e] = z;
    }
  } else {
    const int tot2 = nr * rnxp;
    for (int t = threadIdx.x; t < tot2; t += blockDim.x) {
      int row = t / rnxp, e = t - row * rnxp;
      T v = (e < nxp) ? res[e * ldw + row].x * postscale : (T)0;
      if (add) v += add[(long)row * rnxp + e];
      base[(long)row * rnxp + e] = epilogue<T>(v, epi);
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

template <typename T>
int launch_rows(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nxp, int nyp, int nzp,
                T scale, cudaStream_t st, int epi = kEpiNone)
{
  const bool even = (nxp % 2) == 0;
  const int m = even ? nxp / 2 : nxp;
  AxisPlan p;
  if (!make_axis_plan(m, &p)) {
    set_error("x length %d has a prime factor above 7 or exceeds %d", nxp, kMaxFFT);
    return CG_ERR_UNSUPPORTED;
  }
  const C2<T> *tw = twiddle_table<T>(nxp);
  if (!tw) return cuda_status(cudaGetLastError(), "twiddle table");
  const int nrows = nyp * nzp;
  if constexpr (sizeof(T) == 4) {
    const int rc = fast_rows(forward, cs, addend, ncubes, nxp, nrows, (float)scale, (const float2 *)tw, st, epi);
    if (rc < 0) return rc;
    if (rc == 1) return CG_OK;
  }
  const size_t bufb = forward ? (size_t)m * (kRows + 1) : c2r_bufb_elems(m, nxp / 2 + 1);
  size_t smem = ((size_t)m * (kRows + 1) + bufb + (size_t)nxp) * sizeof(C2<T>);
  if (smem > kMaxSmem) {
    set_error("x length %d needs %zu bytes of shared memory per tile (limit %zu)", nxp, smem, (size_t)kMaxSmem);
    return CG_ERR_UNSUPPORTED;
  }
  dim3 grid(ceil_div(nrows, kRows), 1, ncubes);
  const int cnxp = nxp / 2 + 1;
  TraceScope ts(forward ? "k_r2c_rows" : "k_c2r_rows", st,
                (double)ncubes * nrows * ((double)nxp * sizeof(T) + (double)cnxp * sizeof(C2<T>)));
  if (forward) {
    static bool attr[64] = {};
    CG_CUDA(smem_limit_once(k_r2c_rows<T>, kMaxSmem, attr));
    k_r2c_rows<T><<<grid, kFFTThreads, smem, st>>>(cs, p, tw, nxp, nrows, scale);
  } else {
    static bool attr[64] = {};
    CG_CUDA(smem_limit_once(k_c2r_rows<T>, kMaxSmem, attr));
    k_c2r_rows<T><<<grid, kFFTThreads, smem, st>>>(cs, addend, p, tw, nxp, nrows, scale, epi);
  }
  CG_CHECK_LAUNCH(forward ? "k_r2c_rows" : "k_c2r_rows");
  return CG_OK;
}

template <typename T>
int launch_cols(const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride, long batch_stride, int nbatch,
                int sign, cudaStream_t st)
{
  if (n == 1) return CG_OK;
  AxisPlan p;
  if (!make_axis_plan(n, &p)) {
    set_error("axis length %d has a prime factor above 7 or exceeds %d", n, kMaxFFT);
    return CG_ERR_UNSUPPORTED;
  }
  const C2<T> *tw = twiddle_table<T>(n);
  if (!tw) return cuda_status(cudaGetLastError(), "twiddle table");
  int col0 = 0;
  if constexpr (sizeof(T) == 4) {
    int done = 0;
    const int rc = fast_cols(cs, ncubes, n, ncols, axis_stride, batch_stride, nbatch, sign, (const float2 *)tw, st,
                             &done);
    if (rc < 0) return rc;
    col0 = done;
    ncols -= done;
    if (ncols == 0) return CG_OK;
  }
  // tile width: 16 columns (128 B rows for float) when shared memory allows
  const size_t budget = 200 * 1024;
  int wfull = 16 / (int)(sizeof(T) / sizeof(float));
  while (wfull > 1 && (2 * (size_t)n * (wfull + 1) + n) * sizeof(C2<T>) > budget) wfull /= 2;
  int ntiles = ceil_div(ncols, wfull);
  if (ntiles > 1 && ncols - (ntiles - 1) * wfull == 1) ntiles--;  // fold a lone Nyquist column into the last tile
  if (ntiles == 1 && ncols > wfull + 1) {
    set_error("internal tiling error");
    return CG_ERR_STATE;
  }
  if (ncols > wfull + 1 && ntiles * wfull < ncols - 1) {
    set_error("internal tiling error");
    return CG_ERR_STATE;
  }
  size_t smem = (2 * (size_t)n * (wfull + 1) + (size_t)n) * sizeof(C2<T>);
  if (smem > budget + 8 * 1024) {
    set_error("axis length %d too long for the shared-memory tile", n);
    return CG_ERR_UNSUPPORTED;
  }
  static bool attr[64] = {};
  CG_CUDA(smem_limit_once(k_fft_cols<T>, kMaxSmem, attr));
  dim3 grid(ntiles, nbatch, ncubes);
  TraceScope ts("k_fft_cols", st, 2.0 * ncubes * nbatch * (double)ncols * n * sizeof(C2<T>));
  k_fft_cols<T><<<grid, kFFTThreads, smem, st>>>(cs, p, tw, col0, ncols, wfull, ntiles, axis_stride, batch_stride,
                                                 sign);
  CG_CHECK_LAUNCH("k_fft_cols");
  return CG_OK;
}

int check_dims(int nxp, int nyp, int nzp, int count)
{
  if (nxp < 1 || nyp < 1 || nzp < 1 || count < 1) {
    set_error("bad dimensions nxp=%d nyp=%d nzp=%d count=%d", nxp, nyp, nzp, count);
    return CG_ERR_ARG;
  }
  if (nxp > kMaxFFT || nyp > kMaxFFT || nzp > kMaxFFT) {
    set_error("axis length above %d", kMaxFFT);
    return CG_ERR_UNSUPPORTED;
  }
  if (nyp > 65535 || nzp > 65535) {
    set_error("nyp/nzp above 65535");
    return CG_ERR_UNSUPPORTED;
  }
  return CG_OK;
}

}  // namespace

template <typename T>
int fft3d(void *const *bufs, int count, int nxp, int nyp, int nzp, int cubetype, bool forward, cudaStream_t st)
{
  return fft3d_add<T>(bufs, nullptr, count, nxp, nyp, nzp, cubetype, forward, st);
}

template <typename T>
int fft3d_c2r_add(void *const *bufs, const void *const *addends, int count, int nxp, int nyp, int nzp, int cubetype,
                  cudaStream_t st)
{
  return fft3d_add<T>(bufs, addends, count, nxp, nyp, nzp, cubetype, false, st);
}

template <typename T>
int fft3d_c2r_epi(void *const *bufs, int count, int nxp, int nyp, int nzp, int cubetype, int epi, cudaStream_t st)
{
  return fft3d_add<T>(bufs, nullptr, count, nxp, nyp, nzp, cubetype, false, st, epi);
}

template <typename T>
int fft3d_add(void *const *bufs, const void *const *addends, int count, int nxp, int nyp, int nzp, int cubetype,
              bool forward, cudaStream_t st, int epi)
{
  int rc = check_dims(nxp, nyp, nzp, count);
  if (rc) return rc;
  if (cubetype < CG_CTMISSING || cubetype > CG_OPERATOR || cubetype == CG_CTMISSING) {
    set_error("cubetype %d is not one of DATA/PARAMETER/COVARIANCE/VELOCITY/OPERATOR", cubetype);
    return CG_ERR_ARG;
  }
  const int cnxp = nxp / 2 + 1;
  const double N = (double)nxp * nyp * nzp;
  const bool covlike = (cubetype == CG_COVARIANCE || cubetype == CG_OPERATOR);
  for (int b0 = 0; b0 < count; b0 += kMaxBatch) {
    int nb = count - b0 < kMaxBatch ? count - b0 : kMaxBatch;
    CubeSet cs, ad;
    for (int i = 0; i < kMaxBatch; i++) { cs.ptr[i] = nullptr; ad.ptr[i] = nullptr; }
    for (int i = 0; i < nb; i++) {
      if (!bufs[b0 + i]) {
        set_error("null buffer %d", b0 + i);
        return CG_ERR_ARG;
      }
      cs.ptr[i] = bufs[b0 + i];
      if (addends) ad.ptr[i] = (void *)addends[b0 + i];
    }
    if (forward) {
      T pre = covlike ? (T)1 : (T)(1.0 / sqrt(N));
      int xy = 0;
      if constexpr (sizeof(T) == 4) {
        xy = xy_planes(true, cs, ad, nb, nxp, nyp, nzp, (float)pre, st, kEpiNone);
        if (xy < 0) return xy;
      }
      if (!xy) {
        if ((rc = launch_rows<T>(true, cs, ad, nb, nxp, nyp, nzp, pre, st))) return rc;
        if ((rc = launch_cols<T>(cs, nb, nyp, cnxp, cnxp, (long)nyp * cnxp, nzp, -1, st))) return rc;
      }
      if ((rc = launch_cols<T>(cs, nb, nzp, cnxp, (long)cnxp * nyp, cnxp, nyp, -1, st))) return rc;
    } else {
      T post = covlike ? (T)(1.0 / N) : (T)(1.0 / sqrt(N));
      if ((rc = launch_cols<T>(cs, nb, nzp, cnxp, (long)cnxp * nyp, cnxp, nyp, +1, st))) return rc;
      int xy = 0;
      if constexpr (sizeof(T) == 4) {
        xy = xy_planes(false, cs, ad, nb, nxp, nyp, nzp, (float)post, st, epi);
        if (xy < 0) return xy;
      }
      if (!xy) {
        if ((rc = launch_cols<T>(cs, nb, nyp, cnxp, cnxp, (long)nyp * cnxp, nzp, +1, st))) return rc;
        if ((rc = launch_rows<T>(false, cs, ad, nb, nxp, nyp, nzp, post, st, epi))) return rc;
      }
    }
  }
  return CG_OK;
}
// The x and z passes of a 3D transform only (forward: x rows then z columns;
// inverse: z columns then x rows), with the full 3D scaling.  The y pass is
// left to the caller (the fused y-transform + bin kernel).
template <typename T>
int fft3d_xz(void *const *bufs, int count, int nxp, int nyp, int nzp, int cubetype, bool forward, cudaStream_t st)
{
  int rc = check_dims(nxp, nyp, nzp, count);
  if (rc) return rc;
  if (cubetype < CG_DATA || cubetype > CG_OPERATOR) {
    set_error("cubetype %d is not one of DATA/PARAMETER/COVARIANCE/VELOCITY/OPERATOR", cubetype);
    return CG_ERR_ARG;
  }
  const int cnxp = nxp / 2 + 1;
  const double N = (double)nxp * nyp * nzp;
  const bool covlike = (cubetype == CG_COVARIANCE || cubetype == CG_OPERATOR);
  for (int b0 = 0; b0 < count; b0 += kMaxBatch) {
    const int nb = count - b0 < kMaxBatch ? count - b0 : kMaxBatch;
    CubeSet cs, ad;
    for (int i = 0; i < kMaxBatch; i++) { cs.ptr[i] = nullptr; ad.ptr[i] = nullptr; }
    for (int i = 0; i < nb; i++) {
      if (!bufs[b0 + i]) { set_error("null buffer %d", b0 + i); return CG_ERR_ARG; }
      cs.ptr[i] = bufs[b0 + i];
    }
    if (forward) {
      const T pre = covlike ? (T)1 : (T)(1.0 / sqrt(N));
      if ((rc = launch_rows<T>(true, cs, ad, nb, nxp, nyp, nzp, pre, st))) return rc;
      if ((rc = launch_cols<T>(cs, nb, nzp, cnxp, (long)cnxp * nyp, cnxp, nyp, -1, st))) return rc;
    } else {
      const T post = covlike ? (T)(1.0 / N) : (T)(1.0 / sqrt(N));
      if ((rc = launch_cols<T>(cs, nb, nzp, cnxp, (long)cnxp * nyp, cnxp, nyp, +1, st))) return rc;
      if ((rc = launch_rows<T>(false, cs, ad, nb, nxp, nyp, nzp, post, st))) return rc;
    }
  }
  return CG_OK;
}

// 1D real transforms of nrows rows of length nx in the FFTW in-place row
// layout (pitch 2*(nx/2+1) floats); scale multiplies the input (forward) or
// the output (inverse)
template <typename T>
int fft_rows(void *buf, int nx, int nrows, bool forward, T scale, cudaStream_t st)
{
  if (!buf || nx < 1 || nrows < 1) { set_error("fft_rows: bad argument"); return CG_ERR_ARG; }
  CubeSet cs, ad;
  for (int i = 0; i < kMaxBatch; i++) { cs.ptr[i] = nullptr; ad.ptr[i] = nullptr; }
  cs.ptr[0] = buf;
  return launch_rows<T>(forward, cs, ad, 1, nx, nrows, 1, scale, st);
}

// one column pass (length n, ncols columns of nbatch batch rows) over count
// cubes given by their first element
template <typename T>
int fft_cols(void *const *bufs, int count, int n, int ncols, long axis_stride, long batch_stride, int nbatch, int sign,
             cudaStream_t st)
{
  if (!bufs || count < 1 || count > kMaxBatch) { set_error("fft_cols: bad argument"); return CG_ERR_ARG; }
  CubeSet cs;
  for (int i = 0; i < kMaxBatch; i++) cs.ptr[i] = i < count ? bufs[i] : nullptr;
  return launch_cols<T>(cs, count, n, ncols, axis_stride, batch_stride, nbatch, sign, st);
}

// the x pass alone (R2C forward with prescale, C2R inverse with postscale) over count cubes
template <typename T>
int fft_x_pass(void *const *bufs, int count, int nxp, int nyp, int nzp, bool forward, T scale, cudaStream_t st)
{
  if (!bufs || count < 1 || count > kMaxBatch) { set_error("fft_x_pass: bad argument"); return CG_ERR_ARG; }
  CubeSet cs, ad;
  for (int i = 0; i < kMaxBatch; i++) { cs.ptr[i] = i < count ? bufs[i] : nullptr; ad.ptr[i] = nullptr; }
  return launch_rows<T>(forward, cs, ad, count, nxp, nyp, nzp, scale, st);
}

template int fft3d<float>(void *const *, int, int, int, int, int, bool, cudaStream_t);
template int fft3d_xz<float>(void *const *, int, int, int, int, int, bool, cudaStream_t);
template int fft_x_pass<float>(void *const *, int, int, int, int, bool, float, cudaStream_t);
template int fft_cols<float>(void *const *, int, int, int, long, long, int, int, cudaStream_t);
template int fft_rows<float>(void *, int, int, bool, float, cudaStream_t);
template int fft3d<double>(void *const *, int, int, int, int, int, bool, cudaStream_t);
template int fft3d_c2r_add<float>(void *const *, const void *const *, int, int, int, int, int, cudaStream_t);
template int fft3d_c2r_epi<float>(void *const *, int, int, int, int, int, int, cudaStream_t);

}  // namespace cg

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
using namespace cg;

extern "C" int cg_fft_max_length(void) { return kMaxFFT; }

extern "C" int cg_fft3d_r2c(float *buf, int nxp, int nyp, int nzp, int cubetype, void *stream)
{
  void *b[1] = {buf};
  return fft3d<float>(b, 1, nxp, nyp, nzp, cubetype, true, (cudaStream_t)stream);
}

extern "C" int cg_fft3d_c2r(float *buf, int nxp, int nyp, int nzp, int cubetype, void *stream)
{
  void *b[1] = {buf};
  return fft3d<float>(b, 1, nxp, nyp, nzp, cubetype, false, (cudaStream_t)stream);
}

extern "C" int cg_fft3d_r2c_batch(float *const *bufs, int count, int nxp, int nyp, int nzp, int cubetype,
                                  void *stream)
{
  if (!bufs) { set_error("null buffer list"); return CG_ERR_ARG; }
  return fft3d<float>((void *const *)bufs, count, nxp, nyp, nzp, cubetype, true, (cudaStream_t)stream);
}

extern "C" int cg_fft3d_c2r_batch(float *const *bufs, int count, int nxp, int nyp, int nzp, int cubetype,
                                  void *stream)
{
  if (!bufs) { set_error("null buffer list"); return CG_ERR_ARG; }
  return fft3d<float>((void *const *)bufs, count, nxp, nyp, nzp, cubetype, false, (cudaStream_t)stream);
}

extern "C" int cg_fft3d_r2c_f64(double *buf, int nxp, int nyp, int nzp, int cubetype, void *stream)
{
  void *b[1] = {buf};
  return fft3d<double>(b, 1, nxp, nyp, nzp, cubetype, true, (cudaStream_t)stream);
}

extern "C" int cg_fft3d_c2r_f64(double *buf, int nxp, int nyp, int nzp, int cubetype, void *stream)
{
  void *b[1] = {buf};
  return fft3d<double>(b, 1, nxp, nyp, nzp, cubetype, false, (cudaStream_t)stream);
}

static int fft_host(float *hbuf, int nxp, int nyp, int nzp, int cubetype, bool forward)
{
  if (!hbuf) { set_error("null host buffer"); return CG_ERR_ARG; }
  int rc = CG_OK;
  size_t bytes = sizeof(float) * 2 * (size_t)(nxp / 2 + 1) * nyp * nzp;
  float *d = nullptr;
  count_alloc();
  CG_CUDA(cudaMalloc(&d, bytes));
  cudaError_t e = cudaMemcpy(d, hbuf, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { cudaFree(d); return cuda_status(e, "H2D"); }
  void *b[1] = {d};
  rc = fft3d<float>(b, 1, nxp, nyp, nzp, cubetype, forward, 0);
  if (rc == CG_OK) {
    e = cudaMemcpy(hbuf, d, bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_status(e, "D2H");
  }
  cudaFree(d);
  return rc;
}

extern "C" int cg_fft3d_r2c_host(float *hbuf, int nxp, int nyp, int nzp, int cubetype)
{
  return fft_host(hbuf, nxp, nyp, nzp, cubetype, true);
}

extern "C" int cg_fft3d_c2r_host(float *hbuf, int nxp, int nyp, int nzp, int cubetype)
{
  return fft_host(hbuf, nxp, nyp, nzp, cubetype, false);
}
