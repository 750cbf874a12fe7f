// Shared-memory Stockham FFT building blocks (device) and FFT plan types.
#pragma once

#include "common.cuh"

namespace cg {

constexpr int kMaxStages = 16;
constexpr int kMaxFFT = 8192;  // longest axis handled by one shared-memory tile
constexpr int kFFTThreads = 256;
constexpr int kRows = 16;      // x rows per CTA in the row passes
constexpr int kMaxBatch = 16;  // cubes per launch
constexpr size_t kMaxSmem = 227 * 1024;  // dynamic shared memory per CTA on sm_103a

struct AxisPlan {
  int n;
  int nstages;
  int radix[kMaxStages];
};

struct CubeSet {
  void *ptr[kMaxBatch];
};

bool make_axis_plan(int n, AxisPlan *p);

// Raise a kernel's dynamic shared-memory limit once per device (the attribute
// is per device; setting it on every launch would be wasted work and is not
// wanted inside a stream capture).
template <typename K>
inline cudaError_t smem_limit_once(K kernel, size_t bytes, bool *done_per_device)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (done_per_device[dev]) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) done_per_device[dev] = true;
  return e;
}
template <typename T> const C2<T> *twiddle_table(int n);
template <typename T>
int fft3d(void *const *bufs, int count, int nxp, int nyp, int nzp, int cubetype, bool forward, cudaStream_t st);
template <typename T>
int fft3d_add(void *const *bufs, const void *const *addends, int count, int nxp, int nyp, int nzp, int cubetype,
              bool forward, cudaStream_t st, int epi = kEpiNone);
// 1D real transforms of rows (see fft.cu)
template <typename T>
int fft_rows(void *buf, int nx, int nrows, bool forward, T scale, cudaStream_t st);
// the x pass alone over given cube pointers (see fft.cu)
template <typename T>
int fft_x_pass(void *const *bufs, int count, int nxp, int nyp, int nzp, bool forward, T scale, cudaStream_t st);
// one column pass over given cube pointers (see fft.cu)
template <typename T>
int fft_cols(void *const *bufs, int count, int n, int ncols, long axis_stride, long batch_stride, int nbatch, int sign,
             cudaStream_t st);
// x and z passes only (see fft.cu)
template <typename T>
int fft3d_xz(void *const *bufs, int count, int nxp, int nyp, int nzp, int cubetype, bool forward, cudaStream_t st);
// inverse transform whose last pass applies an output epilogue (kEpiExp: FFTGrid::expTransf fused)
template <typename T>
int fft3d_c2r_epi(void *const *bufs, int count, int nxp, int nyp, int nzp, int cubetype, int epi, cudaStream_t st);
// inverse transform with a real cube added to each result (FFTGrid::add fused)
template <typename T>
int fft3d_c2r_add(void *const *bufs, const void *const *addends, int count, int nxp, int nyp, int nzp, int cubetype,
                  cudaStream_t st);

// twiddle W (forward table entry) applied with the transform's sign
template <typename T>
__device__ __forceinline__ C2<T> tw_at(const C2<T> *tw, int idx, int sign)
{
  C2<T> w = tw[idx];
  if (sign > 0) w.y = -w.y;
  return w;
}

// multiply by sign*i
template <typename T>
__device__ __forceinline__ C2<T> mul_si(C2<T> a, int sign)
{
  return sign > 0 ? mk<T>(-a.y, a.x) : mk<T>(a.y, -a.x);
}

template <typename T>
__device__ __forceinline__ void dft2(C2<T> *v)
{
  C2<T> a = v[0], b = v[1];
  v[0] = cadd<T>(a, b);
  v[1] = csub<T>(a, b);
}

template <typename T>
__device__ __forceinline__ void dft4(C2<T> *v, int sign)
{
  C2<T> s02 = cadd<T>(v[0], v[2]), d02 = csub<T>(v[0], v[2]);
  C2<T> s13 = cadd<T>(v[1], v[3]), d13 = mul_si<T>(csub<T>(v[1], v[3]), sign);
  v[0] = cadd<T>(s02, s13);
  v[2] = csub<T>(s02, s13);
  v[1] = cadd<T>(d02, d13);
  v[3] = csub<T>(d02, d13);
}

template <typename T>
__device__ __forceinline__ void dft8(C2<T> *v, int sign)
{
  C2<T> e[4] = {v[0], v[2], v[4], v[6]};
  C2<T> o[4] = {v[1], v[3], v[5], v[7]};
  dft4<T>(e, sign);
  dft4<T>(o, sign);
  const T h = (T)0.70710678118654752440;
  // W8^1 = (1 + s i)/sqrt2, W8^2 = s i, W8^3 = (-1 + s i)/sqrt2
  C2<T> o1 = o[1], o3 = o[3];
  C2<T> t1 = mk<T>((o1.x - sign * o1.y) * h, (o1.y + sign * o1.x) * h);
  C2<T> t2 = mul_si<T>(o[2], sign);
  C2<T> t3 = mk<T>((-o3.x - sign * o3.y) * h, (-o3.y + sign * o3.x) * h);
  v[0] = cadd<T>(e[0], o[0]);
  v[4] = csub<T>(e[0], o[0]);
  v[1] = cadd<T>(e[1], t1);
  v[5] = csub<T>(e[1], t1);
  v[2] = cadd<T>(e[2], t2);
  v[6] = csub<T>(e[2], t2);
  v[3] = cadd<T>(e[3], t3);
  v[7] = csub<T>(e[3], t3);
}

// cos(2 pi m / R) and sin(2 pi m / R) for the odd prime radices, m = 1 .. (R-1)/2 (the values of the
// roots of unity to 22 digits; other m fold onto these by symmetry)
__host__ __device__ constexpr double root_cos(int r, int m)
{
  return r == 3 ? -0.5
       : r == 5 ? (m == 1 ? 0.3090169943749474241023 : -0.8090169943749474241023)
       : (m == 1 ? 0.623489801858733530525 : m == 2 ? -0.2225209339563144042889 : -0.9009688679024191262361);
}
__host__ __device__ constexpr double root_sin(int r, int m)
{
  return r == 3 ? 0.8660254037844386467637
       : r == 5 ? (m == 1 ? 0.9510565162951535721164 : 0.5877852522924731291687)
       : (m == 1 ? 0.7818314824680298087084 : m == 2 ? 0.9749279121818236070181 : 0.4338837391175581204758);
}
// cos / sin of 2 pi m / R for any m
__host__ __device__ constexpr double rc(int r, int m)
{
  return m % r == 0 ? 1.0 : m % r <= r / 2 ? root_cos(r, m % r) : root_cos(r, r - m % r);
}
__host__ __device__ constexpr double rs(int r, int m)
{
  return m % r == 0 ? 0.0 : m % r <= r / 2 ? root_sin(r, m % r) : -root_sin(r, r - m % r);
}

// odd prime radix R (3, 5, 7): the DFT X[u] = sum_q v[q] W^(qu), W = exp(sign 2 pi i / R), folded over the
// conjugate-symmetric pairs: with t_q = v[q] + v[R-q], d_q = v[q] - v[R-q] (q = 1 .. (R-1)/2),
//   X[0] = v[0] + sum t_q,   X[u], X[R-u] = A_u +- i sign B_u,
//   A_u = v[0] + sum_q t_q cos(2 pi qu/R),   B_u = sum_q d_q sin(2 pi qu/R),
// real constants in place of the (R-1)^2 complex products of the direct sum.  (tw and rstride are unused:
// the roots are compile-time constants.)
template <typename T, int R>
__device__ __forceinline__ void dft_odd(C2<T> *v, int sign, const C2<T> *, int)
{
  constexpr int H = (R - 1) / 2;
  C2<T> t[H], d[H];
#pragma unroll
  for (int q = 1; q <= H; q++) {
    t[q - 1] = cadd<T>(v[q], v[R - q]);
    d[q - 1] = csub<T>(v[q], v[R - q]);
  }
  const C2<T> v0 = v[0];
  C2<T> x0 = v0;
#pragma unroll
  for (int q = 0; q < H; q++) x0 = cadd<T>(x0, t[q]);
#pragma unroll
  for (int u = 1; u <= H; u++) {
    T ax = v0.x, ay = v0.y, bx = 0, by = 0;
#pragma unroll
    for (int q = 1; q <= H; q++) {
      const T c = (T)rc(R, q * u), sn = (T)rs(R, q * u);
      ax += t[q - 1].x * c;
      ay += t[q - 1].y * c;
      bx += d[q - 1].x * sn;
      by += d[q - 1].y * sn;
    }
    // i sign B = sign (-by, bx)
    if (sign > 0) {
      v[u] = mk<T>(ax - by, ay + bx);
      v[R - u] = mk<T>(ax + by, ay - bx);
    } else {
      v[u] = mk<T>(ax + by, ay - bx);
      v[R - u] = mk<T>(ax - by, ay + bx);
    }
  }
  v[0] = x0;
}

// One Stockham stage for the butterfly j of column c:
// reads src[(j + r*nb)], twiddles by W_{Ns R}^{(j mod Ns) r}, radix-R DFT,
// writes dst[(j div Ns)*Ns*R + (j mod Ns) + r*Ns].
template <typename T, int R>
__device__ __forceinline__ void stockham_bfly(const C2<T> *src, C2<T> *dst, int j, int c, int nb, int Ns, int span,
                                              int ldw, const C2<T> *tw, int twstride, int sign)
{
  C2<T> v[R];
#pragma unroll
  for (int r = 0; r < R; r++) v[r] = src[(j + r * nb) * ldw + c];
  const int jm = j % Ns;
  if (jm) {
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = cmul<T>(v[r], tw_at<T>(tw, jm * r * span * twstride, sign));
  }
  if constexpr (R == 2) dft2<T>(v);
  else if constexpr (R == 4) dft4<T>(v, sign);
  else if constexpr (R == 8) dft8<T>(v, sign);
  else dft_odd<T, R>(v, sign, tw, nb * twstride);
  const int d = (j - jm) * R + jm;
#pragma unroll
  for (int r = 0; r < R; r++) dst[(d + r * Ns) * ldw + c] = v[r];
}

// Transform `width` columns of length p.n held in shared memory at a[e*ldw+c].
// tw holds W_N^t for a table length N = p.n*twstride.  All threads of the CTA
// must call it; returns the buffer that holds the result.
template <typename T>
__device__ C2<T> *smem_fft(C2<T> *a, C2<T> *b, const AxisPlan &p, int width, int ldw, const C2<T> *tw, int twstride,
                           int sign)
{
  const int n = p.n;
  int Ns = 1;
  for (int s = 0; s < p.nstages; s++) {
    const int R = p.radix[s];
    const int nb = n / R;
    const int span = n / (Ns * R);
    const int total = nb * width;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int j = t / width;
      const int c = t - j * width;
      switch (R) {
        case 8: stockham_bfly<T, 8>(a, b, j, c, nb, Ns, span, ldw, tw, twstride, sign); break;
        case 4: stockham_bfly<T, 4>(a, b, j, c, nb, Ns, span, ldw, tw, twstride, sign); break;
        case 2: stockham_bfly<T, 2>(a, b, j, c, nb, Ns, span, ldw, tw, twstride, sign); break;
        case 3: stockham_bfly<T, 3>(a, b, j, c, nb, Ns, span, ldw, tw, twstride, sign); break;
        case 5: stockham_bfly<T, 5>(a, b, j, c, nb, Ns, span, ldw, tw, twstride, sign); break;
        default: stockham_bfly<T, 7>(a, b, j, c, nb, Ns, span, ldw, tw, twstride, sign); break;
      }
    }
    __syncthreads();
    C2<T> *t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

}  // namespace cg
