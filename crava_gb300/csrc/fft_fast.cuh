// Compile-time specialised FFT passes for the common padded lengths.
//
// Same transforms as the generic kernels in fft.cu, but with the length N
// and tile width W known at compile time:
//   * the Stockham plan (radices 8, 4, 2, 3, 5, 7 in that order, exactly as
//     make_axis_plan) and every index of every stage fold to constants;
//   * one shared buffer: each stage reads all of a thread's butterflies into
//     registers, synchronises, then writes them back in place (Stockham
//     stages are permutations, so this is race free), halving shared memory
//     and raising resident CTAs per SM;
//   * the tile is staged with cp.async, so every load of the tile is in
//     flight at once instead of one dependent load per thread.
#pragma once

#include "fft.cuh"

namespace cg {

__host__ __device__ constexpr int radix_order(int q) { return q == 0 ? 8 : q == 1 ? 4 : q == 2 ? 2 : q == 3 ? 3 : q == 4 ? 5 : 7; }

__host__ __device__ constexpr int plan_nstages(int n)
{
  int m = n, s = 0;
  for (int q = 0; q < 6; q++)
    while (m % radix_order(q) == 0) { m /= radix_order(q); s++; }
  return m == 1 ? s : -1;
}

__host__ __device__ constexpr int plan_radix(int n, int stage)
{
  int m = n, s = 0;
  for (int q = 0; q < 6; q++)
    while (m % radix_order(q) == 0) {
      if (s == stage) return radix_order(q);
      m /= radix_order(q);
      s++;
    }
  return 1;
}

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
  return (unsigned)__cvta_generic_to_shared(p);
}

// 8-byte global -> shared asynchronous copy (LDGSTS through L1)
__device__ __forceinline__ void cp_async8(void *smem_dst, const void *gsrc)
{
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_u32(smem_dst)), "l"(gsrc) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

template <typename T, int R>
__device__ __forceinline__ void dft_any(C2<T> *v, int sign, const C2<T> *tw, int rstride)
{
  if constexpr (R == 2) dft2<T>(v);
  else if constexpr (R == 4) dft4<T>(v, sign);
  else if constexpr (R == 8) dft8<T>(v, sign);
  else dft_odd<T, R>(v, sign, tw, rstride);
}

// All Stockham stages of a length-N transform on W columns held in place at
// buf[e*LDW + c]; the twiddle table has N*TWS entries.
template <typename T, int N, int W, int LDW, int TWS, int S = 0, int NS = 1>
__device__ __forceinline__ void cstages(C2<T> *buf, const C2<T> *tw, int sign)
{
  if constexpr (S < plan_nstages(N)) {
    constexpr int R = plan_radix(N, S);
    constexpr int NB = N / R;
    constexpr int SPAN = N / (NS * R);
    constexpr int TOT = NB * W;
    constexpr int BPT = (TOT + kFFTThreads - 1) / kFFTThreads;
    C2<T> v[BPT][R];
#pragma unroll
    for (int q = 0; q < BPT; q++) {
      const int t = q * kFFTThreads + threadIdx.x;
      if (TOT % kFFTThreads == 0 || t < TOT) {
        const int j = t / W, c = t % W;
#pragma unroll
        for (int r = 0; r < R; r++) v[q][r] = buf[(j + r * NB) * LDW + c];
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < BPT; q++) {
      const int t = q * kFFTThreads + threadIdx.x;
      if (TOT % kFFTThreads == 0 || t < TOT) {
        const int j = t / W, c = t % W;
        const int jm = j % NS;
        if (NS > 1) {
#pragma unroll
          for (int r = 1; r < R; r++) v[q][r] = cmul<T>(v[q][r], tw_at<T>(tw, jm * r * SPAN * TWS, sign));
        }
        dft_any<T, R>(v[q], sign, tw, NB * TWS);
        const int d = (j - jm) * R + jm;
#pragma unroll
        for (int r = 0; r < R; r++) buf[(d + r * NS) * LDW + c] = v[q][r];
      }
    }
    __syncthreads();
    cstages<T, N, W, LDW, TWS, S + 1, NS * R>(buf, tw, sign);
  }
}

// ---------------------------------------------------------------------------
// strided column pass on tiles of W columns.  Element (e, c) of the tile of
// CTA (x, y, z) is cube z at  y*by + x*bx + c*cs + e*axis_stride, and only
// columns with x*W + c < climit exist.  Full tiles of adjacent columns use
// (by, bx, cs) = (batch stride, W, 1); the columns left over after the full
// tiles (the Nyquist column of an odd cnxp) are gathered across the batch
// with (by, bx, cs) = (1, W*batch stride, batch stride).
// ---------------------------------------------------------------------------
struct ColsGeom {
  long axis_stride;   // between elements of one column
  long batch_stride;  // between batch rows (y)
  int nfull;          // full W-column tiles per batch row (grid.x = nfull + 1 when ntail > 0)
  int ntail;          // leftover columns after the full tiles
  int nbatch;
  int trows;          // four-step kernel: batch rows per tail tile (its tail tiles are ntail x trows blocks)
};

template <int N, int W, int MINB>
__global__ void __launch_bounds__(kFFTThreads, MINB) k_fft_cols_fast(const __grid_constant__ CubeSet cs, const float2 *__restrict__ twg,
                                                                     ColsGeom g, int sign)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf = (float2 *)smem_raw;
  float2 *tw = buf + N * W;
  // full tiles: (x < nfull, y = batch row); grid columns x >= nfull hold the
  // tail tiles, numbered (x - nfull)*nbatch + y (CTAs past the last one exit)
  long by, bx, cstride;
  int cvalid;
  float2 *cube = (float2 *)cs.ptr[blockIdx.z];
  if ((int)blockIdx.x < g.nfull) {
    by = g.batch_stride; bx = W; cstride = 1; cvalid = W;
  } else {
    // tail tile tt = (x - nfull)*nbatch + y, tt < ntail*groups
    const int groups = (g.nbatch + W - 1) / W;
    const int tt = ((int)blockIdx.x - g.nfull) * g.nbatch + (int)blockIdx.y;
    const int tcol = tt / groups, grp = tt % groups;
    if (tcol >= g.ntail) return;
    cube += (long)g.nfull * W + tcol;
    by = 0; bx = 0; cstride = g.batch_stride;
    cube += (long)grp * W * g.batch_stride;
    cvalid = g.nbatch - grp * W;
  }
  const long axis_stride = g.axis_stride;
  float2 *base = cube + ((int)blockIdx.x < g.nfull ? (long)blockIdx.y * by + (long)blockIdx.x * bx : 0);
  for (int t = threadIdx.x; t < N; t += kFFTThreads) tw[t] = twg[t];
#pragma unroll
  for (int t0 = 0; t0 < N * W; t0 += kFFTThreads) {
    const int t = t0 + threadIdx.x;
    if ((N * W) % kFFTThreads == 0 || t < N * W) {
      const int e = t / W, c = t % W;
      if (c < cvalid) cp_async8(&buf[e * W + c], &base[(long)e * axis_stride + (long)c * cstride]);
      else buf[e * W + c] = make_float2(0.f, 0.f);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  cstages<float, N, W, W, 1>(buf, tw, sign);
#pragma unroll
  for (int t0 = 0; t0 < N * W; t0 += kFFTThreads) {
    const int t = t0 + threadIdx.x;
    if ((N * W) % kFFTThreads == 0 || t < N * W) {
      const int e = t / W, c = t % W;
      if (c < cvalid) base[(long)e * axis_stride + (long)c * cstride] = buf[e * W + c];
    }
  }
}

// ---------------------------------------------------------------------------
// persistent, double-buffered column pass: CTA b handles tiles b, b+G, b+2G...
// of a linear tile list (per cube: nbatch*nfull full tiles, then ntail*groups
// gathered tail tiles); the next tile is prefetched with cp.async while the
// current one is transformed and stored.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory"); }

struct TileRef {
  float2 *base;
  long cstride;
  int cvalid;
};

template <int W>
__device__ __forceinline__ TileRef cols_tile(const CubeSet &cs, const ColsGeom &g, int t)
{
  const int groups = (g.nbatch + W - 1) / W;
  const int per_cube = g.nbatch * g.nfull + g.ntail * groups;
  const int z = t / per_cube, r = t - z * per_cube;
  float2 *cube = (float2 *)cs.ptr[z];
  TileRef ref;
  if (r < g.nbatch * g.nfull) {
    const int y = r / g.nfull, x = r - y * g.nfull;
    ref.base = cube + (long)y * g.batch_stride + (long)x * W;
    ref.cstride = 1;
    ref.cvalid = W;
  } else {
    const int q = r - g.nbatch * g.nfull;
    const int tcol = q / groups, grp = q - tcol * groups;
    ref.base = cube + (long)g.nfull * W + tcol + (long)grp * W * g.batch_stride;
    ref.cstride = g.batch_stride;
    ref.cvalid = g.nbatch - grp * W;
  }
  return ref;
}

template <int N, int W>
__device__ __forceinline__ void cols_prefetch(float2 *buf, const TileRef &ref, long axis_stride)
{
#pragma unroll
  for (int t0 = 0; t0 < N * W; t0 += kFFTThreads) {
    const int t = t0 + threadIdx.x;
    if ((N * W) % kFFTThreads == 0 || t < N * W) {
      const int e = t / W, c = t % W;
      if (c < ref.cvalid) cp_async8(&buf[e * W + c], &ref.base[(long)e * axis_stride + (long)c * ref.cstride]);
      else buf[e * W + c] = make_float2(0.f, 0.f);
    }
  }
}

template <int N, int W, int MINB>
__global__ void __launch_bounds__(kFFTThreads, MINB) k_fft_cols_pipe(const __grid_constant__ CubeSet cs, const float2 *__restrict__ twg,
                                                                     ColsGeom g, int ntiles, int sign)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf0 = (float2 *)smem_raw;
  float2 *buf1 = buf0 + N * W;
  float2 *tw = buf1 + N * W;
  for (int t = threadIdx.x; t < N; t += kFFTThreads) tw[t] = twg[t];
  int tile = blockIdx.x;
  if (tile < ntiles) cols_prefetch<N, W>(buf0, cols_tile<W>(cs, g, tile), g.axis_stride);
  cp_async_commit();
  for (int it = 0; tile < ntiles; it++) {
    float2 *cur = (it & 1) ? buf1 : buf0;
    float2 *nxt = (it & 1) ? buf0 : buf1;
    const int next = tile + gridDim.x;
    if (next < ntiles) cols_prefetch<N, W>(nxt, cols_tile<W>(cs, g, next), g.axis_stride);
    cp_async_commit();
    cp_async_wait<1>();  // the current tile's copies are done; the next tile's may be in flight
    __syncthreads();
    cstages<float, N, W, W, 1>(cur, tw, sign);
    const TileRef ref = cols_tile<W>(cs, g, tile);
#pragma unroll
    for (int t0 = 0; t0 < N * W; t0 += kFFTThreads) {
      const int t = t0 + threadIdx.x;
      if ((N * W) % kFFTThreads == 0 || t < N * W) {
        const int e = t / W, c = t % W;
        if (c < ref.cvalid) ref.base[(long)e * g.axis_stride + (long)c * ref.cstride] = cur[e * W + c];
      }
    }
    __syncthreads();  // cur is refilled by the prefetch two iterations on
    tile = next;
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// register-direct column pass: the first Stockham stage reads its operands
// straight from global memory (each butterfly's R operands are R tile rows
// apart, and a warp covers 16 adjacent columns, so every load is part of a
// 128-byte row segment) and the last stage writes straight back, halving the
// shared-memory traffic of the staged kernel.
// ---------------------------------------------------------------------------
template <typename T, int N, int W, int LDW, int TWS, int S, int NS, int SEND>
__device__ __forceinline__ void cstages_range(C2<T> *buf, const C2<T> *tw, int sign)
{
  if constexpr (S < SEND) {
    constexpr int R = plan_radix(N, S);
    constexpr int NB = N / R;
    constexpr int SPAN = N / (NS * R);
    constexpr int TOT = NB * W;
    constexpr int BPT = (TOT + kFFTThreads - 1) / kFFTThreads;
    C2<T> v[BPT][R];
#pragma unroll
    for (int q = 0; q < BPT; q++) {
      const int t = q * kFFTThreads + threadIdx.x;
      if (TOT % kFFTThreads == 0 || t < TOT) {
        const int j = t / W, c = t % W;
#pragma unroll
        for (int r = 0; r < R; r++) v[q][r] = buf[(j + r * NB) * LDW + c];
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < BPT; q++) {
      const int t = q * kFFTThreads + threadIdx.x;
      if (TOT % kFFTThreads == 0 || t < TOT) {
        const int j = t / W, c = t % W;
        const int jm = j % NS;
        if (NS > 1) {
#pragma unroll
          for (int r = 1; r < R; r++) v[q][r] = cmul<T>(v[q][r], tw_at<T>(tw, jm * r * SPAN * TWS, sign));
        }
        dft_any<T, R>(v[q], sign, tw, NB * TWS);
        const int d = (j - jm) * R + jm;
#pragma unroll
        for (int r = 0; r < R; r++) buf[(d + r * NS) * LDW + c] = v[q][r];
      }
    }
    __syncthreads();
    cstages_range<T, N, W, LDW, TWS, S + 1, NS * R, SEND>(buf, tw, sign);
  }
}

__host__ __device__ constexpr int plan_ns_before(int n, int stage)
{
  int ns = 1;
  for (int s = 0; s < stage; s++) ns *= plan_radix(n, s);
  return ns;
}

template <int N, int W, int MINB>
__global__ void __launch_bounds__(kFFTThreads, MINB) k_fft_cols_rd(const __grid_constant__ CubeSet cs, const float2 *__restrict__ twg,
                                                                   ColsGeom g, int sign)
{
  static_assert(plan_nstages(N) >= 2, "register-direct pass needs two stages or more");
  constexpr int NST = plan_nstages(N);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf = (float2 *)smem_raw;
  float2 *tw = buf + N * W;
  float2 *cube = (float2 *)cs.ptr[blockIdx.z];
  long cstride;
  int cvalid;
  float2 *base;
  if ((int)blockIdx.x < g.nfull) {
    base = cube + (long)blockIdx.y * g.batch_stride + (long)blockIdx.x * W;
    cstride = 1;
    cvalid = W;
  } else {
    const int groups = (g.nbatch + W - 1) / W;
    const int tt = ((int)blockIdx.x - g.nfull) * g.nbatch + (int)blockIdx.y;
    const int tcol = tt / groups, grp = tt % groups;
    if (tcol >= g.ntail) return;
    base = cube + (long)g.nfull * W + tcol + (long)grp * W * g.batch_stride;
    cstride = g.batch_stride;
    cvalid = g.nbatch - grp * W;
  }
  const long as = g.axis_stride;
  for (int t = threadIdx.x; t < N; t += kFFTThreads) tw[t] = twg[t];
  // first stage (no twiddles): global -> registers -> shared
  {
    constexpr int R = plan_radix(N, 0);
    constexpr int NB = N / R;
    constexpr int TOT = NB * W;
    constexpr int BPT = (TOT + kFFTThreads - 1) / kFFTThreads;
    float2 v[BPT][R];
#pragma unroll
    for (int q = 0; q < BPT; q++) {
      const int t = q * kFFTThreads + threadIdx.x;
      const int j = t / W, c = t % W;
      const bool ok = (TOT % kFFTThreads == 0 || t < TOT) && c < cvalid;
#pragma unroll
      for (int r = 0; r < R; r++) v[q][r] = ok ? base[(long)(j + r * NB) * as + (long)c * cstride] : make_float2(0.f, 0.f);
    }
    // odd radices read the twiddle table inside the DFT; radices 2, 4 and 8 use
    // constants, so their warps start as soon as their own operands arrive (the
    // barrier after this stage publishes the table to the later stages)
    if constexpr (R % 2 == 1) __syncthreads();
#pragma unroll
    for (int q = 0; q < BPT; q++) {
      const int t = q * kFFTThreads + threadIdx.x;
      if (TOT % kFFTThreads == 0 || t < TOT) {
        const int j = t / W, c = t % W;
        dft_any<float, R>(v[q], sign, tw, NB);
#pragma unroll
        for (int r = 0; r < R; r++) buf[(j * R + r) * W + c] = v[q][r];
      }
    }
    __syncthreads();
  }
  // middle stages in shared memory
  cstages_range<float, N, W, W, 1, 1, plan_radix(N, 0), NST - 1>(buf, tw, sign);
  // last stage: shared -> registers -> global
  {
    constexpr int S = NST - 1;
    constexpr int R = plan_radix(N, S);
    constexpr int NS = plan_ns_before(N, S);
    constexpr int NB = N / R;
    constexpr int SPAN = N / (NS * R);
    constexpr int TOT = NB * W;
    constexpr int BPT = (TOT + kFFTThreads - 1) / kFFTThreads;
#pragma unroll
    for (int q = 0; q < BPT; q++) {
      const int t = q * kFFTThreads + threadIdx.x;
      if (TOT % kFFTThreads == 0 || t < TOT) {
        const int j = t / W, c = t % W;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = buf[(j + r * NB) * W + c];
        const int jm = j % NS;
#pragma unroll
        for (int r = 1; r < R; r++) v[r] = cmul<float>(v[r], tw_at<float>(tw, jm * r * SPAN, sign));
        dft_any<float, R>(v, sign, tw, NB);
        const int d = (j - jm) * R + jm;
        if (c < cvalid) {
#pragma unroll
          for (int r = 0; r < R; r++) base[(long)(d + r * NS) * as + (long)c * cstride] = v[r];
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// register-direct column pass on persistent CTAs that keep the next tile's
// loads in flight: CTA b transforms tiles b, b + G, ... of the tile list of
// k_fft_cols_pipe; before transforming tile i it issues the global loads of
// tile i + G into a second register set, so the loads of one tile overlap the
// arithmetic and stores of the previous one.
// ---------------------------------------------------------------------------
template <int N, int W, int MINB>
__global__ void __launch_bounds__(kFFTThreads, MINB) k_fft_cols_rdp(const __grid_constant__ CubeSet cs, const float2 *__restrict__ twg,
                                                                    ColsGeom g, int ntiles, int sign)
{
  static_assert(plan_nstages(N) >= 2, "register-direct pass needs two stages or more");
  constexpr int NST = plan_nstages(N);
  constexpr int R0 = plan_radix(N, 0);
  constexpr int NB0 = N / R0;
  constexpr int TOT0 = NB0 * W;
  constexpr int BPT0 = (TOT0 + kFFTThreads - 1) / kFFTThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf = (float2 *)smem_raw;
  float2 *tw = buf + N * W;
  const long as = g.axis_stride;
  for (int t = threadIdx.x; t < N; t += kFFTThreads) tw[t] = twg[t];
  auto load0 = [&](const TileRef &ref, float2 (*v)[R0]) {
#pragma unroll
    for (int q = 0; q < BPT0; q++) {
      const int t = q * kFFTThreads + threadIdx.x;
      const int j = t / W, c = t % W;
      const bool ok = (TOT0 % kFFTThreads == 0 || t < TOT0) && c < ref.cvalid;
#pragma unroll
      for (int r = 0; r < R0; r++) v[q][r] = ok ? ref.base[(long)(j + r * NB0) * as + (long)c * ref.cstride] : make_float2(0.f, 0.f);
    }
  };
  int tile = blockIdx.x;
  float2 vn[BPT0][R0];
  if (tile < ntiles) load0(cols_tile<W>(cs, g, tile), vn);
  __syncthreads();  // twiddles staged
  for (; tile < ntiles; tile += gridDim.x) {
    float2 v[BPT0][R0];
#pragma unroll
    for (int q = 0; q < BPT0; q++)
#pragma unroll
      for (int r = 0; r < R0; r++) v[q][r] = vn[q][r];
    const TileRef ref = cols_tile<W>(cs, g, tile);
    const int next = tile + gridDim.x;
    if (next < ntiles) load0(cols_tile<W>(cs, g, next), vn);  // consumed in the next iteration
    // first stage: registers -> shared
#pragma unroll
    for (int q = 0; q < BPT0; q++) {
      const int t = q * kFFTThreads + threadIdx.x;
      if (TOT0 % kFFTThreads == 0 || t < TOT0) {
        const int j = t / W, c = t % W;
        dft_any<float, R0>(v[q], sign, tw, NB0);
#pragma unroll
        for (int r = 0; r < R0; r++) buf[(j * R0 + r) * W + c] = v[q][r];
      }
    }
    __syncthreads();
    cstages_range<float, N, W, W, 1, 1, R0, NST - 1>(buf, tw, sign);
    // last stage: shared -> registers -> global
    {
      constexpr int S = NST - 1;
      constexpr int R = plan_radix(N, S);
      constexpr int NS = plan_ns_before(N, S);
      constexpr int NB = N / R;
      constexpr int SPAN = N / (NS * R);
      constexpr int TOT = NB * W;
      constexpr int BPT = (TOT + kFFTThreads - 1) / kFFTThreads;
#pragma unroll
      for (int q = 0; q < BPT; q++) {
        const int t = q * kFFTThreads + threadIdx.x;
        if (TOT % kFFTThreads == 0 || t < TOT) {
          const int j = t / W, c = t % W;
          float2 u[R];
#pragma unroll
          for (int r = 0; r < R; r++) u[r] = buf[(j + r * NB) * W + c];
          const int jm = j % NS;
#pragma unroll
          for (int r = 1; r < R; r++) u[r] = cmul<float>(u[r], tw_at<float>(tw, jm * r * SPAN, sign));
          dft_any<float, R>(u, sign, tw, NB);
          const int d = (j - jm) * R + jm;
          if (c < ref.cvalid) {
#pragma unroll
            for (int r = 0; r < R; r++) ref.base[(long)(d + r * NS) * as + (long)c * ref.cstride] = u[r];
          }
        }
      }
    }
    __syncthreads();  // buf is rewritten by the next tile's first stage
  }
}

// ---------------------------------------------------------------------------
// x rows, real -> half spectrum (even nxp = 2M), prescale applied to X
// ---------------------------------------------------------------------------
template <int M>
__global__ void __launch_bounds__(kFFTThreads) k_r2c_rows_fast(const __grid_constant__ CubeSet cs, const float2 *__restrict__ twg, int nrows,
                                                               float prescale)
{
  constexpr int LDW = kRows + 1;
  constexpr int NX = 2 * M, CN = M + 1, RN = 2 * CN;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf = (float2 *)smem_raw;
  float2 *tw = buf + M * LDW;
  const int r0 = blockIdx.x * kRows;
  const int nr = min(kRows, nrows - r0);
  float *base = (float *)cs.ptr[blockIdx.z] + (long)r0 * RN;
  for (int t = threadIdx.x; t < NX; t += kFFTThreads) tw[t] = twg[t];
#pragma unroll
  for (int t0 = 0; t0 < kRows * M; t0 += kFFTThreads) {
    const int t = t0 + threadIdx.x;
    if ((kRows * M) % kFFTThreads == 0 || t < kRows * M) {
      const int row = t / M, e = t % M;
      if (row < nr) cp_async8(&buf[e * LDW + row], base + (long)row * RN + 2 * e);
      else buf[e * LDW + row] = make_float2(0.f, 0.f);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  cstages<float, M, kRows, LDW, 2>(buf, tw, -1);
  for (int t = threadIdx.x; t < nr * CN; t += kFFTThreads) {
    const int row = t / CN, k = t - row * CN;
    const float2 A = buf[(k == M ? 0 : k) * LDW + row];
    const float2 Bc = buf[(k == 0 ? 0 : M - k) * LDW + row];
    const float2 B = make_float2(Bc.x, -Bc.y);
    const float2 E = make_float2((A.x + B.x) * 0.5f, (A.y + B.y) * 0.5f);
    const float2 O = make_float2((A.y - B.y) * 0.5f, -(A.x - B.x) * 0.5f);
    float2 X = cadd<float>(E, cmul<float>(tw[k], O));
    X.x *= prescale;
    X.y *= prescale;
    ((float2 *)(base + (long)row * RN))[k] = X;
  }
}

// ---------------------------------------------------------------------------
// x rows, half spectrum -> real (even nxp = 2M), postscale and optional add
// ---------------------------------------------------------------------------
template <int M>
__global__ void __launch_bounds__(kFFTThreads) k_c2r_rows_fast(const __grid_constant__ CubeSet cs, const __grid_constant__ CubeSet addend,
                                                               const float2 *__restrict__ twg, int nrows,
                                                               float postscale, int epi)
{
  constexpr int LDW = kRows + 1;
  constexpr int NX = 2 * M, CN = M + 1, RN = 2 * CN;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf = (float2 *)smem_raw;
  float2 *tw = buf + M * LDW;
  const int r0 = blockIdx.x * kRows;
  const int nr = min(kRows, nrows - r0);
  float *base = (float *)cs.ptr[blockIdx.z] + (long)r0 * RN;
  for (int t = threadIdx.x; t < NX; t += kFFTThreads) tw[t] = twg[t];
  // pack X[k], conj X[M-k] of every row straight from global memory (the
  // second read of each row hits L1)
  constexpr int NIT = (kRows * M + kFFTThreads - 1) / kFFTThreads;
  float2 xk[NIT], xm[NIT];
#pragma unroll
  for (int q = 0; q < NIT; q++) {
    const int t = q * kFFTThreads + threadIdx.x;
    const int row = t / M, k = t % M;
    if ((t < kRows * M) && row < nr) {
      const float2 *rp = (const float2 *)(base + (long)row * RN);
      xk[q] = __ldg(rp + k);
      xm[q] = __ldg(rp + (M - k));
    } else {
      xk[q] = make_float2(0.f, 0.f);
      xm[q] = make_float2(0.f, 0.f);
    }
  }
  __syncthreads();  // twiddles staged
#pragma unroll
  for (int q = 0; q < NIT; q++) {
    const int t = q * kFFTThreads + threadIdx.x;
    if (t < kRows * M) {
      const int row = t / M, k = t % M;
      float2 Xk = xk[q], Xm = xm[q];
      if (k == 0) { Xk.y = 0.f; Xm.y = 0.f; }  // rfftw_c2hc keeps only Re of DC and Nyquist
      Xm.y = -Xm.y;
      const float2 E = cadd<float>(Xk, Xm);
      const float2 O = cmulc<float>(csub<float>(Xk, Xm), tw[k]);
      buf[k * LDW + row] = make_float2(E.x - O.y, E.y + O.x);
    }
  }
  __syncthreads();
  cstages<float, M, kRows, LDW, 2>(buf, tw, +1);
  const float *add = addend.ptr[blockIdx.z] ? (const float *)addend.ptr[blockIdx.z] + (long)r0 * RN : nullptr;
  for (int t = threadIdx.x; t < nr * CN; t += kFFTThreads) {
    const int row = t / CN, e = t - row * CN;
    float2 z = (e < M) ? buf[e * LDW + row] : make_float2(0.f, 0.f);
    z.x *= postscale;
    z.y *= postscale;
    if (add) {
      const float2 a = ((const float2 *)(add + (long)row * RN))[e];
      z.x += a.x;
      z.y += a.y;
    }
    z.x = epilogue<float>(z.x, epi);
    z.y = epilogue<float>(z.y, epi);
    ((float2 *)(base + (long)row * RN))[e] = z;
  }
}

// host-side dispatch (fft_fast_*.cu): return 1 if a specialisation ran the pass
int tma_cols(const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride, long batch_stride, int nbatch,
             int sign, const float2 *tw, cudaStream_t st);
// no_alloc keeps the pass off kernels that allocate on first use (the TMA
// column pass and its device fault word)
int fast_cols(const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride, long batch_stride, int nbatch,
              int sign, const float2 *tw, cudaStream_t st, int *done_cols, bool no_alloc = false);
int fast_rows(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nxp, int nrows, float scale,
              const float2 *tw, cudaStream_t st, int epi = kEpiNone);
// x and y passes of one z-plane per cluster (fft_xy.cu): 1 if they ran, 0 when (nxp, nyp) has no plane
// kernel or the tuning table (CG_TUNE_XY_PLANE) selects the separate passes
int xy_planes(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nxp, int nyp, int nzp,
              float scale, cudaStream_t st, int epi);
// four-step kernels (fft_4step_*.cu); chosen by the tuning table
int four_step_cols(int minb, const CubeSet &cs, int ncubes, int n, int ncols, long axis_stride, long batch_stride,
                   int nbatch, int sign, const float2 *tw, cudaStream_t st);
int four_step_rows(bool forward, const CubeSet &cs, const CubeSet &addend, int ncubes, int nxp, int nrows, float scale,
                   const float2 *tw, cudaStream_t st, int epi = kEpiNone);

}  // namespace cg
