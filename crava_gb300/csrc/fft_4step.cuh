// Four-step FFT passes: a length-N transform split as N = N1 x N2 and done
// mostly in registers.
//
//   x[n], n = N2*n1 + n2        X[k], k = k1 + N1*k2
//   X[k1 + N1*k2] = sum_n2 W_N2^(n2 k2) * [ W_N^(n2 k1) * sum_n1 x[N2 n1 + n2] W_N1^(n1 k1) ]
//
// Pass 1: one thread per (line, n2) loads its N1 inputs straight from global
// memory, does the N1-point DFT in registers and the W_N^(n2 k1) twiddles, and
// writes the N1 results to shared memory.  Pass 2: one thread per (line, k1)
// reads N2 values back, does the N2-point DFT in registers and stores the
// outputs straight to global memory.  Every element crosses shared memory
// once (one write, one read) instead of once per Stockham stage, which is what
// bounds the staged kernels in fft_fast.cuh.
//
// The in-register DFTs are fully unrolled Stockham plans (radices 8, 4, 2, 3,
// 5, 7 as in make_axis_plan): every index is a compile-time constant, so the
// stage permutations are register renames.  Twiddles come from the same
// forward table as the other kernels (W_L^t for the table length L), staged
// in shared memory.
#pragma once

#include "fft_fast.cuh"

namespace cg {

// all stages of a length-N DFT held in v[]; tw[m*TWS] = W_N^m (forward table)
template <typename T, int N, int TWS, int S = 0, int NS = 1>
__device__ __forceinline__ void reg_fft(C2<T> *v, int sign, const C2<T> *tw)
{
  if constexpr (S < plan_nstages(N)) {
    constexpr int R = plan_radix(N, S);
    constexpr int NB = N / R;
    constexpr int SPAN = N / (NS * R);
    C2<T> w[N];
#pragma unroll
    for (int j = 0; j < NB; j++) {
      C2<T> a[R];
#pragma unroll
      for (int r = 0; r < R; r++) a[r] = v[j + r * NB];
      const int jm = j % NS;
      if (NS > 1 && jm > 0) {
#pragma unroll
        for (int r = 1; r < R; r++) a[r] = cmul<T>(a[r], tw_at<T>(tw, jm * r * SPAN * TWS, sign));
      }
      dft_any<T, R>(a, sign, tw, NB * TWS);
      const int d = (j - jm) * R + jm;
#pragma unroll
      for (int r = 0; r < R; r++) w[d + r * NS] = a[r];
    }
#pragma unroll
    for (int i = 0; i < N; i++) v[i] = w[i];
    reg_fft<T, N, TWS, S + 1, NS * R>(v, sign, tw);
  }
}

// N1: the smallest divisor of N not below sqrt(N) (both factors stay small
// enough for registers; N1 is even for every specialised length)
__host__ __device__ constexpr int fs_n1(int n)
{
  for (int d = 1; d <= n; d++)
    if (n % d == 0 && d * d >= n) return d;
  return n;
}

// N1 for the x-row passes: for even M the smallest EVEN divisor not below
// sqrt(M) (the R2C unpack then pairs column 0 with N1/2), for odd M the
// smallest divisor not below sqrt(M) (column 0 is then unpaired)
__host__ __device__ constexpr int fs_n1_rows(int m)
{
  if (m % 2) return fs_n1(m);
  for (int d = 2; d <= m; d += 2)
    if (m % d == 0 && d * d >= m) return d;
  return m;
}

// pass-2 items per row of the R2C pass: column pairs (k1, N1 - k1), with
// column 0 paired with N1/2 (even N1) or alone (odd N1)
__host__ __device__ constexpr int fs_r2c_items(int m) { return (fs_n1_rows(m) + 1) / 2; }

// column tile width: 16 columns when both factors are >= 16 (256 items per
// pass), else 32
__host__ __device__ constexpr int fs_cols_w(int n)
{
  return (fs_n1(n) >= 16 && n / fs_n1(n) >= 16) ? 16 : 32;
}

// the tile shapes the tuning table chooses among per length (CG_TUNE_COLS_SHAPE):
// bit 0 swaps the factors (N1 = N / fs_n1(N), the largest divisor not above
// sqrt(N)), bit 1 takes the other tile width (16 <-> 32 columns)
__host__ __device__ constexpr int fs_shape_n1(int n, int shape) { return (shape & 1) ? n / fs_n1(n) : fs_n1(n); }
__host__ __device__ constexpr int fs_shape_w(int n, int shape)
{
  return (shape & 2) ? (fs_cols_w(n) == 16 ? 32 : 16) : fs_cols_w(n);
}

// ---------------------------------------------------------------------------
// strided column pass.  Full tiles are W adjacent columns of one batch row.
// The ntail columns left over in each batch row, taken row after row, form a
// list of ntail*nbatch columns cut into tail tiles of W: a tail tile reads runs
// of ntail adjacent elements and every lane but those of the last tile works.
// Grid columns x >= nfull hold the tail tiles, numbered (x - nfull)*nbatch + y.
// Shared layout: buf[(k1*N2 + n2)*W + c] (conflict-free for both passes).
// ---------------------------------------------------------------------------
template <int N, int W, int N1_, int MINB>
__global__ void __launch_bounds__(kFFTThreads, MINB) k_fft_cols_4s(const __grid_constant__ CubeSet cs, const float2 *__restrict__ twg,
                                                                   ColsGeom g, int sign)
{
  constexpr int N1 = N1_, N2 = N / N1;
  static_assert(N % N1 == 0, "N1 must divide N");
  constexpr int P1 = W * N2, P2 = W * N1;
  constexpr int B1 = (P1 + kFFTThreads - 1) / kFFTThreads, B2 = (P2 + kFFTThreads - 1) / kFFTThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf = (float2 *)smem_raw;
  float2 *tw = buf + N * W;
  float2 *cube = (float2 *)cs.ptr[blockIdx.z];
  float2 *base;
  int e0, tdiv, tvalid;  // lane c -> column (e0 + c) % tdiv of batch row (e0 + c) / tdiv; lanes c >= tvalid idle
  if ((int)blockIdx.x < g.nfull) {
    base = cube + (long)blockIdx.y * g.batch_stride + (long)blockIdx.x * W;
    e0 = 0;
    tdiv = W;
    tvalid = W;
  } else {
    const long tt = (long)((int)blockIdx.x - g.nfull) * g.nbatch + (int)blockIdx.y;
    const long ntot = (long)g.ntail * g.nbatch;
    if (tt * W >= ntot) return;
    base = cube + (long)g.nfull * W;
    e0 = (int)(tt * W);
    tdiv = g.ntail;
    tvalid = (int)min((long)W, ntot - tt * W);
  }
  const long as = g.axis_stride, bs = g.batch_stride;
  auto coff = [&](int c) -> long { return (long)((e0 + c) % tdiv) + (long)((e0 + c) / tdiv) * bs; };
  for (int t = threadIdx.x; t < N; t += kFFTThreads) tw[t] = twg[t];
  // pass 1, one item at a time (registers hold one item); the first item's
  // loads are issued before the barrier that publishes the twiddle table
  auto load1 = [&](int q, float2 *v) {
    const int t = q * kFFTThreads + threadIdx.x;
    const int c = t % W, n2 = t / W;
    const bool ok = (P1 % kFFTThreads == 0 || t < P1) && c < tvalid;
    const long o = ok ? coff(c) : 0;
#pragma unroll
    for (int n1 = 0; n1 < N1; n1++)
      v[n1] = ok ? base[(long)(N2 * n1 + n2) * as + o] : make_float2(0.f, 0.f);
  };
  float2 v[N1];
  load1(0, v);
  __syncthreads();
#pragma unroll
  for (int q = 0; q < B1; q++) {
    if (q > 0) load1(q, v);
    const int t = q * kFFTThreads + threadIdx.x;
    if (P1 % kFFTThreads == 0 || t < P1) {
      const int c = t % W, n2 = t / W;
      reg_fft<float, N1, N2>(v, sign, tw);
#pragma unroll
      for (int k1 = 1; k1 < N1; k1++) v[k1] = cmul<float>(v[k1], tw_at<float>(tw, n2 * k1, sign));
#pragma unroll
      for (int k1 = 0; k1 < N1; k1++) buf[(k1 * N2 + n2) * W + c] = v[k1];
    }
  }
  __syncthreads();
  // pass 2
#pragma unroll
  for (int q = 0; q < B2; q++) {
    const int t = q * kFFTThreads + threadIdx.x;
    if (P2 % kFFTThreads == 0 || t < P2) {
      const int c = t % W, k1 = t / W;
      float2 u[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; n2++) u[n2] = buf[(k1 * N2 + n2) * W + c];
      reg_fft<float, N2, N1>(u, sign, tw);
      if (c < tvalid) {
        const long o = coff(c);
#pragma unroll
        for (int k2 = 0; k2 < N2; k2++) base[(long)(k1 + N1 * k2) * as + o] = u[k2];
      }
    }
  }
}

// rows per CTA for the row passes: enough (row, n2) items and (row, k1 pair)
// items for the 256 threads of both passes
__host__ __device__ constexpr int fs_rows_per_cta(int m)
{
  const int a = kFFTThreads / (m / fs_n1_rows(m)), b = kFFTThreads / fs_r2c_items(m);
  return a > b ? a : b;
}

// pitch (float2) of one row's exchange block: >= N2*(N1+1), = 8 mod 16 so the
// two rows a half-warp touches fall in opposite bank halves
__host__ __device__ constexpr int fs_row_pitch(int m)
{
  const int need = (m / fs_n1_rows(m)) * (fs_n1_rows(m) + 1);
  return need + ((8 - need % 16) + 16) % 16;
}

// ---------------------------------------------------------------------------
// x rows, real -> half spectrum (even nxp = 2M), prescale applied.
// The 2M reals of a row are read as M complex z[n] = x[2n] + i x[2n+1]; the
// M-point four-step gives Z[k], and the half-length unpack
//   X[k] = E + W_2M^k O,  E = (Z[k] + conj Z[M-k])/2,  O = -i (Z[k] - conj Z[M-k])/2
// needs Z[k] and Z[M-k] together: a pass-2 thread transforms the two columns
// k1 and N1-k1, which hold exactly those partners; column 0 holds its own
// partners and is paired with N1/2 when N1 is even, alone when N1 is odd.
// ---------------------------------------------------------------------------
template <int M>
__global__ void __launch_bounds__(kFFTThreads) k_r2c_rows_4s(const __grid_constant__ CubeSet cs, const float2 *__restrict__ twg, int nrows,
                                                             float prescale)
{
  constexpr int N1 = fs_n1_rows(M), N2 = M / N1, NI = fs_r2c_items(M);
  constexpr int RPC = fs_rows_per_cta(M), P = fs_row_pitch(M), Q = N1 + 1;
  constexpr int NX = 2 * M, CN = M + 1;
  constexpr int P1 = RPC * N2, P2 = RPC * NI;
  constexpr int B1 = (P1 + kFFTThreads - 1) / kFFTThreads, B2 = (P2 + kFFTThreads - 1) / kFFTThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf = (float2 *)smem_raw;
  float2 *tw = buf + RPC * P;
  float2 *tw1 = tw + NX;  // tw1[k1 * N2 + n2] = W_2M^(2 n2 k1): pass-1 twiddles without bank conflicts
  const int r0 = blockIdx.x * RPC;
  const int nr = min(RPC, nrows - r0);
  float2 *base = (float2 *)cs.ptr[blockIdx.z] + (long)r0 * CN;
  for (int t = threadIdx.x; t < NX; t += kFFTThreads) tw[t] = twg[t];
  for (int t = threadIdx.x; t < N1 * N2; t += kFFTThreads) tw1[t] = twg[2 * (t % N2) * (t / N2)];
  auto load1 = [&](int q, float2 *v) {
    const int t = q * kFFTThreads + threadIdx.x;
    const int n2 = t % N2, row = t / N2;
    const bool ok = (P1 % kFFTThreads == 0 || t < P1) && row < nr;
    const float2 *rp = base + (long)row * CN;
#pragma unroll
    for (int n1 = 0; n1 < N1; n1++) v[n1] = ok ? rp[N2 * n1 + n2] : make_float2(0.f, 0.f);
  };
  float2 v[N1];
  load1(0, v);
  __syncthreads();
#pragma unroll
  for (int q = 0; q < B1; q++) {
    if (q > 0) load1(q, v);
    const int t = q * kFFTThreads + threadIdx.x;
    if (P1 % kFFTThreads == 0 || t < P1) {
      const int n2 = t % N2, row = t / N2;
      reg_fft<float, N1, 2 * N2>(v, -1, tw);
#pragma unroll
      for (int k1 = 1; k1 < N1; k1++) v[k1] = cmul<float>(v[k1], tw1[k1 * N2 + n2]);
#pragma unroll
      for (int k1 = 0; k1 < N1; k1++) buf[row * P + n2 * Q + k1] = v[k1];
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < B2; q++) {
    const int t = q * kFFTThreads + threadIdx.x;
    if (P2 % kFFTThreads == 0 || t < P2) {
      const int ka = t % NI, row = t / NI;
      // partner column (none for column 0 when N1 is odd: it is read but not used)
      const bool has_b = ka != 0 || N1 % 2 == 0;
      const int kb = ka == 0 ? (N1 % 2 == 0 ? N1 / 2 : 0) : N1 - ka;
      float2 a[N2], b[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; n2++) {
        a[n2] = buf[row * P + n2 * Q + ka];
        b[n2] = buf[row * P + n2 * Q + kb];
      }
      reg_fft<float, N2, 2 * N1>(a, -1, tw);
      if (has_b) reg_fft<float, N2, 2 * N1>(b, -1, tw);
      if (row < nr) {
        float2 *op = base + (long)row * CN;
        // Z[M-k] for k = ka + N1*k2 sits in b[N2-1-k2]; for ka = 0 it is a[(N2-k2) % N2]
        // and for kb = N1/2 (paired with ka = 0) it is b[N2-1-k2]; for kb = N1-ka it is a[N2-1-k2]
#pragma unroll
        for (int k2 = 0; k2 < N2; k2++) {
          {
            const int k = ka + N1 * k2;
            const float2 A = a[k2];
            const float2 Bc = ka == 0 ? a[(N2 - k2) % N2] : b[N2 - 1 - k2];
            const float2 B = make_float2(Bc.x, -Bc.y);
            const float2 E = make_float2((A.x + B.x) * 0.5f, (A.y + B.y) * 0.5f);
            const float2 O = make_float2((A.y - B.y) * 0.5f, -(A.x - B.x) * 0.5f);
            float2 X = cadd<float>(E, cmul<float>(tw[k], O));
            op[k] = make_float2(X.x * prescale, X.y * prescale);
          }
          if (has_b) {
            const int k = kb + N1 * k2;
            const float2 A = b[k2];
            const float2 Bc = ka == 0 ? b[N2 - 1 - k2] : a[N2 - 1 - k2];
            const float2 B = make_float2(Bc.x, -Bc.y);
            const float2 E = make_float2((A.x + B.x) * 0.5f, (A.y + B.y) * 0.5f);
            const float2 O = make_float2((A.y - B.y) * 0.5f, -(A.x - B.x) * 0.5f);
            float2 X = cadd<float>(E, cmul<float>(tw[k], O));
            op[k] = make_float2(X.x * prescale, X.y * prescale);
          }
        }
        if (ka == 0) {
          // Nyquist bin k = M: A = Z[0], B = conj Z[0], W_2M^M = -1
          const float2 A = a[0];
          op[M] = make_float2((A.x - A.y) * prescale, 0.f);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// x rows, half spectrum -> real (even nxp = 2M), postscale and optional add.
// Pass 1 packs Z[k] = E + i O from X[k] and conj X[M-k] read straight from
// global memory (the second read of a row hits L1), so no shared memory is
// used before the exchange; pass 2 stores z[n] = (x[2n], x[2n+1]).
// ---------------------------------------------------------------------------
// ADD: the launch has addends (the posterior-mean add of simulation); they are
// loaded before pass 2's DFT so their latency overlaps it (a load after each
// store could not be hoisted over the stores, which may alias)
template <int M, bool ADD>
__global__ void __launch_bounds__(kFFTThreads) k_c2r_rows_4s(const __grid_constant__ CubeSet cs, const __grid_constant__ CubeSet addend,
                                                             const float2 *__restrict__ twg, int nrows,
                                                             float postscale, int epi)
{
  constexpr int N1 = fs_n1_rows(M), N2 = M / N1;
  constexpr int RPC = fs_rows_per_cta(M), P = fs_row_pitch(M), Q = N1 + 1;
  constexpr int NX = 2 * M, CN = M + 1;
  constexpr int P1 = RPC * N2, P2 = RPC * N1;
  constexpr int B1 = (P1 + kFFTThreads - 1) / kFFTThreads, B2 = (P2 + kFFTThreads - 1) / kFFTThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf = (float2 *)smem_raw;
  float2 *tw = buf + RPC * P;
  float2 *tw1 = tw + NX;  // tw1[k1 * N2 + n2] = W_2M^(2 n2 k1): pass-1 twiddles without bank conflicts
  const int r0 = blockIdx.x * RPC;
  const int nr = min(RPC, nrows - r0);
  float2 *base = (float2 *)cs.ptr[blockIdx.z] + (long)r0 * CN;
  for (int t = threadIdx.x; t < NX; t += kFFTThreads) tw[t] = twg[t];
  for (int t = threadIdx.x; t < N1 * N2; t += kFFTThreads) tw1[t] = twg[2 * (t % N2) * (t / N2)];
  // X[M-k] for k = N2 n1 + n2 (n2 > 0) is X[N2 (N1-1-n1) + (N2-n2)], the
  // xk[N1-1-n1] of the item (N2-n2, row); when a row's N2 items sit in
  // consecutive lanes of one warp it is taken from that lane by a shuffle, and
  // the n2 = 0 item reads its partners from its own xk (X[M] is loaded).
  // Otherwise X[M-k] is loaded as well (the second read of a row hits L1).
  constexpr bool kShfl = 32 % N2 == 0 && P1 % 32 == 0;
  auto load1 = [&](int q, float2 *xk, float2 *xm) {
    const int t = q * kFFTThreads + threadIdx.x;
    const int n2 = t % N2, row = t / N2;
    const bool ok = (P1 % kFFTThreads == 0 || t < P1) && row < nr;
    const float2 *rp = base + (long)row * CN;
#pragma unroll
    for (int n1 = 0; n1 < N1; n1++) {
      const int k = N2 * n1 + n2;
      xk[n1] = ok ? __ldg(rp + k) : make_float2(0.f, 0.f);
      if constexpr (!kShfl) xm[n1] = ok ? __ldg(rp + (M - k)) : make_float2(0.f, 0.f);
    }
    if constexpr (kShfl) xm[0] = ok && n2 == 0 ? __ldg(rp + M) : make_float2(0.f, 0.f);
  };
  float2 xk[N1], xm[kShfl ? 1 : N1];
  load1(0, xk, xm);
  __syncthreads();  // twiddles staged
#pragma unroll
  for (int q = 0; q < B1; q++) {
    if (q > 0) load1(q, xk, xm);
    const int t = q * kFFTThreads + threadIdx.x;
    if (P1 % kFFTThreads == 0 || t < P1) {  // warp-uniform when kShfl
      const int n2 = t % N2, row = t / N2;
      const int lane = threadIdx.x & 31;
      const int partner = (lane & ~(N2 - 1)) | ((N2 - n2) & (N2 - 1));
      float2 v[N1];
#pragma unroll
      for (int n1 = 0; n1 < N1; n1++) {
        const int k = N2 * n1 + n2;
        float2 Xk = xk[n1], Xm;
        if constexpr (kShfl) {
          const float2 mine = xk[N1 - 1 - n1];
          const float2 other = make_float2(__shfl_sync(0xffffffffu, mine.x, partner),
                                           __shfl_sync(0xffffffffu, mine.y, partner));
          Xm = n2 != 0 ? other : (n1 == 0 ? xm[0] : xk[(N1 - n1) % N1]);
        } else {
          Xm = xm[n1];
        }
        if (k == 0) { Xk.y = 0.f; Xm.y = 0.f; }  // rfftw_c2hc keeps only Re of DC and Nyquist
        Xm.y = -Xm.y;
        const float2 E = cadd<float>(Xk, Xm);
        const float2 O = cmulc<float>(csub<float>(Xk, Xm), tw[k]);
        v[n1] = make_float2(E.x - O.y, E.y + O.x);
      }
      reg_fft<float, N1, 2 * N2>(v, +1, tw);
#pragma unroll
      for (int k1 = 1; k1 < N1; k1++) v[k1] = cmul<float>(v[k1], tw_at<float>(tw1, k1 * N2 + n2, +1));
#pragma unroll
      for (int k1 = 0; k1 < N1; k1++) buf[row * P + n2 * Q + k1] = v[k1];
    }
  }
  __syncthreads();
  const float2 *add = ADD && addend.ptr[blockIdx.z] ? (const float2 *)addend.ptr[blockIdx.z] + (long)r0 * CN : nullptr;
#pragma unroll
  for (int q = 0; q < B2; q++) {
    const int t = q * kFFTThreads + threadIdx.x;
    if (P2 % kFFTThreads == 0 || t < P2) {
      const int k1 = t % N1, row = t / N1;
      float2 u[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; n2++) u[n2] = buf[row * P + n2 * Q + k1];
      const float2 *ap = (ADD && add && row < nr) ? add + (long)row * CN : nullptr;
      float2 av[ADD ? N2 + 1 : 1];
      if constexpr (ADD) {
        if (ap) {
#pragma unroll
          for (int k2 = 0; k2 < N2; k2++) av[k2] = __ldg(ap + k1 + N1 * k2);
          av[N2] = k1 == 0 ? __ldg(ap + M) : make_float2(0.f, 0.f);
        }
      }
      reg_fft<float, N2, 2 * N1>(u, +1, tw);
      if (row < nr) {
        float2 *op = base + (long)row * CN;
#pragma unroll
        for (int k2 = 0; k2 < N2; k2++) {
          const int e = k1 + N1 * k2;
          float2 z = make_float2(u[k2].x * postscale, u[k2].y * postscale);
          if constexpr (ADD) {
            if (ap) {
              z.x += av[k2].x;
              z.y += av[k2].y;
            }
          }
          op[e] = make_float2(epilogue<float>(z.x, epi), epilogue<float>(z.y, epi));
        }
        if (k1 == 0) {
          // the row's padding pair: zero, plus the addend's padding
          float2 z = make_float2(0.f, 0.f);
          if constexpr (ADD) {
            if (ap) {
              z.x += av[N2].x;
              z.y += av[N2].y;
            }
          }
          op[M] = make_float2(epilogue<float>(z.x, epi), epilogue<float>(z.y, epi));
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// x rows of ODD length NX (no half-length trick): the real row is transformed
// as a complex row with zero imaginary part, and the first cnxp = (NX+1)/2
// bins are kept (R2C); the inverse rebuilds the Hermitian row from those bins
// (Im of DC dropped, as rfftw_c2hc does) and keeps the real part (C2R).
// Rows have pitch NX + 1 floats = cnxp complex.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int fs_odd_rows_per_cta(int nx)
{
  return kFFTThreads / (nx / fs_n1(nx)) < 1 ? 1 : kFFTThreads / (nx / fs_n1(nx));
}
__host__ __device__ constexpr int fs_odd_row_pitch(int nx)
{
  const int need = (nx / fs_n1(nx)) * (fs_n1(nx) + 1);
  return need + ((8 - need % 16) + 16) % 16;
}

template <int NX>
__global__ void __launch_bounds__(kFFTThreads) k_r2c_rows_odd(const __grid_constant__ CubeSet cs, const float2 *__restrict__ twg, int nrows,
                                                              float prescale)
{
  constexpr int N1 = fs_n1(NX), N2 = NX / N1, CN = (NX + 1) / 2, RN = NX + 1;
  constexpr int RPC = fs_odd_rows_per_cta(NX), P = fs_odd_row_pitch(NX), Q = N1 + 1;
  constexpr int P1 = RPC * N2, P2 = RPC * N1;
  constexpr int B1 = (P1 + kFFTThreads - 1) / kFFTThreads, B2 = (P2 + kFFTThreads - 1) / kFFTThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf = (float2 *)smem_raw;
  float2 *tw = buf + RPC * P;
  const int r0 = blockIdx.x * RPC;
  const int nr = min(RPC, nrows - r0);
  float *rbase = (float *)cs.ptr[blockIdx.z] + (long)r0 * RN;
  float2 *cbase = (float2 *)cs.ptr[blockIdx.z] + (long)r0 * CN;
  for (int t = threadIdx.x; t < NX; t += kFFTThreads) tw[t] = twg[t];
  auto load1 = [&](int q, float2 *v) {
    const int t = q * kFFTThreads + threadIdx.x;
    const int n2 = t % N2, row = t / N2;
    const bool ok = (P1 % kFFTThreads == 0 || t < P1) && row < nr;
    const float *rp = rbase + (long)row * RN;
#pragma unroll
    for (int n1 = 0; n1 < N1; n1++) v[n1] = make_float2(ok ? rp[N2 * n1 + n2] : 0.f, 0.f);
  };
  float2 v[N1];
  load1(0, v);
  __syncthreads();
#pragma unroll
  for (int q = 0; q < B1; q++) {
    if (q > 0) load1(q, v);
    const int t = q * kFFTThreads + threadIdx.x;
    if (P1 % kFFTThreads == 0 || t < P1) {
      const int n2 = t % N2, row = t / N2;
      reg_fft<float, N1, N2>(v, -1, tw);
#pragma unroll
      for (int k1 = 1; k1 < N1; k1++) v[k1] = cmul<float>(v[k1], tw[n2 * k1]);
#pragma unroll
      for (int k1 = 0; k1 < N1; k1++) buf[row * P + n2 * Q + k1] = v[k1];
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < B2; q++) {
    const int t = q * kFFTThreads + threadIdx.x;
    if (P2 % kFFTThreads == 0 || t < P2) {
      const int k1 = t % N1, row = t / N1;
      float2 u[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; n2++) u[n2] = buf[row * P + n2 * Q + k1];
      reg_fft<float, N2, N1>(u, -1, tw);
      if (row < nr) {
        float2 *op = cbase + (long)row * CN;
#pragma unroll
        for (int k2 = 0; k2 < N2; k2++) {
          const int k = k1 + N1 * k2;
          if (k < CN) op[k] = make_float2(u[k2].x * prescale, u[k2].y * prescale);
        }
      }
    }
  }
}

template <int NX>
__global__ void __launch_bounds__(kFFTThreads) k_c2r_rows_odd(const __grid_constant__ CubeSet cs, const __grid_constant__ CubeSet addend,
                                                              const float2 *__restrict__ twg, int nrows,
                                                              float postscale, int epi)
{
  constexpr int N1 = fs_n1(NX), N2 = NX / N1, CN = (NX + 1) / 2, RN = NX + 1;
  constexpr int RPC = fs_odd_rows_per_cta(NX), P = fs_odd_row_pitch(NX), Q = N1 + 1;
  constexpr int P1 = RPC * N2, P2 = RPC * N1;
  constexpr int B1 = (P1 + kFFTThreads - 1) / kFFTThreads, B2 = (P2 + kFFTThreads - 1) / kFFTThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *buf = (float2 *)smem_raw;
  float2 *tw = buf + RPC * P;
  const int r0 = blockIdx.x * RPC;
  const int nr = min(RPC, nrows - r0);
  float *rbase = (float *)cs.ptr[blockIdx.z] + (long)r0 * RN;
  const float2 *cbase = (const float2 *)cs.ptr[blockIdx.z] + (long)r0 * CN;
  for (int t = threadIdx.x; t < NX; t += kFFTThreads) tw[t] = twg[t];
  // Hermitian row from the half spectrum: Z[k] = X[k] (k < CN), conj X[NX-k] above; Im X[0] dropped
  auto load1 = [&](int q, float2 *v) {
    const int t = q * kFFTThreads + threadIdx.x;
    const int n2 = t % N2, row = t / N2;
    const bool ok = (P1 % kFFTThreads == 0 || t < P1) && row < nr;
    const float2 *cp = cbase + (long)row * CN;
#pragma unroll
    for (int n1 = 0; n1 < N1; n1++) {
      const int k = N2 * n1 + n2;
      float2 z = make_float2(0.f, 0.f);
      if (ok) {
        if (k < CN) {
          z = __ldg(cp + k);
          if (k == 0) z.y = 0.f;
        } else {
          const float2 x = __ldg(cp + (NX - k));
          z = make_float2(x.x, -x.y);
        }
      }
      v[n1] = z;
    }
  };
  float2 v[N1];
  load1(0, v);
  __syncthreads();  // twiddles staged; every thread's row reads done before the exchange
#pragma unroll
  for (int q = 0; q < B1; q++) {
    if (q > 0) load1(q, v);
    const int t = q * kFFTThreads + threadIdx.x;
    if (P1 % kFFTThreads == 0 || t < P1) {
      const int n2 = t % N2, row = t / N2;
      reg_fft<float, N1, N2>(v, +1, tw);
#pragma unroll
      for (int k1 = 1; k1 < N1; k1++) v[k1] = cmul<float>(v[k1], tw_at<float>(tw, n2 * k1, +1));
#pragma unroll
      for (int k1 = 0; k1 < N1; k1++) buf[row * P + n2 * Q + k1] = v[k1];
    }
  }
  __syncthreads();
  const float *add = addend.ptr[blockIdx.z] ? (const float *)addend.ptr[blockIdx.z] + (long)r0 * RN : nullptr;
#pragma unroll
  for (int q = 0; q < B2; q++) {
    const int t = q * kFFTThreads + threadIdx.x;
    if (P2 % kFFTThreads == 0 || t < P2) {
      const int k1 = t % N1, row = t / N1;
      float2 u[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; n2++) u[n2] = buf[row * P + n2 * Q + k1];
      reg_fft<float, N2, N1>(u, +1, tw);
      if (row < nr) {
        float *op = rbase + (long)row * RN;
        const float *ap = add ? add + (long)row * RN : nullptr;
#pragma unroll
        for (int k2 = 0; k2 < N2; k2++) {
          const int e = k1 + N1 * k2;
          float x = u[k2].x * postscale;
          if (ap) x += ap[e];
          op[e] = epilogue<float>(x, epi);
        }
        if (k1 == 0) op[NX] = epilogue<float>(ap ? ap[NX] : 0.f, epi);  // the row's padding float
      }
    }
  }
}

}  // namespace cg
