// Column pass of length 256 fed by the tensor memory accelerator.
//
// A persistent CTA walks the tile list (16 adjacent columns x 256 elements of
// one batch row) with two shared stage buffers: one thread issues the
// cp.async.bulk.tensor loads of tile i+1 (completion counted on an mbarrier)
// while the CTA transforms tile i, so HBM reads stay in flight through the
// arithmetic without holding registers.  The transform is the four-step
// 16 x 16 of k_fft_cols_4s: pass 1 reads its 16 operands from the stage
// buffer, does a 16-point DFT and the W_256^(n2 k1) twiddles and writes the
// exchange back into the same buffer; pass 2 does the second 16-point DFT and
// stores straight to global memory.
//
// Tensor maps need 16-byte strides, and the FFTGrid complex row pitch is
// cnxp = nxp/2 + 1 elements of 8 bytes (1032 bytes at nxp = 256).  The maps
// therefore view a cube as "super-rows" of two rows: dims (2 cnxp, nyp/2, nzp)
// with strides (16 cnxp, 8 cnxp nyp) bytes, which needs nyp even.  Row 2s of a
// super-row starts at element 0, row 2s+1 at element cnxp; every box starts at
// an even element, so its byte offset is a multiple of 16.
//  * y pass (batch = z-plane): box A (16, nyp/2, 1) at element 16g holds the
//    even rows of column group g; box B (WB, nyp/2, 1) at element
//    (cnxp + 16g) & ~1 holds the odd rows, shifted by sh = cnxp & 1 columns
//    (WB = 16 + 2 sh keeps the box a multiple of 16 bytes).
//  * z pass (batch = y row b): one box (16, 1, nzp) at element 16g (b even) or
//    cnxp + 16g - sh (b odd): odd rows use column groups shifted by -sh.
// Columns outside 0..cnxp-1 (a group's tail, or the column before the first
// shifted group) are loaded but never stored.
#pragma once

#include <cuda.h>

#include "fft_4step.cuh"

namespace cg {

constexpr int kTmaN = 256;      // transform length
constexpr int kTmaW = 16;       // columns per tile
constexpr int kTmaBuf = 4352;   // complex elements per stage buffer (y pass: 128*16 + 128*18)
constexpr int kTmaWaitLimit = 1 << 20;

struct ColsTmaArgs {
  CUtensorMap mapA[kMaxBatch];  // y pass: box (16, nyp/2, 1); z pass: box (16, 1, nzp)
  CUtensorMap mapB[kMaxBatch];  // y pass: box (16 + 2 sh, nyp/2, 1); unused by the z pass
  float2 *ptr[kMaxBatch];
  long plane;   // cnxp * nyp
  int cnxp;
  int nyp;
  int nbatch;   // z-planes (y pass) or y rows (z pass)
  int ngroups;  // column groups per batch row
  int ntiles;   // ncubes * nbatch * ngroups
  int *fault;   // set to 1 when a wait for a tile gives up
};

__device__ __forceinline__ unsigned tma_smem(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// true once the phase of the given parity has completed; false after
// kTmaWaitLimit polls
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity)
{
  for (int it = 0; it < kTmaWaitLimit; it++) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap *map, int x, int y, int z, unsigned bar)
{
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(dst), "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// AXIS 0: transform along y (nyp = 256), batch over z-planes.
// AXIS 1: transform along z (nzp = 256), batch over y rows.
template <int AXIS>
__global__ void __launch_bounds__(kFFTThreads, 3) k_fft_cols_tma(const __grid_constant__ ColsTmaArgs a,
                                                                 const float2 *__restrict__ twg, int sign)
{
  constexpr int N1 = 16, N2 = 16, W = kTmaW;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // stage buffers at a 128-byte boundary (the launch adds 128 bytes of slack)
  const unsigned raw = tma_smem(smem_raw);
  float2 *buf0 = (float2 *)(smem_raw + (((raw + 127u) & ~127u) - raw));
  float2 *tw = buf0 + 2 * kTmaBuf;
  __shared__ __align__(8) unsigned long long mbar[2];
  const int cnxp = a.cnxp, sh = cnxp & 1;
  const int per_cube = a.nbatch * a.ngroups;
  const int half = a.nyp >> 1;
  const int wb = 16 + 2 * sh;

  if (threadIdx.x == 0) {
    mbar_init(tma_smem(&mbar[0]), 1);
    mbar_init(tma_smem(&mbar[1]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int t = threadIdx.x; t < kTmaN; t += kFFTThreads) tw[t] = twg[t];
  __syncthreads();

  // thread 0: issue the loads of tile t into stage buffer s
  auto issue = [&](int t, int s) {
    const int cube = t / per_cube, r = t - cube * per_cube;
    const int b = r / a.ngroups, g = r - b * a.ngroups;
    const unsigned dst = tma_smem(buf0 + s * kTmaBuf), bar = tma_smem(&mbar[s]);
    if (AXIS == 0) {
      mbar_expect_tx(bar, (unsigned)((16 + wb) * half * 8));
      tma_load_3d(dst, &a.mapA[cube], 16 * g, 0, b, bar);
      tma_load_3d(dst + 16 * half * 8, &a.mapB[cube], (cnxp + 16 * g) & ~1, 0, b, bar);
    } else {
      mbar_expect_tx(bar, (unsigned)(16 * kTmaN * 8));
      const int xe = (b & 1) ? cnxp + 16 * g - sh : 16 * g;
      tma_load_3d(dst, &a.mapA[cube], xe, b >> 1, 0, bar);
    }
  };

  int tile = blockIdx.x;
  if (threadIdx.x == 0 && tile < a.ntiles) issue(tile, 0);
  const int c = threadIdx.x % W, q = threadIdx.x / W;  // lane column; n2 in pass 1, k1 in pass 2
  bool fail = false;
  int fail_it = 0;
  // pass-1 operand e = 16 n1 + q of column c sits at p1 + n1 * s1 in a stage
  // buffer (e has the parity of q: even rows in box A, odd rows in box B)
  int p1, s1;
  if (AXIS == 0) {
    if (q & 1) p1 = 16 * half + (q >> 1) * wb + c + sh, s1 = 8 * wb;
    else p1 = (q >> 1) * 16 + c, s1 = 8 * 16;
  } else {
    p1 = q * 16 + c, s1 = N2 * 16;
  }
  for (int it = 0; tile < a.ntiles; it++, tile += gridDim.x) {
    const int s = it & 1;
    float2 *cur = buf0 + s * kTmaBuf;
    const int next = tile + gridDim.x;
    const bool ok = mbar_wait(tma_smem(&mbar[s]), (unsigned)((it >> 1) & 1));
    const int cube = tile / per_cube, r = tile - cube * per_cube;
    const int b = r / a.ngroups, g = r - b * a.ngroups;
    float2 v[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; n1++) v[n1] = cur[p1 + n1 * s1];
    if (__syncthreads_or(!ok)) {  // every operand read; a failed wait ends the CTA
      fail = true;
      fail_it = it;
      break;
    }
    if (threadIdx.x == 0 && next < a.ntiles) {
      // every thread is past the barrier above, so the other buffer's last
      // reads (the previous tile's pass 2) are done; order those generic
      // accesses before the async writes of the next tile's loads
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(next, s ^ 1);
    }
    reg_fft<float, N1, N2>(v, sign, tw);
#pragma unroll
    for (int k1 = 1; k1 < N1; k1++) v[k1] = cmul<float>(v[k1], tw_at<float>(tw, q * k1, sign));
#pragma unroll
    for (int k1 = 0; k1 < N1; k1++) cur[(k1 * N2 + q) * W + c] = v[k1];
    __syncthreads();
    // pass 2: k1 = q
#pragma unroll
    for (int n2 = 0; n2 < N2; n2++) v[n2] = cur[(q * N2 + n2) * W + c];
    reg_fft<float, N2, N1>(v, sign, tw);
    const int x = AXIS == 0 ? 16 * g + c : 16 * g + c - ((b & 1) ? sh : 0);
    if (x >= 0 && x < cnxp) {
      float2 *p;
      long as;
      if (AXIS == 0) { p = a.ptr[cube] + (long)b * a.plane + x; as = cnxp; }
      else { p = a.ptr[cube] + (long)b * cnxp + x; as = a.plane; }
#pragma unroll
      for (int k2 = 0; k2 < N2; k2++) p[(long)(q + N1 * k2) * as] = v[k2];
    }
    // no barrier here: the next tile's first barrier orders this tile's pass-2
    // reads before this buffer is refilled
  }
  if (fail && threadIdx.x == 0) {
    atomicExch(a.fault, 1);
    // let the load still in flight land (bounded) before the CTA's shared
    // memory is released: the tile whose wait gave up (the next tile's loads
    // are issued only after a successful wait)
    mbar_wait(tma_smem(&mbar[fail_it & 1]), (unsigned)((fail_it >> 1) & 1));
  }
}

}  // namespace cg
