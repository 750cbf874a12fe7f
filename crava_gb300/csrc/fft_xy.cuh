// x + y passes of a 3D transform in one launch: one z-plane per thread-block
// cluster, the plane's intermediate spectrum held in the cluster's shared
// memory (distributed shared memory), so the plane crosses HBM once per
// direction instead of twice.
//
// The in-place FFTGrid plane z of a cube is CN*NY complex values (CN = M+1,
// x fastest) starting at cube + z*CN*NY; a row is the rnxp = 2*CN floats of one
// y.  The cluster's CL CTAs split the plane two ways:
//   * by rows for the x pass: CTA r transforms rows [r*NY/CL, (r+1)*NY/CL);
//   * by columns for the y pass: CTA r owns the half-spectrum columns
//     [r*CW, min((r+1)*CW, CN)), CW = ceil(CN/CL), and holds all NY rows of
//     them in its shared array H (pitch HP).
// Forward (k_xy_r2c): x rows R2C (the four-step of k_r2c_rows_4s, prescale
// applied) with each output X[k] stored straight into the H of the CTA that
// owns column k (a st.shared::cluster for a peer), a cluster barrier, then the
// y columns of H (the four-step of k_fft_cols_4s) stored to global memory.
// Inverse (k_yx_c2r): y columns of the CTA's own columns loaded from global
// memory, inverse transformed and stored into its H, a cluster barrier, then
// the x rows C2R (the four-step of k_c2r_rows_4s) reading X[k] and X[M-k] from
// the owning CTA's H (ld.shared::cluster for a peer), postscale, addend and
// epilogue applied, real rows stored to global memory.
//
// The arithmetic of both passes is that of the separate four-step kernels
// (same plans, twiddles and operation order), so the results are identical to
// the x-row pass followed by the four-step column pass.
//
// Synchronisation: one cluster barrier before the first access to a peer's
// shared memory (every CTA of the cluster has started), one between the two
// passes, and, in the inverse, one before exit (no CTA leaves while a peer
// may still read its H).  These are hardware barriers over the cluster's own
// threads; no thread spins on memory.
#pragma once

#include "fft_4step.cuh"

namespace cg {

constexpr int kXYThreads = 512;

__device__ __forceinline__ unsigned cluster_rank()
{
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_map(unsigned local_smem, unsigned rank)
{
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(local_smem), "r"(rank));
  return r;
}
__device__ __forceinline__ void dsm_store(unsigned addr, float2 v)
{
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};\n" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ float2 dsm_load(unsigned addr)
{
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];\n" : "=f"(v.x), "=f"(v.y) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ void cluster_arrive_relaxed()
{
  asm volatile("barrier.cluster.arrive.relaxed.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_arrive()
{
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait()
{
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// hb[i] for a runtime i without indexing the array (which would place it in local memory)
template <int CL>
__device__ __forceinline__ unsigned pick(const unsigned (&hb)[CL], int i)
{
  unsigned a = hb[0];
#pragma unroll
  for (int r = 1; r < CL; r++) a = i == r ? hb[r] : a;
  return a;
}

// compile-time geometry of a plane kernel
template <int M, int NY, int CL>
struct XYGeom {
  static constexpr int CN = M + 1;                       // complex values per row
  static constexpr int CW = (CN + CL - 1) / CL;          // columns per CTA (the last CTA may own fewer)
  static constexpr int HP = CW + ((20 - CW % 16) % 16);  // H pitch (float2), = 4 mod 16: the x pass's stores
                                                         // (4 rows x 8 columns per warp) spread over all banks
  static constexpr int RPCT = NY / CL;                   // rows per CTA in the x pass
  // x pass (four-step over M = N1 x N2, as k_r2c_rows_4s / k_c2r_rows_4s)
  static constexpr int N1 = fs_n1_rows(M), N2 = M / N1, NI = fs_r2c_items(M);
  static constexpr int P = fs_row_pitch(M), Q = N1 + 1;
  static constexpr int RB0 = kXYThreads / (N2 > NI ? N2 : NI);
  static constexpr int RB = RB0 < RPCT ? RB0 : RPCT;  // rows per batch
  static constexpr int NBX = (RPCT + RB - 1) / RB;     // batches per CTA
  // y pass (four-step over NY = Y1 x Y2, as k_fft_cols_4s)
  static constexpr int Y1 = fs_n1(NY), Y2 = NY / Y1;
  static constexpr int W = kXYThreads / (Y1 > Y2 ? Y1 : Y2);  // columns per batch
  // shared memory (float2): H | exchange | x twiddles (2M) | x pass-1 twiddles (M) | y twiddles (NY)
  static constexpr int HSZ = NY * HP;
  static constexpr int XSZ = RB * P > W * NY ? RB * P : W * NY;
  static constexpr size_t SMEM = (size_t)(HSZ + XSZ + 2 * M + M + NY) * sizeof(float2);
  static_assert(NY % CL == 0, "rows must split evenly over the cluster");
};

// ---------------------------------------------------------------------------
// forward: x rows R2C into the cluster's H, then y columns to global memory
// ---------------------------------------------------------------------------
template <int M, int NY, int CL>
__global__ void __launch_bounds__(kXYThreads, 1) k_xy_r2c(const __grid_constant__ CubeSet cs,
                                                          const float2 *__restrict__ twx,
                                                          const float2 *__restrict__ twy, float prescale)
{
  using G = XYGeom<M, NY, CL>;
  constexpr int CN = G::CN, CW = G::CW, HP = G::HP, N1 = G::N1, N2 = G::N2, NI = G::NI, P = G::P, Q = G::Q;
  constexpr int RB = G::RB, Y1 = G::Y1, Y2 = G::Y2, W = G::W;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *H = (float2 *)smem_raw;
  float2 *buf = H + G::HSZ;
  float2 *tw = buf + G::XSZ;
  float2 *tw1 = tw + 2 * M;
  float2 *ty = tw1 + M;
  const unsigned rank = CL > 1 ? cluster_rank() : 0;
  float2 *plane = (float2 *)cs.ptr[blockIdx.z] + (long)blockIdx.y * CN * NY;
  for (int t = threadIdx.x; t < 2 * M; t += kXYThreads) tw[t] = twx[t];
  for (int t = threadIdx.x; t < N1 * N2; t += kXYThreads) tw1[t] = twx[2 * (t % N2) * (t / N2)];
  for (int t = threadIdx.x; t < NY; t += kXYThreads) ty[t] = twy[t];
  unsigned hb[CL];  // cluster address of every CTA's H
#pragma unroll
  for (int r = 0; r < CL; r++) hb[r] = CL > 1 ? cluster_map(smem_u32(H), r) : smem_u32(H);
  if constexpr (CL > 1) cluster_arrive_relaxed();  // waited for before the first store to a peer
  __syncthreads();

  // ---- x pass: rows [rank*RPCT, (rank+1)*RPCT) in batches of RB
  constexpr int PX1 = RB * N2, PX2 = RB * NI;
  constexpr int BX1 = (PX1 + kXYThreads - 1) / kXYThreads, BX2 = (PX2 + kXYThreads - 1) / kXYThreads;
  auto put = [&](int grow, int k, float2 v) {
    const int owner = k / CW, col = k - owner * CW;
    if (CL == 1 || owner == (int)rank) H[grow * HP + col] = v;
    else dsm_store(pick(hb, owner) + (unsigned)((grow * HP + col) * sizeof(float2)), v);
  };
#pragma unroll 1
  for (int b = 0; b < G::NBX; b++) {
    const int row0 = rank * G::RPCT + b * RB;
    const int nr = min(RB, (int)((rank + 1) * G::RPCT) - row0);
#pragma unroll
    for (int q = 0; q < BX1; q++) {
      const int t = q * kXYThreads + threadIdx.x;
      if (PX1 % kXYThreads == 0 || t < PX1) {
        const int n2 = t % N2, row = t / N2;
        float2 v[N1];
        const float2 *rp = plane + (long)(row0 + row) * CN;
#pragma unroll
        for (int n1 = 0; n1 < N1; n1++) v[n1] = row < nr ? __ldg(rp + N2 * n1 + n2) : make_float2(0.f, 0.f);
        reg_fft<float, N1, 2 * N2>(v, -1, tw);
#pragma unroll
        for (int k1 = 1; k1 < N1; k1++) v[k1] = cmul<float>(v[k1], tw1[k1 * N2 + n2]);
#pragma unroll
        for (int k1 = 0; k1 < N1; k1++) buf[row * P + n2 * Q + k1] = v[k1];
      }
    }
    __syncthreads();
    if (CL > 1 && b == 0) cluster_wait();  // every CTA of the cluster has started: peers' H may be written
#pragma unroll
    for (int q = 0; q < BX2; q++) {
      const int t = q * kXYThreads + threadIdx.x;
      if (PX2 % kXYThreads == 0 || t < PX2) {
        const int ka = t % NI, row = t / NI;
        const bool has_b = ka != 0 || N1 % 2 == 0;
        const int kb = ka == 0 ? (N1 % 2 == 0 ? N1 / 2 : 0) : N1 - ka;
        float2 a[N2], bb[N2];
#pragma unroll
        for (int n2 = 0; n2 < N2; n2++) {
          a[n2] = buf[row * P + n2 * Q + ka];
          bb[n2] = buf[row * P + n2 * Q + kb];
        }
        reg_fft<float, N2, 2 * N1>(a, -1, tw);
        if (has_b) reg_fft<float, N2, 2 * N1>(bb, -1, tw);
        if (row < nr) {
          const int grow = row0 + row;
#pragma unroll
          for (int k2 = 0; k2 < N2; k2++) {
            {
              const int k = ka + N1 * k2;
              const float2 A = a[k2];
              const float2 Bc = ka == 0 ? a[(N2 - k2) % N2] : bb[N2 - 1 - k2];
              const float2 B = make_float2(Bc.x, -Bc.y);
              const float2 E = make_float2((A.x + B.x) * 0.5f, (A.y + B.y) * 0.5f);
              const float2 O = make_float2((A.y - B.y) * 0.5f, -(A.x - B.x) * 0.5f);
              const float2 X = cadd<float>(E, cmul<float>(tw[k], O));
              put(grow, k, make_float2(X.x * prescale, X.y * prescale));
            }
            if (has_b) {
              const int k = kb + N1 * k2;
              const float2 A = bb[k2];
              const float2 Bc = ka == 0 ? bb[N2 - 1 - k2] : a[N2 - 1 - k2];
              const float2 B = make_float2(Bc.x, -Bc.y);
              const float2 E = make_float2((A.x + B.x) * 0.5f, (A.y + B.y) * 0.5f);
              const float2 O = make_float2((A.y - B.y) * 0.5f, -(A.x - B.x) * 0.5f);
              const float2 X = cadd<float>(E, cmul<float>(tw[k], O));
              put(grow, k, make_float2(X.x * prescale, X.y * prescale));
            }
          }
          if (ka == 0) {
            const float2 A = a[0];
            put(grow, M, make_float2((A.x - A.y) * prescale, 0.f));
          }
        }
      }
    }
    __syncthreads();  // buf is rewritten by the next batch
  }
  if constexpr (CL > 1) {
    cluster_arrive();  // this CTA's stores into the cluster's H are done ...
    cluster_wait();    // ... and so are every peer's
  }

  // ---- y pass over this CTA's columns [c0, c0 + ncols)
  const int c0 = rank * CW;
  const int ncols = min(CW, CN - c0);
  constexpr int PY = W * Y2, PY2 = W * Y1;
  constexpr int BY1 = (PY + kXYThreads - 1) / kXYThreads, BY2 = (PY2 + kXYThreads - 1) / kXYThreads;
#pragma unroll 1
  for (int cb = 0; cb < ncols; cb += W) {
    const int nc = min(W, ncols - cb);
#pragma unroll
    for (int q = 0; q < BY1; q++) {
      const int t = q * kXYThreads + threadIdx.x;
      if (PY % kXYThreads == 0 || t < PY) {
        const int c = t % W, n2 = t / W;
        float2 v[Y1];
#pragma unroll
        for (int n1 = 0; n1 < Y1; n1++) v[n1] = c < nc ? H[(Y2 * n1 + n2) * HP + cb + c] : make_float2(0.f, 0.f);
        reg_fft<float, Y1, Y2>(v, -1, ty);
#pragma unroll
        for (int k1 = 1; k1 < Y1; k1++) v[k1] = cmul<float>(v[k1], tw_at<float>(ty, n2 * k1, -1));
#pragma unroll
        for (int k1 = 0; k1 < Y1; k1++) buf[(k1 * Y2 + n2) * W + c] = v[k1];
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < BY2; q++) {
      const int t = q * kXYThreads + threadIdx.x;
      if (PY2 % kXYThreads == 0 || t < PY2) {
        const int c = t % W, k1 = t / W;
        float2 u[Y2];
#pragma unroll
        for (int n2 = 0; n2 < Y2; n2++) u[n2] = buf[(k1 * Y2 + n2) * W + c];
        reg_fft<float, Y2, Y1>(u, -1, ty);
        if (c < nc) {
          float2 *op = plane + c0 + cb + c;
#pragma unroll
          for (int k2 = 0; k2 < Y2; k2++) op[(long)(k1 + Y1 * k2) * CN] = u[k2];
        }
      }
    }
    __syncthreads();  // buf is rewritten by the next batch
  }
}

// ---------------------------------------------------------------------------
// inverse: y columns of this CTA's own columns into H, then x rows C2R from
// the cluster's H to global memory (postscale, optional addend, epilogue)
// ---------------------------------------------------------------------------
template <int M, int NY, int CL>
__global__ void __launch_bounds__(kXYThreads, 1) k_yx_c2r(const __grid_constant__ CubeSet cs,
                                                          const __grid_constant__ CubeSet addend,
                                                          const float2 *__restrict__ twx,
                                                          const float2 *__restrict__ twy, float postscale, int epi)
{
  using G = XYGeom<M, NY, CL>;
  constexpr int CN = G::CN, CW = G::CW, HP = G::HP, N1 = G::N1, N2 = G::N2, P = G::P, Q = G::Q;
  constexpr int RB = G::RB, Y1 = G::Y1, Y2 = G::Y2, W = G::W;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *H = (float2 *)smem_raw;
  float2 *buf = H + G::HSZ;
  float2 *tw = buf + G::XSZ;
  float2 *tw1 = tw + 2 * M;
  float2 *ty = tw1 + M;
  const unsigned rank = CL > 1 ? cluster_rank() : 0;
  float2 *plane = (float2 *)cs.ptr[blockIdx.z] + (long)blockIdx.y * CN * NY;
  for (int t = threadIdx.x; t < 2 * M; t += kXYThreads) tw[t] = twx[t];
  for (int t = threadIdx.x; t < N1 * N2; t += kXYThreads) tw1[t] = twx[2 * (t % N2) * (t / N2)];
  for (int t = threadIdx.x; t < NY; t += kXYThreads) ty[t] = twy[t];
  unsigned hb[CL];
#pragma unroll
  for (int r = 0; r < CL; r++) hb[r] = CL > 1 ? cluster_map(smem_u32(H), r) : smem_u32(H);
  __syncthreads();

  // ---- y pass over this CTA's columns, global -> H
  const int c0 = rank * CW;
  const int ncols = min(CW, CN - c0);
  constexpr int PY = W * Y2, PY2 = W * Y1;
  constexpr int BY1 = (PY + kXYThreads - 1) / kXYThreads, BY2 = (PY2 + kXYThreads - 1) / kXYThreads;
#pragma unroll 1
  for (int cb = 0; cb < ncols; cb += W) {
    const int nc = min(W, ncols - cb);
#pragma unroll
    for (int q = 0; q < BY1; q++) {
      const int t = q * kXYThreads + threadIdx.x;
      if (PY % kXYThreads == 0 || t < PY) {
        const int c = t % W, n2 = t / W;
        float2 v[Y1];
        const float2 *ip = plane + c0 + cb + c;
#pragma unroll
        for (int n1 = 0; n1 < Y1; n1++) v[n1] = c < nc ? __ldg(ip + (long)(Y2 * n1 + n2) * CN) : make_float2(0.f, 0.f);
        reg_fft<float, Y1, Y2>(v, +1, ty);
#pragma unroll
        for (int k1 = 1; k1 < Y1; k1++) v[k1] = cmul<float>(v[k1], tw_at<float>(ty, n2 * k1, +1));
#pragma unroll
        for (int k1 = 0; k1 < Y1; k1++) buf[(k1 * Y2 + n2) * W + c] = v[k1];
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < BY2; q++) {
      const int t = q * kXYThreads + threadIdx.x;
      if (PY2 % kXYThreads == 0 || t < PY2) {
        const int c = t % W, k1 = t / W;
        float2 u[Y2];
#pragma unroll
        for (int n2 = 0; n2 < Y2; n2++) u[n2] = buf[(k1 * Y2 + n2) * W + c];
        reg_fft<float, Y2, Y1>(u, +1, ty);
        if (c < nc) {
#pragma unroll
          for (int k2 = 0; k2 < Y2; k2++) H[(k1 + Y1 * k2) * HP + cb + c] = u[k2];
        }
      }
    }
    __syncthreads();
  }
  if constexpr (CL > 1) {
    cluster_arrive();  // this CTA's H is complete (and every CTA has started) ...
    cluster_wait();    // ... and so is every peer's
  }

  // ---- x pass: rows [rank*RPCT, (rank+1)*RPCT), C2R from the cluster's H
  auto get = [&](int grow, int k) -> float2 {
    const int owner = k / CW, col = k - owner * CW;
    if (CL == 1 || owner == (int)rank) return H[grow * HP + col];
    return dsm_load(pick(hb, owner) + (unsigned)((grow * HP + col) * sizeof(float2)));
  };
  constexpr int PX1 = RB * N2, PX2 = RB * N1;
  constexpr int BX1 = (PX1 + kXYThreads - 1) / kXYThreads, BX2 = (PX2 + kXYThreads - 1) / kXYThreads;
  const float2 *add = addend.ptr[blockIdx.z] ? (const float2 *)addend.ptr[blockIdx.z] + (long)blockIdx.y * CN * NY
                                             : nullptr;
#pragma unroll 1
  for (int b = 0; b < G::NBX; b++) {
    const int row0 = rank * G::RPCT + b * RB;
    const int nr = min(RB, (int)((rank + 1) * G::RPCT) - row0);
#pragma unroll
    for (int q = 0; q < BX1; q++) {
      const int t = q * kXYThreads + threadIdx.x;
      if (PX1 % kXYThreads == 0 || t < PX1) {
        const int n2 = t % N2, row = t / N2;
        const bool ok = row < nr;
        const int grow = row0 + row;
        float2 v[N1];
#pragma unroll
        for (int n1 = 0; n1 < N1; n1++) {
          const int k = N2 * n1 + n2;
          float2 Xk = ok ? get(grow, k) : make_float2(0.f, 0.f);
          float2 Xm = ok ? get(grow, M - k) : make_float2(0.f, 0.f);
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
    if (CL > 1 && b == G::NBX - 1) cluster_arrive();  // the last read of a peer's H is done
    __syncthreads();
#pragma unroll
    for (int q = 0; q < BX2; q++) {
      const int t = q * kXYThreads + threadIdx.x;
      if (PX2 % kXYThreads == 0 || t < PX2) {
        const int k1 = t % N1, row = t / N1;
        float2 u[N2];
#pragma unroll
        for (int n2 = 0; n2 < N2; n2++) u[n2] = buf[row * P + n2 * Q + k1];
        reg_fft<float, N2, 2 * N1>(u, +1, tw);
        if (row < nr) {
          float2 *op = plane + (long)(row0 + row) * CN;
          const float2 *ap = add ? add + (long)(row0 + row) * CN : nullptr;
#pragma unroll
          for (int k2 = 0; k2 < N2; k2++) {
            const int e = k1 + N1 * k2;
            float2 z = make_float2(u[k2].x * postscale, u[k2].y * postscale);
            if (ap) {
              const float2 s = ap[e];
              z.x += s.x;
              z.y += s.y;
            }
            op[e] = make_float2(epilogue<float>(z.x, epi), epilogue<float>(z.y, epi));
          }
          if (k1 == 0) {
            float2 z = make_float2(0.f, 0.f);
            if (ap) {
              const float2 s = ap[M];
              z.x += s.x;
              z.y += s.y;
            }
            op[M] = make_float2(epilogue<float>(z.x, epi), epilogue<float>(z.y, epi));
          }
        }
      }
    }
    __syncthreads();
  }
  if constexpr (CL > 1) cluster_wait();  // no peer reads this CTA's H any more
}

}  // namespace cg
