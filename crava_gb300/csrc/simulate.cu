// Posterior stochastic simulation, Crava::simulate (src/crava.cpp:1551-1734).
//
// The reference, per realisation: draws three complex white-noise cubes
// (FFTGrid::fillInComplexNoise, src/fftgrid.cpp:1191-1241), Cholesky-factors
// the 3x3 posterior covariance of every bin (lib_matrCholCpx) and multiplies
// (lib_matrProdCholVec), zero noise where the factorisation fails
// (src/crava.cpp:1644-1651), then three C2R transforms (PARAMETER) and adds the
// posterior mean.
//
// Here the factor is computed once (it does not change between
// realisations) and stored as nine float planes; each realisation is one
// pass that forms z = L xi for every bin, with xi either injected (three
// complex cubes, for parity with the reference's generator) or drawn in the
// kernel from a counter-based Philox4x32-10 stream keyed by (seed,
// realisation) and indexed by the bin, with the same Hermitian structure the
// reference imposes on the x=0 plane and, through its flat-index parity test,
// on half of the last x plane.  The C2R transforms then run batched with the
// posterior-mean add fused into their last pass.
#include <cstring>

#include "common.cuh"
#include "fft.cuh"
#include "trace.cuh"

namespace cg {

constexpr double kTolChol = 1e-20;

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): 10 rounds of the 4x32 bijection with the published
// multipliers and Weyl key increments.
// ---------------------------------------------------------------------------
struct U4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1)
{
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    U4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// four standard normals from one Philox block (Box-Muller on (0,1) uniforms).  The
// radius and angle use the hardware approximations (__logf, rsqrtf, __sincosf:
// errors near 1e-6, immaterial to the distribution); the accurate library
// functions made this kernel issue-bound on their range reductions.
__device__ __forceinline__ void normals4(U4 r, float *g)
{
  const float s = 2.3283064365386963e-10f;  // 2^-32
  const float u0 = ((float)r.x + 0.5f) * s, u1 = ((float)r.y + 0.5f) * s;
  const float u2 = ((float)r.z + 0.5f) * s, u3 = ((float)r.w + 0.5f) * s;
  // u rounds to 1.0f for draws within 128 of 2^32 (t = -0): radius 0 there, as sqrt would give
  const float t0 = -2.0f * __logf(u0), t1 = -2.0f * __logf(u2);
  const float r0 = t0 > 0.0f ? t0 * rsqrtf(t0) : 0.0f, r1 = t1 > 0.0f ? t1 * rsqrtf(t1) : 0.0f;
  const float two_pi = 6.283185307179586f;
  float s0, c0, s1, c1;
  __sincosf(two_pi * u1, &s0, &c0);
  __sincosf(two_pi * u3, &s1, &c1);
  g[0] = r0 * c0;
  g[1] = r0 * s0;
  g[2] = r1 * c1;
  g[3] = r1 * s1;
}

// six normals (three complex values, one per parameter) for bin b
__device__ __forceinline__ void bin_normals(uint64_t seed, int realisation, long b, float *g6)
{
  float g[8];
  U4 c0 = {(uint32_t)b, (uint32_t)((uint64_t)b >> 32), (uint32_t)realisation, 0u};
  U4 c1 = {(uint32_t)b, (uint32_t)((uint64_t)b >> 32), (uint32_t)realisation, 1u};
  normals4(philox4x32_10(c0, (uint32_t)seed, (uint32_t)(seed >> 32)), g);
  normals4(philox4x32_10(c1, (uint32_t)seed, (uint32_t)(seed >> 32)), g + 4);
#pragma unroll
  for (int t = 0; t < 6; t++) g6[t] = g[t];
}

// Structure of FFTGrid::fillInComplexNoise at flat bin index i: bins of the
// x=0 plane (and of the last x plane where the flat index is odd) are real
// when self-conjugate and the conjugate of their partner's draw when the
// partner comes first in the flat order; every other bin is an independent
// complex draw of variance 1.  The structure does not depend on the
// realisation, so it is worked out once per bin: *src is the bin whose draw
// is used, the return value the kind (0 complex draw, 1 real draw, 2
// conjugate of the partner's draw).
__device__ __forceinline__ int noise_kind(long i, int cnxp, int nyp, int nzp, long *src)
{
  const long xshift = i % cnxp;
  *src = i;
  if (xshift == 0 || (xshift == cnxp - 1 && (i % 2) == 1)) {
    const long jk = (i - xshift) / cnxp;
    const long j = jk % nyp, k = jk / nyp;
    const long jcc = j == 0 ? 0 : nyp - j;
    const long kcc = k == 0 ? 0 : nzp - k;
    const long jkcc = jcc + kcc * nyp;
    if (jkcc == jk) return 1;
    if (jkcc < jk) { *src = jkcc * cnxp + xshift; return 2; }
  }
  return 0;
}

// complex noise of the three parameters for one realisation, given the bin's
// noise_kind
__device__ __forceinline__ void noise3_from(uint64_t seed, int realisation, long src, int kind, float2 *s)
{
  const float sd = 0.70710678118654752f;
  float g[6];
  bin_normals(seed, realisation, src, g);
#pragma unroll
  for (int p = 0; p < 3; p++) {
    if (kind == 1) s[p] = make_float2(g[2 * p], 0.0f);
    else if (kind == 2) s[p] = make_float2(sd * g[2 * p], -sd * g[2 * p + 1]);
    else s[p] = make_float2(sd * g[2 * p], sd * g[2 * p + 1]);
  }
}

// lib_matrCholCpx on the 3x3 posterior covariance (reference semantics)
__device__ __forceinline__ bool chol3_ref(float2 *L /* packed lower, 6 */)
{
  const float factor = L[0].x;
  if (!(factor > 0.0f)) return false;
#pragma unroll
  for (int t = 0; t < 6; t++) { L[t].x /= factor; L[t].y /= factor; }
  const int tr[3][3] = {{0, -1, -1}, {1, 2, -1}, {3, 4, 5}};
#pragma unroll
  for (int i = 0; i < 3; i++) {
    if (L[tr[i][i]].x <= (float)kTolChol) return false;
#pragma unroll
    for (int j = 0; j < i; j++) {
      float lr = 0, li = 0;
#pragma unroll
      for (int k = 0; k < j; k++) {
        lr += (L[tr[i][k]].x * L[tr[j][k]].x) + (L[tr[i][k]].y * L[tr[j][k]].y);
        li += -(L[tr[i][k]].x * L[tr[j][k]].y) + (L[tr[i][k]].y * L[tr[j][k]].x);
      }
      const float2 ljj = L[tr[j][j]], lij = L[tr[i][j]];
      const float help = ljj.x * ljj.x + ljj.y * ljj.y;
      L[tr[i][j]] = make_float2(((lij.x - lr) * ljj.x + (lij.y - li) * ljj.y) / help,
                                ((lij.y - li) * ljj.x - (lij.x - lr) * ljj.y) / help);
    }
    float lr = 0;
#pragma unroll
    for (int k = 0; k < i; k++) lr += (L[tr[i][k]].x * L[tr[i][k]].x) + (L[tr[i][k]].y * L[tr[i][k]].y);
    lr = L[tr[i][i]].x - lr;
    if (lr <= (float)kTolChol) return false;
    L[tr[i][i]] = make_float2(sqrtf(lr), 0.0f);
  }
  const float sf = sqrtf(factor);
#pragma unroll
  for (int t = 0; t < 6; t++) { L[t].x *= sf; L[t].y *= sf; }
  return true;
}

struct CholArgs {
  const float2 *cov[6];  // 00 11 22 01 02 12
  float *L;              // 9 planes of csize floats: L00 L11 L22 L10r L10i L20r L20i L21r L21i
  long csize;
  int *nfail;
};

__global__ void k_post_chol(CholArgs a)
{
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.csize) return;
  float2 P[6];
  P[0] = a.cov[0][b];                                       // (0,0)
  const float2 c01 = a.cov[3][b];
  P[1] = make_float2(c01.x, -c01.y);                        // (1,0) = conj(0,1)
  P[2] = a.cov[1][b];                                       // (1,1)
  const float2 c02 = a.cov[4][b];
  P[3] = make_float2(c02.x, -c02.y);                        // (2,0)
  const float2 c12 = a.cov[5][b];
  P[4] = make_float2(c12.x, -c12.y);                        // (2,1)
  P[5] = a.cov[2][b];                                       // (2,2)
  float v[9];
  if (chol3_ref(P)) {
    v[0] = P[0].x; v[1] = P[2].x; v[2] = P[5].x;
    v[3] = P[1].x; v[4] = P[1].y; v[5] = P[3].x; v[6] = P[3].y; v[7] = P[4].x; v[8] = P[4].y;
  } else {
    // a failed factorisation gives zero noise for this bin (src/crava.cpp:1644-1651)
#pragma unroll
    for (int t = 0; t < 9; t++) v[t] = 0.0f;
    if (a.nfail) atomicAdd(a.nfail, 1);
  }
#pragma unroll
  for (int t = 0; t < 9; t++) a.L[(long)t * a.csize + b] = v[t];
}

struct ApplyArgs {
  const float *L;
  const float2 *noise[3];   // injected noise (nullptr: generate)
  float2 *out[kMaxBatch];   // 3 per realisation
  int nreal;
  int real0;                // index of the first realisation of this launch
  uint64_t seed;
  long csize;
  int cnxp, nyp, nzp;
};

// z = L xi for every bin of `nreal` realisations (lib_matrProdCholVec order)
__global__ void k_sim_apply(ApplyArgs a)
{
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.csize) return;
  float l[9];
#pragma unroll
  for (int t = 0; t < 9; t++) l[t] = a.L[(long)t * a.csize + b];
  const float2 L00 = make_float2(l[0], 0), L11 = make_float2(l[1], 0), L22 = make_float2(l[2], 0);
  const float2 L10 = make_float2(l[3], l[4]), L20 = make_float2(l[5], l[6]), L21 = make_float2(l[7], l[8]);
  long src = b;
  const int kind = a.noise[0] ? 0 : noise_kind(b, a.cnxp, a.nyp, a.nzp, &src);
  for (int r = 0; r < a.nreal; r++) {
    float2 s[3];
    if (a.noise[0]) {
#pragma unroll
      for (int p = 0; p < 3; p++) s[p] = a.noise[p][b];
    } else {
      noise3_from(a.seed, a.real0 + r, src, kind, s);
    }
    float2 o[3];
    o[0] = cmul<float>(L00, s[0]);
    o[1] = cadd<float>(cmul<float>(L10, s[0]), cmul<float>(L11, s[1]));
    o[2] = cadd<float>(cadd<float>(cmul<float>(L20, s[0]), cmul<float>(L21, s[1])), cmul<float>(L22, s[2]));
#pragma unroll
    for (int p = 0; p < 3; p++) a.out[3 * r + p][b] = o[p];
  }
}

}  // namespace cg

using namespace cg;

extern "C" int cg_posterior_cholesky(float *const *post_cov, float *chol, int nxp, int nyp, int nzp, int *nfail_dev,
                                     void *stream)
{
  if (!post_cov || !chol || nxp < 1 || nyp < 1 || nzp < 1) { set_error("cg_posterior_cholesky: bad argument"); return CG_ERR_ARG; }
  CholArgs a;
  for (int t = 0; t < 6; t++) {
    if (!post_cov[t]) { set_error("null post_cov[%d]", t); return CG_ERR_ARG; }
    a.cov[t] = (const float2 *)post_cov[t];
  }
  a.L = chol;
  a.csize = (long)(nxp / 2 + 1) * nyp * nzp;
  a.nfail = nfail_dev;
  TraceScope ts("k_post_chol", (cudaStream_t)stream, 48.0 * a.csize + 36.0 * a.csize);
  k_post_chol<<<ceil_div(a.csize, 256), 256, 0, (cudaStream_t)stream>>>(a);
  CG_CHECK_LAUNCH("k_post_chol");
  return CG_OK;
}

extern "C" int cg_simulate_fields(const float *chol, const float *const *noise, float *const *fields, int nreal,
                                  int real0, uint64_t seed, int nxp, int nyp, int nzp, const float *const *post_mean,
                                  void *stream)
{
  if (!chol || !fields || nreal < 1 || nxp < 1 || nyp < 1 || nzp < 1) { set_error("cg_simulate_fields: bad argument"); return CG_ERR_ARG; }
  if (noise && nreal != 1) { set_error("injected noise supports one realisation per call"); return CG_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  const long csize = (long)(nxp / 2 + 1) * nyp * nzp;
  const int per_launch = kMaxBatch / 3;  // realisations per apply launch (3 cubes each)
  for (int r0 = 0; r0 < nreal; r0 += per_launch) {
    const int nr = nreal - r0 < per_launch ? nreal - r0 : per_launch;
    ApplyArgs a;
    memset(&a, 0, sizeof(a));
    a.L = chol;
    for (int p = 0; p < 3; p++) a.noise[p] = noise ? (const float2 *)noise[p] : nullptr;
    for (int t = 0; t < 3 * nr; t++) {
      if (!fields[3 * r0 + t]) { set_error("null field %d", 3 * r0 + t); return CG_ERR_ARG; }
      a.out[t] = (float2 *)fields[3 * r0 + t];
    }
    a.nreal = nr;
    a.real0 = real0 + r0;
    a.seed = seed;
    a.csize = csize;
    a.cnxp = nxp / 2 + 1;
    a.nyp = nyp;
    a.nzp = nzp;
    {
      TraceScope ts("k_sim_apply", st, 36.0 * csize + (noise ? 24.0 * csize : 0.0) + 24.0 * csize * nr);
      k_sim_apply<<<ceil_div(csize, 256), 256, 0, st>>>(a);
      CG_CHECK_LAUNCH("k_sim_apply");
    }
    // C2R of the 3*nr noise fields (PARAMETER scaling), posterior mean added in the last pass
    const void *add[kMaxBatch];
    for (int t = 0; t < 3 * nr; t++) add[t] = post_mean ? post_mean[t % 3] : nullptr;
    int rc = fft3d_c2r_add<float>((void *const *)(fields + 3 * r0), post_mean ? add : nullptr, 3 * nr, nxp, nyp,
                                  nzp, CG_PARAMETER, st);
    if (rc) return rc;
  }
  return CG_OK;
}
