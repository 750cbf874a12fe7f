// Non-constant simbox thickness: per-trace scaling of the seismic data by the
// stretched local wavelet, and the interpolation of dead traces.
//
// Crava::divideDataByScaleWavelet (src/crava.cpp:678-804) takes every padded
// trace of every angle cube, tapers the z padding (k > nz, getDistToBoundary),
// transforms it (R2C of length nzp), multiplies the spectrum inside the band
// lowCut < f_k < highCut (f_k = k * nz*1000/(relThick*lz*nzp)) by the factor
// of computeAdjustmentFactor (:807-903) and zeroes it outside, transforms back
// (C2R) and scales by 1/nzp.  The factor compares the inversion of one trace
// with the local wavelet (the global wavelet shifted by the local time shift,
// scaled by the local gain and stretched by the relative thickness: getCAmp(k,
// sf) interpolates the spectrum at k/sf and multiplies by 1/sf) with the one
// the global wavelet gives.
// multiplyDataByScaleWaveletAndWriteToFile (:906-968) is the inverse step on
// output cubes: every simbox trace times the conjugate stretched local wavelet
// spectrum.  FFTGrid::interpolateSeismic (src/fftgrid.cpp:2576-2738) then
// replaces traces whose energy is at or below a threshold by the mean of their
// good neighbours and refills the padding from the edge traces.
//
// GB300 layout: the 1D real transforms along z of two neighbouring x traces
// are one complex transform of the cube's complex view (x pair c = traces 2c
// and 2c + 1), so the batched z-column kernels of the 3D transform do the
// transforms.  One pointwise kernel splits each bin pair (k, nzp - k) into the
// two real spectra (X = (Z_k + conj Z_{nzp-k})/2, Y = (Z_k - conj Z_{nzp-k})/2i),
// applies each trace's factor, drops the imaginary part of the DC and Nyquist
// products as the C2R does, and recombines.  The factor is computed per
// (trace, k) from per-angle tables (W, the normalised third-difference
// spectrum E3, tau2; built on the host by cg_scale_wavelet_tables) and per-
// trace parameters; the local wavelet's shift is exp(-2 pi i iShift m / nzp)
// evaluated with an exact float split of iShift/nzp.  The local wavelet's
// normalised E3 is the phase-rotated global one: the gain cancels in the
// normalisation and the phase has unit modulus.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "fft.cuh"
#include "trace.cuh"

namespace cg {
namespace {

struct __align__(16) SwTrace {
  float sf;    // stretch = relative thickness
  float gain;  // local gain
  float ahi;   // iShift / nzp = ahi + alo, ahi with at most 11 significant bits
  float alo;
  float2 step; // exp(-2 pi i iShift / nzp): the shift phase of one bin
  float2 pad;
};

// FFTGrid::getDistToBoundary (src/fftgrid.cpp:1353-1389)
__host__ __device__ inline float dist_to_boundary(int i, int n, int np)
{
  if (i >= np) return kRMissing;
  if (i < n) return 0.0f;
  const float taper = (float)((double)(n < np - n ? n : np - n) / 2.1);
  const int below = np - i, above = i - (n - 1);
  return above < below ? (float)above / taper : (float)below / taper;
}

// FFTGrid::getFillNumber (src/fftgrid.cpp:1298-1336), -1 for IMISSING
__host__ __device__ inline int fill_number(int i, int n, int np)
{
  if (i >= np) return -1;
  if (i < n) return i;
  const int below = np - i - 1, above = i - n + 1;
  if (above < below) return (n - above) > n / 2 ? (n - above) : n / 2;
  return below < n / 2 ? below : n / 2;
}

// the wavelet-surface index of a padded trace (src/crava.cpp:710-730)
__device__ inline int mirror_index(int i, int n, int np)
{
  int ii = i;
  if (ii > 3 * n - 1) ii = 0;
  if (ii > (np + n) / 2) ii = np - ii;
  if (ii >= n) ii = 2 * n - ii - 1;
  return ii;
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Per trace (and angle): stretch, gain, shift phase split; per trace: the band
// [klo, khi] of bins with lowCut < deltaF*k < highCut (double, as the reference).
__global__ void k_sw_params(SwTrace *__restrict__ tp, int2 *__restrict__ kb, const float *__restrict__ rel_thick,
                            const float *__restrict__ shift, const float *__restrict__ gain, int ncubes, int nx,
                            int ny, int nz, int nxp, int nyp, int nzp, float dz, float lz, float low_cut,
                            float high_cut, int mirror)
{
  const long ntr = (long)nxp * nyp;
  const long total = ntr * ncubes;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int l = (int)(idx / ntr);
    const long c = idx - (long)l * ntr;
    const int x = (int)(c % nxp), j = (int)(c / nxp);
    const float rt = rel_thick[c];
    const bool valid = rt > 0.0f && isfinite(rt);
    if (l == 0 && kb) {
      const int half = nzp / 2;
      int klo = 1, khi = 0;
      if (valid) {
        const double deltaF = (double)nz * 1000.0 / ((double)rt * (double)lz * (double)nzp);
        const double lo = (double)low_cut, hi = (double)high_cut;
        double f0 = floor(lo / deltaF);
        klo = f0 < 0.0 ? 0 : (f0 > half + 1.0 ? half + 1 : (int)f0);
        while (klo <= half && !(deltaF * klo > lo)) klo++;
        while (klo > 0 && deltaF * (klo - 1) > lo) klo--;
        double f1 = ceil(hi / deltaF);
        khi = f1 < 0.0 ? -1 : (f1 > half ? half : (int)f1);
        while (khi >= 0 && !(deltaF * khi < hi)) khi--;
        while (khi < half && deltaF * (khi + 1) < hi) khi++;
      }
      kb[c] = make_int2(klo, khi);
    }
    int ii = x, jj = j;
    if (mirror) {
      ii = mirror_index(x, nx, nxp);
      jj = mirror_index(j, ny, nyp);
    }
    const bool in = ii >= 0 && ii < nx && jj >= 0 && jj < ny;
    const long sidx = ((long)l * ny + jj) * nx + ii;
    const float ts = (shift && in) ? shift[sidx] : 0.0f;
    const float g = (gain && in) ? gain[sidx] : 1.0f;
    const float ishift = ts / dz;
    const double a = (double)ishift / (double)nzp;
    int e = 0;
    const double fr = frexp(a, &e);
    const double hi = ldexp(rint(ldexp(fr, 10)), e - 10);
    SwTrace t;
    t.sf = valid ? rt : 1.0f;
    t.gain = g;
    t.ahi = (float)hi;
    t.alo = (float)(a - hi);
    float sn, cs;
    sincospif(2.0f * ((t.ahi - rintf(t.ahi)) + t.alo), &sn, &cs);
    t.step = make_float2(cs, -sn);
    t.pad = make_float2(0.0f, 0.0f);
    tp[idx] = t;
  }
}

// exp(-2 pi i (ahi + alo) m): ahi*m is exact in float, its integer part drops out
__device__ __forceinline__ float2 shift_phasor(const SwTrace &t, int m)
{
  float h = t.ahi * (float)m;
  h -= rintf(h);
  const float turns = h + t.alo * (float)m;
  float s, c;
  sincospif(2.0f * turns, &s, &c);
  return make_float2(c, -s);
}

// local wavelet spectrum at bin m after the C2R/R2C round trip of the
// reference (imaginary part of DC and Nyquist dropped)
__device__ __forceinline__ float2 wl_val(const float2 *W, int m, float2 p, float gain, int nzp)
{
  float2 v = cmulf(make_float2(gain * p.x, gain * p.y), W[m]);
  if (m == 0 || 2 * m == nzp) v.y = 0.0f;
  return v;
}

// normalised third-difference spectrum of the local wavelet at bin m; the
// floats past nzp of the last bin are RMISSING (multiplyRAmpByConstant)
__device__ __forceinline__ float2 e3_val(const float2 *E, int m, float2 p, int nzp)
{
  float2 v = cmulf(p, E[m]);
  if (m == nzp / 2) {
    v.y = kRMissing;
    if ((nzp & 1) == 0) v.x = kRMissing;
  }
  return v;
}

template <bool SHIFT>
__device__ __forceinline__ float2 phasor_at(const SwTrace &t, int m)
{
  if constexpr (SHIFT) return shift_phasor(t, m);
  return make_float2(1.0f, 0.0f);
}

// computeAdjustmentFactor at bin k < nzp/2 + 1 for one trace: the
// reference's (wLoc/(tau2 wLoc2Adj + sigma2Loc)) / (wGlob2Adj/(tau2 wGlob2 +
// sigma2Glob)) as one quotient
template <bool SHIFT>
__device__ float2 adjustment(const float *tab, int nzp, const SwTrace &t, int k, float inv_wn2)
{
  const int cnzp = nzp / 2 + 1;
  const float2 *W = (const float2 *)tab;
  const float2 *E = W + cnzp;
  const float *tau = (const float *)(E + cnzp);
  const float modW = tau[cnzp + 1], ev = tau[cnzp + 2], wnc = tau[cnzp + 3];
  float2 wLoc = make_float2(0.0f, 0.0f), eLoc = make_float2(0.0f, 0.0f);
  const float omega = (float)k / t.sf;
  if (omega < (float)cnzp) {
    const int omL = (int)floorf(omega);
    const int omU = omL + 1 < cnzp ? omL + 1 : omL;
    const float d = omega - (float)omL, d1 = 1.0f - d;
    const float2 pL = phasor_at<SHIFT>(t, omL);
    const float2 pU = (SHIFT && omU != omL) ? cmulf(pL, t.step) : pL;
    const float2 wa = wl_val(W, omL, pL, t.gain, nzp), wb = wl_val(W, omU, pU, t.gain, nzp);
    wLoc = make_float2(wa.x * d1 + wb.x * d, wa.y * d1 + wb.y * d);
    const float2 ea = e3_val(E, omL, pL, nzp), eb = e3_val(E, omU, pU, nzp);
    eLoc = make_float2(ea.x * d1 + eb.x * d, ea.y * d1 + eb.y * d);
    // getCAmp(k, sf) returns the interpolated value times 1/sf (src/wavelet.cpp:382-383)
    wLoc = make_float2(wLoc.x / t.sf, wLoc.y / t.sf);
    eLoc = make_float2(eLoc.x / t.sf, eLoc.y / t.sf);
  }
  const float wLoc2 = wLoc.x * wLoc.x + wLoc.y * wLoc.y;
  const float2 wG = W[k];
  const float wGlob2 = wG.x * wG.x + wG.y * wG.y;
  const float sLoc = wLoc2 * inv_wn2 + (eLoc.x * eLoc.x + eLoc.y * eLoc.y);
  const float2 pk = phasor_at<SHIFT>(t, k);
  const float2 gl = wl_val(W, k, pk, t.gain, nzp), eg = e3_val(E, k, pk, nzp);
  const float sGlob = (gl.x * gl.x + gl.y * gl.y) * inv_wn2 + (eg.x * eg.x + eg.y * eg.y);
  float s2L = ev * (wnc + (1.0f - wnc) * 0.5f * sLoc);
  const float s2G = ev * (wnc + (1.0f - wnc) * 0.5f * sGlob);
  const float tau2 = tau[k];
  const float tol = 0.05f;
  const float wG2A = wGlob2 < tol * modW ? 0.5f * (wGlob2 + tol * modW) : wGlob2;
  float wL2A = wLoc2 < tol * modW ? 0.5f * (wLoc2 + tol * modW) : wLoc2;
  if (wL2A < tol * wG2A) {
    wL2A = 0.5f * (wLoc2 + tol * wG2A);
    s2L *= wL2A / wLoc2;
  }
  const float q = tau2 * wL2A + s2L;
  const float f = (tau2 * wGlob2 + s2G) / (wG2A * q);
  return make_float2(wLoc.x * f, wLoc.y * f);
}

// the stretched local wavelet spectrum at bin k (getCAmp(k, sf) of the local wavelet)
template <bool SHIFT>
__device__ float2 local_wavelet(const float *tab, int nzp, const SwTrace &t, int k)
{
  const int cnzp = nzp / 2 + 1;
  const float2 *W = (const float2 *)tab;
  const float omega = (float)k / t.sf;
  if (!(omega < (float)cnzp)) return make_float2(0.0f, 0.0f);
  const int omL = (int)floorf(omega);
  const int omU = omL + 1 < cnzp ? omL + 1 : omL;
  const float d = omega - (float)omL, d1 = 1.0f - d;
  const float2 pL = phasor_at<SHIFT>(t, omL);
  const float2 pU = (SHIFT && omU != omL) ? cmulf(pL, t.step) : pL;
  const float2 wa = wl_val(W, omL, pL, t.gain, nzp);
  const float2 wb = wl_val(W, omU, pU, t.gain, nzp);
  // getCAmp(k, sf) returns the interpolated value times 1/sf (src/wavelet.cpp:382-383)
  return make_float2((wa.x * d1 + wb.x * d) / t.sf, (wa.y * d1 + wb.y * d) / t.sf);
}

enum { kSwDivide = 0, kSwMultiply = 1 };

template <int MODE, bool SHIFT>
__device__ __forceinline__ float2 trace_factor(const float *tab, const SwTrace *tp, const int2 *kb, int l, int x, int j,
                                               int k, int nx, int ny, int nxp, int nyp, int nzp, float inv_wn2)
{
  if (x >= nxp) return make_float2(0.0f, 0.0f);  // slack column of the in-place layout
  const long tix = (long)j * nxp + x;
  if constexpr (MODE == kSwDivide) {
    const int2 b = kb[tix];
    if (k < b.x || k > b.y) return make_float2(0.0f, 0.0f);
    return adjustment<SHIFT>(tab, nzp, tp[(long)l * nxp * nyp + tix], k, inv_wn2);
  } else {
    if (x >= nx || j >= ny) return make_float2(1.0f, 0.0f);
    const float2 v = local_wavelet<SHIFT>(tab, nzp, tp[(long)l * nxp * nyp + tix], k);
    return make_float2(v.x, -v.y);
  }
}

// One thread per (cube, bin pair k / nzp - k, y, x pair).
template <int MODE, bool SHIFT>
__global__ void __launch_bounds__(256) k_sw_spectral(const __grid_constant__ CubeSet cs, int ncubes, const float *__restrict__ tables,
                                                     int tstride, const SwTrace *__restrict__ tp,
                                                     const int2 *__restrict__ kb, int nx, int ny, int nxp, int nyp,
                                                     int nzp, float scale)
{
  const int cnxp = nxp / 2 + 1, cnzp = nzp / 2 + 1;
  const long plane = (long)cnxp * nyp;
  const long total = (long)ncubes * cnzp * plane;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int c = (int)(idx % cnxp);
    long r = idx / cnxp;
    const int j = (int)(r % nyp);
    r /= nyp;
    const int k = (int)(r % cnzp);
    const int l = (int)(r / cnzp);
    float2 *z = (float2 *)cs.ptr[l];
    const bool self = k == 0 || 2 * k == nzp;
    const long i1 = c + (long)cnxp * j + plane * k;
    const long i2 = self ? i1 : c + (long)cnxp * j + plane * (nzp - k);
    const float2 z1 = z[i1], z2 = z[i2];
    const float2 X = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
    const float2 Y = make_float2(0.5f * (z1.y + z2.y), -0.5f * (z1.x - z2.x));
    const float *tab = tables + (long)l * tstride;
    const float inv_wn2 = MODE == kSwDivide ? 1.0f / tab[5 * cnzp] : 0.0f;
    const float2 a0 = trace_factor<MODE, SHIFT>(tab, tp, kb, l, 2 * c, j, k, nx, ny, nxp, nyp, nzp, inv_wn2);
    const float2 a1 = trace_factor<MODE, SHIFT>(tab, tp, kb, l, 2 * c + 1, j, k, nx, ny, nxp, nyp, nzp, inv_wn2);
    float2 xp = cmulf(X, a0), yp = cmulf(Y, a1);
    xp.x *= scale; xp.y *= scale;
    yp.x *= scale; yp.y *= scale;
    if (self) {
      z[i1] = make_float2(xp.x, yp.x);  // the C2R keeps Re of the DC / Nyquist products
    } else {
      z[i1] = make_float2(xp.x - yp.y, xp.y + yp.x);
      z[i2] = make_float2(xp.x + yp.y, yp.x - xp.y);
    }
  }
}

// planes k >= k0: taper max(1 - dist^2, 0) (divideDataByScaleWavelet, src/crava.cpp:737-741)
// and zero slack columns; planes k < k0: slack columns only
__global__ void k_sw_taper(const __grid_constant__ CubeSet cs, int ncubes, int k0, int nz, int nxp, int nyp, int nzp)
{
  const int rnxp = 2 * (nxp / 2 + 1);
  const long rows = (long)(nzp - k0) * nyp;
  const long total = (long)ncubes * rows * rnxp;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int x = (int)(idx % rnxp);
    long r = idx / rnxp;
    const int l = (int)(r / rows);
    r -= (long)l * rows;
    const int k = k0 + (int)(r / nyp);
    float *b = (float *)cs.ptr[l] + ((long)k * nyp + (r % nyp)) * rnxp + x;
    if (x >= nxp) {
      *b = 0.0f;
    } else {
      const float d = dist_to_boundary(k, nz, nzp);
      const float t = 1.0f - __fmul_rn(d, d);
      *b = __fmul_rn(*b, t > 0.0f ? t : 0.0f);
    }
  }
}

__global__ void k_sw_slack(const __grid_constant__ CubeSet cs, int ncubes, int nplanes, int nxp, int nyp)
{
  const int rnxp = 2 * (nxp / 2 + 1), ns = rnxp - nxp;
  const long rows = (long)nplanes * nyp;
  const long total = (long)ncubes * rows * ns;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int s = (int)(idx % ns);
    const long r = idx / ns;
    const int l = (int)(r / rows);
    const long row = r - (long)l * rows;
    ((float *)cs.ptr[l])[row * rnxp + nxp + s] = 0.0f;
  }
}

// traces whose padded input is exactly zero: the reference's transforms keep
// them exactly zero, which the paired transform (rounding from the partner
// trace) would not; the energy test of interpolateSeismic depends on it
__global__ void k_sw_zero_flags(const __grid_constant__ CubeSet cs, int ncubes, int nxp, int nyp, int nzp, unsigned char *__restrict__ zf)
{
  const int rnxp = 2 * (nxp / 2 + 1);
  const long ntr = (long)nxp * nyp;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < ntr * ncubes; idx += (long)gridDim.x * blockDim.x) {
    const int l = (int)(idx / ntr);
    const long c = idx - (long)l * ntr;
    const float *b = (const float *)cs.ptr[l] + (c / nxp) * rnxp + (c % nxp);
    unsigned char zero = 1;
    for (int k = 0; k < nzp && zero; k++) zero = b[(long)k * nyp * rnxp] == 0.0f;
    zf[idx] = zero;
  }
}

__global__ void k_sw_zero_apply(const __grid_constant__ CubeSet cs, int ncubes, int nxp, int nyp, int nzp, const unsigned char *__restrict__ zf)
{
  const int rnxp = 2 * (nxp / 2 + 1);
  const long ntr = (long)nxp * nyp;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < ntr * ncubes; idx += (long)gridDim.x * blockDim.x) {
    if (!zf[idx]) continue;
    const int l = (int)(idx / ntr);
    const long c = idx - (long)l * ntr;
    float *b = (float *)cs.ptr[l] + (c / nxp) * rnxp + (c % nxp);
    for (int k = 0; k < nzp; k++) b[(long)k * nyp * rnxp] = 0.0f;
  }
}

// per-trace energy over the simbox (FFTGrid::interpolateSeismic, src/fftgrid.cpp:2587-2598):
// sequential float sum, no fused multiply-add; loads issued eight at a time
__global__ void k_trace_energy(const __grid_constant__ CubeSet cs, int ncubes, float *__restrict__ energy, int nx, int ny, int nz, int nxp,
                               int nyp)
{
  const int rnxp = 2 * (nxp / 2 + 1);
  const long n = (long)nx * ny;
  const long pstride = (long)nyp * rnxp;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n * ncubes; t += (long)gridDim.x * blockDim.x) {
    const int l = (int)(t / n);
    const long tt = t - (long)l * n;
    const float *b = (const float *)cs.ptr[l] + (tt / nx) * rnxp + (tt % nx);
    float e = 0.0f;
    int k = 0;
    for (; k + 8 <= nz; k += 8) {
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; u++) v[u] = __ldg(b + (long)(k + u) * pstride);
#pragma unroll
      for (int u = 0; u < 8; u++) e = __fadd_rn(e, __fmul_rn(v[u], v[u]));
    }
    for (; k < nz; k++) {
      const float v = __ldg(b + (long)k * pstride);
      e = __fadd_rn(e, __fmul_rn(v, v));
    }
    energy[t] = e;
  }
}

// FFTGrid::interpolateTrace (src/fftgrid.cpp:2668-2707) for one level of
// independent traces: ops[q] = (cube, trace, neighbour mask: 1 left, 2 right,
// 4 up, 8 down)
__global__ void k_interp_traces(const __grid_constant__ CubeSet cs, const int4 *__restrict__ ops, int nops, int nx, int nxp, int nyp, int nzp)
{
  const int rnxp = 2 * (nxp / 2 + 1);
  const long total = (long)nops * nzp;
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
    const int q = (int)(idx / nzp), k = (int)(idx % nzp);
    const int4 op = ops[q];
    float *buf = (float *)cs.ptr[op.x];
    const int i = op.y % nx, j = op.y / nx, m = op.z;
    const long base = (long)k * nyp * rnxp;
    float s = (m & 1) ? buf[base + (long)j * rnxp + i - 1] : 0.0f;
    if (m & 2) s = __fadd_rn(s, buf[base + (long)j * rnxp + i + 1]);
    if (m & 4) s = __fadd_rn(s, buf[base + (long)(j - 1) * rnxp + i]);
    if (m & 8) s = __fadd_rn(s, buf[base + (long)(j + 1) * rnxp + i]);
    buf[base + (long)j * rnxp + i] = __fdiv_rn(s, (float)__popc(m));
  }
}

// FFTGrid::extrapolateSeismic (src/fftgrid.cpp:2710-2738): every trace outside
// the box of good traces (box[l] = imin, imax, jmin, jmax; skipped when
// empty) becomes its clamped fill-number reference trace times
// max(1 - dx^2 - dy^2 - dz^2, 0)^3 (double, as the reference); one thread per
// trace, the z loop inside
__global__ void k_extrapolate(const __grid_constant__ CubeSet cs, int ncubes, const int4 *__restrict__ box, int nx, int ny, int nz, int nxp,
                              int nyp, int nzp)
{
  const int rnxp = 2 * (nxp / 2 + 1);
  const long ntr = (long)nxp * nyp;
  const long pstride = (long)nyp * rnxp;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < ntr * ncubes; t += (long)gridDim.x * blockDim.x) {
    const int l = (int)(t / ntr);
    const long c = t - (long)l * ntr;
    const int i = (int)(c % nxp), j = (int)(c / nxp);
    const int4 bx = box[l];
    if (bx.x > bx.y || bx.z > bx.w) continue;
    if (!(i < bx.x || i > bx.y || j < bx.z || j > bx.w)) continue;
    int refj = fill_number(j, ny, nyp);
    if (refj < bx.z) refj = bx.z;
    else if (refj > bx.w) refj = bx.w;
    int refi = fill_number(i, nx, nxp);
    if (refi < bx.x) refi = bx.x;
    else if (refi > bx.y) refi = bx.y;
    float *buf = (float *)cs.ptr[l];
    const float *src = buf + (long)refj * rnxp + refi;
    float *dst = buf + (long)j * rnxp + i;
    const float dx = dist_to_boundary(i, nx, nxp), dy = dist_to_boundary(j, ny, nyp);
    const double sxy = 1.0 - (double)__fmul_rn(dx, dx) - (double)__fmul_rn(dy, dy);
    // inside the simbox in z (k < nz) the distance in z is 0: one factor for those cells
    double w0 = sxy - 0.0;
    w0 = w0 > 0.0 ? w0 : 0.0;
    const float m0 = (float)(w0 * w0 * w0);
    const int kz = nz < nzp ? nz : nzp;
    int k = 0;
    for (; k + 8 <= kz; k += 8) {  // eight loads in flight
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; u++) v[u] = src[(long)(k + u) * pstride];
#pragma unroll
      for (int u = 0; u < 8; u++) dst[(long)(k + u) * pstride] = __fmul_rn(m0, v[u]);
    }
    for (; k < kz; k++) dst[(long)k * pstride] = __fmul_rn(m0, src[(long)k * pstride]);
    for (k = kz; k < nzp; k++) {
      const float dzz = dist_to_boundary(k, nz, nzp);
      double w = sxy - (double)__fmul_rn(dzz, dzz);
      w = w > 0.0 ? w : 0.0;
      dst[(long)k * pstride] = __fmul_rn((float)(w * w * w), src[(long)k * pstride]);
    }
  }
}

int grid_for(long n, int threads = 256)
{
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    nsm = 152;
  const long want = (n + threads - 1) / threads;
  const long cap = (long)nsm * 16;
  return (int)std::max(1L, std::min(want, cap));
}

int check_sw_dims(int ncubes, int nx, int ny, int nxp, int nyp, int nzp)
{
  if (ncubes < 1 || ncubes > kMaxBatch || nx < 1 || ny < 1 || nx > nxp || ny > nyp || nzp < 2) {
    set_error("scale wavelet: bad sizes (ncubes %d in 1..%d, nx %d <= nxp %d, ny %d <= nyp %d, nzp %d)", ncubes,
              kMaxBatch, nx, nxp, ny, nyp, nzp);
    return CG_ERR_ARG;
  }
  return CG_OK;
}

// the shared transform / pointwise / transform sequence of both directions
int sw_apply(int mode, float *const *data, int ncubes, int nx, int ny, int nz, int nxp, int nyp, int nzp,
             const float *tables, const float *rel_thick, const float *shift, const float *gain, float dz, float lz,
             float low_cut, float high_cut, cudaStream_t st)
{
  int rc = check_sw_dims(ncubes, nx, ny, nxp, nyp, nzp);
  if (rc) return rc;
  if (!data || !tables || !rel_thick) { set_error("scale wavelet: null argument"); return CG_ERR_ARG; }
  if (!(dz > 0.0f) || (mode == kSwDivide && (nz < 1 || nz > nzp || !(lz > 0.0f)))) {
    set_error("scale wavelet: bad dz / lz / nz");
    return CG_ERR_ARG;
  }
  CubeSet cs;
  void *ptrs[kMaxBatch];
  for (int i = 0; i < kMaxBatch; i++) cs.ptr[i] = nullptr;
  for (int l = 0; l < ncubes; l++) {
    if (!data[l]) { set_error("scale wavelet: null cube %d", l); return CG_ERR_ARG; }
    cs.ptr[l] = ptrs[l] = data[l];
  }
  const long ntr = (long)nxp * nyp;
  SwTrace *tp = nullptr;
  int2 *kb = nullptr;
  unsigned char *zf = nullptr;
  CG_CUDA(scratch_alloc((void **)&tp, sizeof(SwTrace) * ntr * ncubes, st));
  cudaError_t e = scratch_alloc((void **)&kb, sizeof(int2) * ntr, st);
  if (e == cudaSuccess && mode == kSwDivide) e = scratch_alloc((void **)&zf, (size_t)ntr * ncubes, st);
  if (e != cudaSuccess) {
    cudaFreeAsync(tp, st);
    if (kb) cudaFreeAsync(kb, st);
    return cuda_status(e, "scale wavelet buffers");
  }
  const int cnxp = nxp / 2 + 1;
  const int tstride = cg_scale_wavelet_table_size(nzp);
  do {
    k_sw_params<<<grid_for(ntr * ncubes), 256, 0, st>>>(tp, kb, rel_thick, shift, gain, ncubes, nx, ny, nz, nxp, nyp,
                                                       nzp, dz, lz, low_cut, high_cut, mode == kSwDivide);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    if (zf) {
      k_sw_zero_flags<<<grid_for(ntr * ncubes), 256, 0, st>>>(cs, ncubes, nxp, nyp, nzp, zf);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
    const int k0 = mode == kSwDivide ? std::min(nz + 1, nzp) : nzp;  // taper planes k > nz
    if (k0 > 0 && 2 * cnxp > nxp) {
      k_sw_slack<<<grid_for((long)ncubes * k0 * nyp * (2 * cnxp - nxp)), 256, 0, st>>>(cs, ncubes, k0, nxp, nyp);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
    if (k0 < nzp) {
      TraceScope ts("k_sw_taper", st, 8.0 * ncubes * (double)(nzp - k0) * nyp * 2 * cnxp);
      k_sw_taper<<<grid_for((long)ncubes * (nzp - k0) * nyp * 2 * cnxp), 256, 0, st>>>(cs, ncubes, k0, nz, nxp, nyp,
                                                                                        nzp);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
    if ((rc = fft_cols<float>(ptrs, ncubes, nzp, cnxp, (long)cnxp * nyp, cnxp, nyp, -1, st))) break;
    const long nel = (long)ncubes * (nzp / 2 + 1) * cnxp * nyp;
    const float scale = 1.0f / (float)nzp;
    {
      TraceScope ts(mode == kSwDivide ? "k_sw_divide" : "k_sw_multiply", st,
                    16.0 * ncubes * (double)cnxp * nyp * nzp);
      if (mode == kSwDivide) {
        if (shift) k_sw_spectral<kSwDivide, true><<<grid_for(nel), 256, 0, st>>>(cs, ncubes, tables, tstride, tp, kb, nx, ny, nxp, nyp, nzp, scale);
        else k_sw_spectral<kSwDivide, false><<<grid_for(nel), 256, 0, st>>>(cs, ncubes, tables, tstride, tp, kb, nx, ny, nxp, nyp, nzp, scale);
      } else {
        if (shift) k_sw_spectral<kSwMultiply, true><<<grid_for(nel), 256, 0, st>>>(cs, ncubes, tables, tstride, tp, kb, nx, ny, nxp, nyp, nzp, scale);
        else k_sw_spectral<kSwMultiply, false><<<grid_for(nel), 256, 0, st>>>(cs, ncubes, tables, tstride, tp, kb, nx, ny, nxp, nyp, nzp, scale);
      }
      if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
    if ((rc = fft_cols<float>(ptrs, ncubes, nzp, cnxp, (long)cnxp * nyp, cnxp, nyp, +1, st))) break;
    if (zf) {
      k_sw_zero_apply<<<grid_for(ntr * ncubes), 256, 0, st>>>(cs, ncubes, nxp, nyp, nzp, zf);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
  } while (false);
  if (zf) cudaFreeAsync(zf, st);
  cudaFreeAsync(kb, st);
  cudaFreeAsync(tp, st);
  if (e != cudaSuccess) return cuda_status(e, "scale wavelet kernels");
  return rc;
}

// Host plan of FFTGrid::interpolateSeismic: the reference's flag scan
// (flags depend on energies only), each interpolated trace recorded with its
// neighbour mask and a level one above the highest level among the traces it
// averages (good traces are level 0), so that one launch per level
// reproduces the sequential order.
struct InterpPlan {
  std::vector<std::vector<int2>> levels;
  int imin, imax, jmin, jmax, nbad;
};

void interp_plan(const std::vector<float> &energy, int nx, int ny, float thr, InterpPlan *p)
{
  const long n = (long)nx * ny;
  std::vector<short> flags(n);
  std::vector<int> lev(n, 0);
  float total = 0.0f;
  for (long t = 0; t < n; t++) total += energy[t];
  const float limit = thr * total / (float)(nx * ny);
  int flag = 0;
  p->imin = nx; p->imax = 0; p->jmin = ny; p->jmax = 0; p->nbad = 0;
  long index = 0;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++, index++) {
      int cur = 0;
      if (energy[index] <= limit) { cur = 1; p->nbad++; }
      flags[index] = (short)(flag + cur);
      if (cur == 1) flag = 2;
      else {
        p->imin = std::min(p->imin, i); p->imax = std::max(p->imax, i);
        p->jmin = std::min(p->jmin, j); p->jmax = std::max(p->jmax, j);
      }
    }
  auto interp = [&](long idx, int i, int j) -> int {
    const bool left = i > 0 && flags[idx - 1] % 2 == 0;
    const bool right = i < nx - 1 && flags[idx + 1] % 2 == 0;
    const bool up = j > 0 && flags[idx - nx] % 2 == 0;
    const bool down = j < ny - 1 && flags[idx + nx] % 2 == 0;
    const int nt = (int)left + (int)right + (int)up + (int)down;
    if (nt > 1) {
      int lv = 0;
      if (left) lv = std::max(lv, lev[idx - 1]);
      if (right) lv = std::max(lv, lev[idx + 1]);
      if (up) lv = std::max(lv, lev[idx - nx]);
      if (down) lv = std::max(lv, lev[idx + nx]);
      lev[idx] = lv + 1;
      if ((int)p->levels.size() < lv + 1) p->levels.resize(lv + 1);
      p->levels[lv].push_back(make_int2((int)idx, (left ? 1 : 0) | (right ? 2 : 0) | (up ? 4 : 0) | (down ? 8 : 0)));
      flags[idx]--;
    }
    return flags[idx];
  };
  long cur = 0;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++, cur++) {
      if (flags[cur] % 2 != 1) continue;
      if (interp(cur, i, j) % 2 != 0) continue;
      long ix = cur - 1;
      while (ix >= 0 && flags[ix] > 1) {
        if (flags[ix] % 2 == 1) interp(ix, (int)(ix % nx), (int)(ix / nx));
        ix--;
      }
      if (ix < 0) ix = 0;
      ix++;
      while (flags[ix - 1] == 0 && ix <= cur) {
        if (flags[ix] > 1) flags[ix] -= 2;
        ix++;
      }
    }
}

// FFTGrid::interpolateSeismic on ncubes cubes: one energy launch, one wait
// for the energies, host plans, then per level one launch over all cubes and
// one extrapolation launch
int interpolate_cubes(float *const *cubes, int ncubes, int nx, int ny, int nz, int nxp, int nyp, int nzp, float thr,
                      int *nbad, cudaStream_t st)
{
  CubeSet cs;
  for (int i = 0; i < kMaxBatch; i++) cs.ptr[i] = i < ncubes ? cubes[i] : nullptr;
  const long n = (long)nx * ny;
  float *energy_d = nullptr;
  CG_CUDA(scratch_alloc((void **)&energy_d, sizeof(float) * n * ncubes, st));
  std::vector<float> energy(n * ncubes);
  cudaError_t e;
  {
    TraceScope ts("k_trace_energy", st, 4.0 * (double)n * nz * ncubes);
    k_trace_energy<<<grid_for(n * ncubes), 256, 0, st>>>(cs, ncubes, energy_d, nx, ny, nz, nxp, nyp);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(energy.data(), energy_d, sizeof(float) * n * ncubes, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(energy_d, st);
  if (e != cudaSuccess) return cuda_status(e, "trace energies");
  // ops grouped by level across cubes, then the boxes: one upload
  std::vector<std::vector<int4>> by_level;
  std::vector<int4> boxes(ncubes);
  for (int l = 0; l < ncubes; l++) {
    InterpPlan plan;
    std::vector<float> el(energy.begin() + (long)l * n, energy.begin() + (long)(l + 1) * n);
    interp_plan(el, nx, ny, thr, &plan);
    if (nbad) nbad[l] = plan.nbad;
    boxes[l] = make_int4(plan.imin, plan.imax, plan.jmin, plan.jmax);
    if (by_level.size() < plan.levels.size()) by_level.resize(plan.levels.size());
    for (size_t v = 0; v < plan.levels.size(); v++)
      for (const int2 &op : plan.levels[v]) by_level[v].push_back(make_int4(l, op.x, op.y, 0));
  }
  std::vector<int4> upload(boxes);
  std::vector<long> off;
  for (auto &lv : by_level) {
    off.push_back((long)upload.size());
    upload.insert(upload.end(), lv.begin(), lv.end());
  }
  int4 *up_d = nullptr;
  CG_CUDA(scratch_alloc((void **)&up_d, sizeof(int4) * upload.size(), st));
  e = cudaMemcpyAsync(up_d, upload.data(), sizeof(int4) * upload.size(), cudaMemcpyHostToDevice, st);
  for (size_t v = 0; v < by_level.size() && e == cudaSuccess; v++) {
    const int cnt = (int)by_level[v].size();
    if (cnt == 0) continue;
    k_interp_traces<<<grid_for((long)cnt * nzp), 256, 0, st>>>(cs, up_d + off[v], cnt, nx, nxp, nyp, nzp);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    TraceScope ts("k_extrapolate", st, 0.0);
    k_extrapolate<<<grid_for((long)nxp * nyp * ncubes), 256, 0, st>>>(cs, ncubes, up_d, nx, ny, nz, nxp, nyp, nzp);
    e = cudaGetLastError();
  }
  cudaFreeAsync(up_d, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // upload is a pageable host buffer
  if (e != cudaSuccess) return cuda_status(e, "trace interpolation");
  return CG_OK;
}

}  // namespace
}  // namespace cg

using namespace cg;

extern "C" int cg_interpolate_seismic(float *data, int nx, int ny, int nz, int nxp, int nyp, int nzp,
                                      float energy_threshold, int *n_bad, void *stream)
{
  int rc = check_sw_dims(1, nx, ny, nxp, nyp, nzp);
  if (rc) return rc;
  if (!data || nz < 1 || nz > nzp) { set_error("cg_interpolate_seismic: bad argument"); return CG_ERR_ARG; }
  float *cubes[1] = {data};
  return interpolate_cubes(cubes, 1, nx, ny, nz, nxp, nyp, nzp, energy_threshold, n_bad, (cudaStream_t)stream);
}

extern "C" int cg_divide_by_scale_wavelet(float *const *data, int ntheta, int nx, int ny, int nz, int nxp, int nyp,
                                          int nzp, const float *tables, const float *rel_thick, const float *shift,
                                          const float *gain, float dz_ms, float lz_ms, float low_cut, float high_cut,
                                          float energy_threshold, int *n_bad, void *stream)
{
  cudaStream_t st = (cudaStream_t)stream;
  int rc = sw_apply(kSwDivide, data, ntheta, nx, ny, nz, nxp, nyp, nzp, tables, rel_thick, shift, gain, dz_ms, lz_ms,
                    low_cut, high_cut, st);
  if (rc) return rc;
  if (energy_threshold < 0.0f) return CG_OK;  // interpolation left to the caller
  return interpolate_cubes(data, ntheta, nx, ny, nz, nxp, nyp, nzp, energy_threshold, n_bad, st);
}

extern "C" int cg_multiply_by_scale_wavelet(float *const *data, int ncubes, int nx, int ny, int nxp, int nyp, int nzp,
                                            const float *tables, const float *rel_thick, const float *shift,
                                            const float *gain, float dz_ms, void *stream)
{
  return sw_apply(kSwMultiply, data, ncubes, nx, ny, 1, nxp, nyp, nzp, tables, rel_thick, shift, gain, dz_ms, 1.0f,
                  0.0f, 0.0f, (cudaStream_t)stream);
}
