// Data ingest: the per-trace numerical core of FFTGrid::fillInData
// (src/fftgrid.cpp:138-370) for every column of a padded real cube.
//
// The caller supplies one trace per column c = i + rnxp*j (its geometry
// lookup: getFillNumber, Simbox::getCoord and the nearest SegY / STORM trace)
// with the trace's start time and the column's simbox top and thickness.
// Per trace, as the reference:
//   non-DATA cubes: leading/trailing zeros extrapolated (extrapolateAtEnds)
//     and the linear trend between the end samples removed
//     (removeTrendFromTrace);
//   DATA cubes: sin^2 / cos^2 taper over smooth_length at both ends
//     (smoothTraceInGuardZone);
//   resampleTrace: real transform of length nt = findClosestFactorableNumber
//     (n_data), spectrum zero-padded to 4*nt, inverse transform, x 1/rnt;
//   interpolateGridValues: linear interpolation of the fine trace at every
//     grid cell, cells in getZSimboxIndex order;
//   non-DATA: addTrendToTrace (trend restored in the simbox, a ramp in the
//     padding).
// Here the traces of all columns go through the two transforms as one
// batch of rows; the per-trace steps are one thread per column.
#include <cmath>

#include "common.cuh"
#include "fft.cuh"
#include "trace.cuh"

namespace cg {

struct IngestArgs {
  const float *traces;         // [ncol][n_data]
  const unsigned char *state;  // [ncol]: 0 trace present, else dead / outside
  const float *z0_data, *z0_grid, *dz_grid;  // [ncol]
  float *coarse;               // [ncol][rnt]
  const float *fine;           // [ncol][rmt]
  float2 *trend;               // [ncol]: first, last
  float *buf;                  // [nzp][nyp][rnxp]
  int *extrap;                 // [2]
  long ncol;
  int n_data, rnt, rmt, nz, nzp, is_data;
  float dz_data, smooth_length;
};

__global__ void k_trace_prep(const __grid_constant__ IngestArgs a)
{
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.ncol) return;
  float *row = a.coarse + c * a.rnt;
  const float *tr = a.traces + c * a.n_data;
  const int n = a.n_data;
  if (a.state[c]) {
    for (int k = 0; k < a.rnt; k++) row[k] = 0.0f;
    return;
  }
  for (int k = 0; k < n; k++) row[k] = tr[k];
  for (int k = n; k < a.rnt; k++) row[k] = 0.0f;
  if (!a.is_data) {
    int first = 0;
    while (first < n && row[first] == 0.0f) first++;
    if (first < n) {  // an all-zero trace is left as it is
      for (int k = 0; k < first; k++) row[k] = row[first];
      int last = n - 1;
      while (row[last] == 0.0f) last--;
      for (int k = last + 1; k < n; k++) row[k] = row[last];
      atomicMax(&a.extrap[0], first);
      atomicMax(&a.extrap[1], n - last - 1);
    }
    const float tf = row[0], tl = row[n - 1];
    const float s = n > 1 ? (tl - tf) / (float)(n - 1) : 0.0f;
    for (int k = 0; k < n; k++) row[k] -= tf + s * (float)k;
    a.trend[c] = make_float2(tf, tl);
  } else {
    const int ns = (int)floor((double)(a.smooth_length / a.dz_data));
    for (int k = 0; k < ns && k < n; k++) {
      const float v = (float)sin(1.5707963267948966 * ((double)k / (double)ns));
      row[k] *= v * v;
    }
    const int k0 = n - ns;
    for (int k = 0; k < ns; k++) {
      if (k0 + k < 0) continue;
      const float v = (float)cos(1.5707963267948966 * ((double)(k + 1) / (double)ns));
      row[k0 + k] *= v * v;
    }
  }
}

// zero-padding of the coarse half spectrum (cnt bins) to the fine one (cmt bins)
__global__ void k_pad_spectrum(const float2 *__restrict__ coarse, float2 *__restrict__ fine, long ncol, int cnt,
                               int cmt)
{
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncol * cmt) return;
  const long c = t / cmt;
  const int u = (int)(t - c * cmt);
  fine[t] = u < cnt ? coarse[c * cnt + u] : make_float2(0.0f, 0.0f);
}

__device__ __forceinline__ float fine_at(const float *f, float dl, int nf)
{
  const int l1 = (int)floorf(dl), l2 = (int)ceilf(dl);
  if (l2 < 0 || l1 > nf - 1) return 0.0f;
  if (l1 < 0) return f[l2];
  if (l2 > nf - 1) return f[l1];
  if (l1 == l2) return f[l1];
  const float w1 = ceilf(dl) - dl, w2 = dl - floorf(dl);
  return w1 * f[l1] + w2 * f[l2];
}

__global__ void k_trace_to_grid(const __grid_constant__ IngestArgs a)
{
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.ncol) return;
  float *out = a.buf + c;  // cell k of column c at out[k * ncol]
  if (a.state[c]) {
    for (int k = 0; k < a.nzp; k++) out[(long)k * a.ncol] = 0.0f;
    return;
  }
  const float *f = a.fine + c * a.rmt;
  const float z0s = a.z0_grid[c] - a.z0_data[c], dzg = a.dz_grid[c];
  const float inv = 1.0f / (a.dz_data / 4.0f);
  const int half = (a.nz + a.nzp) / 2;
  float trend_a = 0.0f, tf = 0.0f, tl = 0.0f, g0 = 0.0f, gn = 0.0f;
  if (!a.is_data) {
    const float2 tr = a.trend[c];
    tf = tr.x;
    tl = tr.y;
    trend_a = a.n_data > 1 ? (tl - tf) / ((float)(a.n_data - 1) * a.dz_data) : 0.0f;
  }
  for (int k = 0; k < a.nzp; k++) {
    const int refk = k < half ? k : k - a.nzp;  // getZSimboxIndex
    float v = fine_at(f, (z0s + (float)refk * dzg) * inv, a.rmt);
    if (!a.is_data) {
      if (k < a.nz) {
        const float z = a.z0_grid[c] + (float)k * dzg;
        v += trend_a * (z - a.z0_data[c]) + tf;
        if (k == 0) g0 = v;
        if (k == a.nz - 1) gn = v;
      } else {
        v = tl - ((gn - g0) / (float)(a.nzp - a.nz)) * (float)(k - a.nz);
      }
    }
    out[(long)k * a.ncol] = v;
  }
}

}  // namespace cg

using namespace cg;

extern "C" int cg_fill_in_data(float *buf, int nxp, int nyp, int nzp, int nz, int cubetype, const float *traces,
                               int n_data, const unsigned char *state, const float *z0_data, const float *z0_grid,
                               const float *dz_grid, float dz_data, float smooth_length, int *extrap_out,
                               void *stream)
{
  if (!buf || !traces || !state || !z0_data || !z0_grid || !dz_grid || nxp < 1 || nyp < 1 || nzp < 1 || nz < 1 ||
      nz > nzp || n_data < 1 || !(dz_data > 0.0f)) {
    set_error("cg_fill_in_data: bad argument");
    return CG_ERR_ARG;
  }
  if (cubetype < CG_DATA || cubetype > CG_OPERATOR) { set_error("cubetype %d is not valid", cubetype); return CG_ERR_ARG; }
  const int nt = cg_find_closest_factorable(n_data), mt = 4 * nt;
  if (mt > cg_fft_max_length()) { set_error("traces of %d samples resample beyond the longest transform", n_data); return CG_ERR_UNSUPPORTED; }
  cudaStream_t st = (cudaStream_t)stream;
  IngestArgs a;
  a.traces = traces;
  a.state = state;
  a.z0_data = z0_data;
  a.z0_grid = z0_grid;
  a.dz_grid = dz_grid;
  a.buf = buf;
  a.ncol = (long)(2 * (nxp / 2 + 1)) * nyp;
  a.n_data = n_data;
  a.rnt = 2 * (nt / 2 + 1);
  a.rmt = 2 * (mt / 2 + 1);
  a.nz = nz;
  a.nzp = nzp;
  a.is_data = cubetype == CG_DATA;
  a.dz_data = dz_data;
  a.smooth_length = smooth_length;
  if (a.ncol > 0x7fffffffL) { set_error("too many columns"); return CG_ERR_UNSUPPORTED; }
  float *coarse = nullptr, *fine = nullptr;
  float2 *trend = nullptr;
  int *ext = nullptr;
  CG_CUDA(scratch_alloc((void **)&coarse, sizeof(float) * (size_t)a.ncol * a.rnt, st));
  cudaError_t e = scratch_alloc((void **)&fine, sizeof(float) * (size_t)a.ncol * a.rmt, st);
  if (e == cudaSuccess) e = scratch_alloc((void **)&trend, sizeof(float2) * (size_t)a.ncol, st);
  if (e == cudaSuccess) e = scratch_alloc((void **)&ext, 2 * sizeof(int), st);
  int rc = CG_OK;
  if (e != cudaSuccess) rc = cuda_status(e, "ingest buffers");
  if (!rc) {
    a.coarse = coarse;
    a.fine = fine;
    a.trend = trend;
    a.extrap = ext;
    e = cudaMemsetAsync(ext, 0, 2 * sizeof(int), st);
    if (e != cudaSuccess) rc = cuda_status(e, "ingest counters");
  }
  if (!rc) {
    TraceScope ts("k_trace_prep", st, 4.0 * a.ncol * ((double)n_data + a.rnt));
    k_trace_prep<<<ceil_div(a.ncol, 128), 128, 0, st>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_status(e, "k_trace_prep");
  }
  if (!rc) rc = fft_rows<float>(coarse, nt, (int)a.ncol, true, 1.0f, st);
  if (!rc) {
    const long n = a.ncol * (mt / 2 + 1);
    k_pad_spectrum<<<ceil_div(n, 256), 256, 0, st>>>((const float2 *)coarse, (float2 *)fine, a.ncol, nt / 2 + 1,
                                                     mt / 2 + 1);
    e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_status(e, "k_pad_spectrum");
  }
  if (!rc) rc = fft_rows<float>(fine, mt, (int)a.ncol, false, 1.0f / (float)a.rnt, st);
  if (!rc) {
    TraceScope ts("k_trace_to_grid", st, 4.0 * a.ncol * ((double)a.rmt + nzp));
    k_trace_to_grid<<<ceil_div(a.ncol, 128), 128, 0, st>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_status(e, "k_trace_to_grid");
  }
  int hext[2] = {0, 0};
  if (!rc && extrap_out) {
    e = cudaMemcpyAsync(hext, ext, sizeof(hext), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_status(e, "ingest counters");
    extrap_out[0] = hext[0];
    extrap_out[1] = hext[1];
  }
  if (coarse) cudaFreeAsync(coarse, st);
  if (fine) cudaFreeAsync(fine, st);
  if (trend) cudaFreeAsync(trend, st);
  if (ext) cudaFreeAsync(ext, st);
  return rc;
}
