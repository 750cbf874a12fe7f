// Host-side per-frequency operator tables of the inversion (C++, no CUDA).
//
// For every temporal frequency index k this builds what
// Crava::fillErrMultVectors (src/crava.cpp:1337-1361, constant-thickness
// branch) hands to the per-bin solve:
//   K[k][l][p] = kD(k) * conj(W_l(k)) * A[l][p]
//   errMult1[k][l] = conj(W_l(k)) / ||w_l||
//   errMult2[k][l] = conj(E3_l(k)) / ||e3_l||
//   errMult3[k][l] = 1
// with kD the spectrum of the forward-difference operator
// (Wavelet1D FIRSTORDERFORWARDDIFF, src/wavelet1D.cpp:367-416), W_l the
// spectrum of the resampled wavelet (Wavelet::fft1DInPlace + getCAmp,
// src/wavelet.cpp:246-325) and e3_l = central(backward(forward(w_l)))
// (Crava::makeErrorSmooth, src/crava.cpp:1289-1323, Wavelet1D ctor
// src/wavelet1D.cpp:419-479), plus the inversion band of
// src/crava.cpp:1104-1105.  Spectra are computed in double by a small
// mixed-radix FFT and rounded to float.
#include <cmath>
#include <complex>
#include <vector>

#include "cravagpu.h"

namespace cg {
void set_error(const char *fmt, ...);
}

namespace {

typedef std::complex<double> cd;

// recursive mixed-radix DFT, sign -1 (forward), out[k] = sum x[j] e^{-2 pi i jk/n}
void dft_rec(const cd *x, int n, int stride, cd *out, const std::vector<cd> &tw, int twstep)
{
  if (n == 1) { out[0] = x[0]; return; }
  int r = 2;
  while (n % r) r++;
  const int m = n / r;
  for (int q = 0; q < r; q++) dft_rec(x + q * stride, m, stride * r, out + q * m, tw, twstep * r);
  std::vector<cd> t(r);
  const int N = (int)tw.size();
  for (int k = 0; k < m; k++) {
    for (int q = 0; q < r; q++) t[q] = out[q * m + k] * tw[((long)q * k * twstep) % N];
    for (int u = 0; u < r; u++) {
      cd acc = 0;
      for (int q = 0; q < r; q++) acc += t[q] * tw[((long)q * u * m * twstep) % N];
      out[u * m + k] = acc;
    }
  }
}

std::vector<cd> rfft(const std::vector<double> &x)
{
  const int n = (int)x.size();
  std::vector<cd> tw(n), in(n), out(n);
  for (int t = 0; t < n; t++) tw[t] = std::polar(1.0, -2.0 * M_PI * t / n);
  for (int t = 0; t < n; t++) in[t] = x[t];
  dft_rec(in.data(), n, 1, out.data(), tw, 1);
  return out;  // full spectrum; getCAmp semantics are applied by the caller
}

double norm2(const std::vector<double> &x)
{
  double s = 0;
  for (double v : x) s += (double)((float)v * (float)v);
  return std::sqrt(s);
}

}  // namespace

extern "C" int cg_operator_tables(int ntheta, int nz, int nzp, const float *wavelets, const float *A, float dt_ms,
                                  float min_rel_thick, float low_cut, float high_cut, float *K, float *em1,
                                  float *em2, float *em3, unsigned char *band)
{
  if (ntheta < 1 || nzp < 2 || nz < 1 || !wavelets || !A || !K || !em1 || !em2 || !em3 || !band) {
    cg::set_error("cg_operator_tables: bad argument");
    return CG_ERR_ARG;
  }
  std::vector<double> d1(nzp, 0.0);
  d1[0] = -1.0;
  d1[nzp - 1] = 1.0;
  const std::vector<cd> kD = rfft(d1);
  const float lz = nz * dt_ms;
  for (int l = 0; l < ntheta; l++) {
    std::vector<double> w(nzp), f(nzp), b(nzp), e3(nzp);
    for (int i = 0; i < nzp; i++) w[i] = wavelets[(long)l * nzp + i];
    for (int i = 0; i < nzp; i++) f[i] = (float)((i == nzp - 1) ? w[0] - w[i] : w[i + 1] - w[i]);
    for (int i = 0; i < nzp; i++) b[i] = (float)((i == 0) ? f[0] - f[nzp - 1] : f[i] - f[i - 1]);
    for (int i = 0; i < nzp; i++) {
      double v = (i == 0) ? 0.5 * (b[1] - b[nzp - 1]) : (i == nzp - 1) ? 0.5 * (b[0] - b[i - 1]) : 0.5 * (b[i + 1] - b[i - 1]);
      e3[i] = (float)v;
    }
    const double wn = (float)norm2(w), en = (float)norm2(e3);
    const std::vector<cd> W = rfft(w), E = rfft(e3);
    for (int k = 0; k < nzp; k++) {
      // the full spectrum already holds getCAmp's reflected/conjugated values for k >= nzp/2+1
      const cd kw = std::conj(W[k]);
      const cd p = kD[k] * kw;
      for (int q = 0; q < 3; q++) {
        const long o = (((long)k * ntheta + l) * 3 + q) * 2;
        K[o] = (float)(p.real() * (double)A[l * 3 + q]);
        K[o + 1] = (float)(p.imag() * (double)A[l * 3 + q]);
      }
      const long o = ((long)k * ntheta + l) * 2;
      em1[o] = (float)(W[k].real() / wn);
      em1[o + 1] = (float)(-W[k].imag() / wn);
      em2[o] = (float)(E[k].real() / en);
      em2[o + 1] = (float)(-E[k].imag() / en);
      em3[o] = 1.0f;
      em3[o + 1] = 0.0f;
    }
  }
  for (int k = 0; k < nzp; k++) {
    const int kk = k < nzp - k ? k : nzp - k;
    const float f = (float)((nz * 1000.0f) / (lz * nzp) * kk);
    band[k] = (f > low_cut * min_rel_thick && f < high_cut) ? 1 : 0;
  }
  return CG_OK;
}

// FFTGrid::findClosestFactorableNumber (src/fftgrid.cpp:2857-2885): smallest
// 2^a 3^b 5^c 7^d that is >= n.
extern "C" int cg_find_closest_factorable(int n)
{
  if (n < 1) return 1;
  long best = -1;
  for (long p2 = 1; p2 < 2L * n; p2 *= 2)
    for (long p3 = p2; p3 < 2L * n; p3 *= 3)
      for (long p5 = p3; p5 < 2L * n; p5 *= 5)
        for (long p7 = p5; p7 < 2L * n; p7 *= 7)
          if (p7 >= n && (best < 0 || p7 < best)) best = p7;
  return (int)best;
}
