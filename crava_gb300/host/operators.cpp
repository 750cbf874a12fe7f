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
// src/crava.cpp:1104-1105.  The non-constant-thickness branch
// (src/crava.cpp:1362-1385) has K = kD * A, errMult1 = 1/||w||,
// errMult2 = kD3/||e3|| (kD3: the third-difference operator) and errMult3 =
// 1/max(|W(k)|, |W(k/0.999)|) (fillInverseAbskWRobust, :1493-1519).
// Spectra are computed in double by a small mixed-radix FFT and rounded to
// float.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "cravagpu.h"

namespace cg {
void set_error(const char *fmt, ...);
}

namespace {

typedef std::complex<double> cd;

// complex product without the library's inf/NaN recovery call (operands are finite)
inline cd cmul(cd a, cd b)
{
  return cd(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
}

// recursive mixed-radix DFT, sign -1 (forward), out[k] = sum x[j] e^{-2 pi i jk/n}.
// tw holds e^{-2 pi i t / N} for the top-level length N; at every level
// n * twstep = N, so the twiddle indices below stay under N without a modulo.
void dft_rec(const cd *x, int n, int stride, cd *out, const std::vector<cd> &tw, int twstep)
{
  if (n == 1) { out[0] = x[0]; return; }
  int r = n % 4 == 0 ? 4 : 2;
  while (n % r) r++;
  const int m = n / r;
  for (int q = 0; q < r; q++) dft_rec(x + q * stride, m, stride * r, out + q * m, tw, twstep * r);
  if (r == 2 || r == 4) {
    // butterflies: W_2 = -1, W_4 = -i
    for (int k = 0; k < m; k++) {
      if (r == 2) {
        const cd a = out[k], b = cmul(out[m + k], tw[(long)k * twstep]);
        out[k] = a + b;
        out[m + k] = a - b;
      } else {
        const cd t0 = out[k], t1 = cmul(out[m + k], tw[(long)k * twstep]);
        const cd t2 = cmul(out[2 * m + k], tw[(long)2 * k * twstep]), t3 = cmul(out[3 * m + k], tw[(long)3 * k * twstep]);
        const cd s02 = t0 + t2, d02 = t0 - t2, s13 = t1 + t3, d13 = t1 - t3;
        const cd jd13(d13.imag(), -d13.real());  // -i (t1 - t3)
        out[k] = s02 + s13;
        out[m + k] = d02 + jd13;
        out[2 * m + k] = s02 - s13;
        out[3 * m + k] = d02 - jd13;
      }
    }
    return;
  }
  cd tb[16], wb[16];
  std::vector<cd> th, wh;
  if (r > 16) { th.resize(r); wh.resize(r); }  // radices above 16 only for lengths with a large prime factor
  cd *t = r > 16 ? th.data() : tb;
  cd *wr = r > 16 ? wh.data() : wb;  // the r-th roots of unity e^{-2 pi i j / r}
  for (int j = 0; j < r; j++) wr[j] = tw[(long)j * m * twstep];
  for (int k = 0; k < m; k++) {
    for (int q = 0; q < r; q++) t[q] = cmul(out[q * m + k], tw[(long)q * k * twstep]);
    for (int u = 0; u < r; u++) {
      cd acc = 0;
      int idx = 0;
      for (int q = 0; q < r; q++) {
        acc += cmul(t[q], wr[idx]);
        idx += u;
        if (idx >= r) idx -= r;
      }
      out[u * m + k] = acc;
    }
  }
}

std::vector<cd> twiddles(int n)
{
  std::vector<cd> tw(n);
  for (int t = 0; t < n; t++) tw[t] = std::polar(1.0, -2.0 * M_PI * t / n);
  return tw;
}

// full spectrum of a real sequence with the reference's half-spectrum semantics: the DC (and, for even
// n, Nyquist) bins are real and bins k >= n/2+1 are the conjugates of bins n-k, as Wavelet::getCAmp
// reflects them (src/wavelet.cpp:309-325), so every table built from it is exactly conjugate-symmetric
std::vector<cd> rfft(const std::vector<double> &x, const std::vector<cd> &tw)
{
  const int n = (int)x.size();
  std::vector<cd> in(x.begin(), x.end()), out(n);
  dft_rec(in.data(), n, 1, out.data(), tw, 1);
  out[0] = cd(out[0].real(), 0.0);
  if (n % 2 == 0) out[n / 2] = cd(out[n / 2].real(), 0.0);
  for (int k = n / 2 + 1; k < n; k++) out[k] = std::conj(out[n - k]);
  return out;
}

std::vector<cd> rfft(const std::vector<double> &x) { return rfft(x, twiddles((int)x.size())); }

double norm2(const std::vector<double> &x)
{
  double s = 0;
  for (double v : x) s += (double)((float)v * (float)v);
  return std::sqrt(s);
}

}  // namespace

extern "C" int cg_operator_tables_ex(int ntheta, int nz, int nzp, const float *wavelets, const float *A, float dt_ms,
                                     float min_rel_thick, float low_cut, float high_cut, int constant_thickness,
                                     float *K, float *em1, float *em2, float *em3, unsigned char *band)
{
  if (ntheta < 1 || nzp < 2 || nz < 1 || !wavelets || !A || !K || !em1 || !em2 || !em3 || !band) {
    cg::set_error("cg_operator_tables: bad argument");
    return CG_ERR_ARG;
  }
  std::vector<double> d1(nzp, 0.0);
  d1[0] = -1.0;
  d1[nzp - 1] = 1.0;
  const std::vector<cd> twz = twiddles(nzp);
  const std::vector<cd> kD = rfft(d1, twz);
  // third-difference operator central(backward(d1)) for the non-constant-thickness errMult2
  std::vector<double> d2(nzp), d3(nzp);
  for (int i = 0; i < nzp; i++) d2[i] = (float)((i == 0) ? d1[0] - d1[nzp - 1] : d1[i] - d1[i - 1]);
  for (int i = 0; i < nzp; i++) {
    const double v = (i == 0) ? 0.5 * (d2[1] - d2[nzp - 1]) : (i == nzp - 1) ? 0.5 * (d2[0] - d2[i - 1]) : 0.5 * (d2[i + 1] - d2[i - 1]);
    d3[i] = (float)v;
  }
  const std::vector<cd> kD3 = rfft(d3, twz);
  const float lz = nz * dt_ms;
  const int cnzp = nzp / 2 + 1;
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
    const std::vector<cd> W = rfft(w, twz), E = rfft(e3, twz);
    for (int k = 0; k < nzp; k++) {
      const long o = ((long)k * ntheta + l) * 2;
      if (constant_thickness) {
        // the full spectrum holds getCAmp's reflected/conjugated values for k >= nzp/2+1
        const cd kw = std::conj(W[k]);
        const cd p = cmul(kD[k], kw);
        for (int q = 0; q < 3; q++) {
          const long oq = (((long)k * ntheta + l) * 3 + q) * 2;
          K[oq] = (float)(p.real() * (double)A[l * 3 + q]);
          K[oq + 1] = (float)(p.imag() * (double)A[l * 3 + q]);
        }
        em1[o] = (float)(W[k].real() / wn);
        em1[o + 1] = (float)(-W[k].imag() / wn);
        em2[o] = (float)(E[k].real() / en);
        em2[o + 1] = (float)(-E[k].imag() / en);
        em3[o] = 1.0f;
        em3[o + 1] = 0.0f;
      } else {
        // K = kD A, errMult1 = 1/||w||, errMult2 = kD3/||e3||, errMult3 = fillInverseAbskWRobust
        for (int q = 0; q < 3; q++) {
          const long oq = (((long)k * ntheta + l) * 3 + q) * 2;
          K[oq] = (float)(kD[k].real() * (double)A[l * 3 + q]);
          K[oq + 1] = (float)(kD[k].imag() * (double)A[l * 3 + q]);
        }
        em1[o] = (float)(1.0 / wn);
        em1[o + 1] = 0.0f;
        em2[o] = (float)(kD3[k].real() / en);
        em2[o + 1] = (float)(kD3[k].imag() / en);
        // |W| at k and at the spectrum stretched by 0.999 (Wavelet::getCAmp(k, 0.999f)), the larger one
        const int kk = k < cnzp ? k : nzp - k;
        const float omega = (float)kk / 0.999f;
        double modf = 0.0;
        if (omega < (float)cnzp) {
          const int omL = (int)std::floor(omega);
          const int omU = omL + 1 < cnzp ? omL + 1 : omL;
          const float d = omega - (float)omL;
          // getCAmp(k, scale) returns the interpolated value times 1/scale (src/wavelet.cpp:382-383)
          const cd v = (W[omL] * (double)(1.0f - d) + W[omU] * (double)d) / (double)0.999f;
          modf = std::norm(v);
        }
        const double maxMod = std::max(std::norm(W[kk]), modf);
        em3[o] = maxMod > 0.0 ? (float)(1.0 / std::sqrt(maxMod)) : (float)(wn * nzp * nzp * 100.0);
        em3[o + 1] = 0.0f;
      }
    }
  }
  for (int k = 0; k < nzp; k++) {
    const int kk = k < nzp - k ? k : nzp - k;
    const float f = (float)((nz * 1000.0f) / (lz * nzp) * kk);
    band[k] = (f > low_cut * min_rel_thick && f < high_cut) ? 1 : 0;
  }
  return CG_OK;
}

extern "C" int cg_operator_tables(int ntheta, int nz, int nzp, const float *wavelets, const float *A, float dt_ms,
                                  float min_rel_thick, float low_cut, float high_cut, float *K, float *em1,
                                  float *em2, float *em3, unsigned char *band)
{
  return cg_operator_tables_ex(ntheta, nz, nzp, wavelets, A, dt_ms, min_rel_thick, low_cut, high_cut, 1, K, em1, em2,
                               em3, band);
}

// ---------------------------------------------------------------------------
// Per-angle tables of Crava::computeAdjustmentFactor (src/crava.cpp:807-903)
// for the non-constant-thickness data scaling (divideDataByScaleWavelet) and
// its inverse (multiplyDataByScaleWaveletAndWriteToFile).  Per angle, with
// c = nzp/2 + 1 frequency bins:
//   [0, 2c)    W     spectrum of the global wavelet (R2C, unnormalised)
//   [2c, 4c)   E3    spectrum of central(backward(forward(w))) divided by its
//                    band-limited norm (Wavelet::findNormWithinFrequencyBand);
//                    the device lookup replaces the floats past nzp by
//                    RMISSING, as Wavelet::multiplyRAmpByConstant leaves them
//   [4c, 5c)   tau2  |Re| of the FFT of the reflection-coefficient time
//                    covariance (computeReflectionCoefficientTimeCovariance)
//   5c + 0..3  ||w||^2, modW (mean squared wavelet amplitude up to highCut),
//              errThetaCov[l][l], wnc
// ---------------------------------------------------------------------------
extern "C" int cg_scale_wavelet_table_size(int nzp) { return ((5 * (nzp / 2 + 1) + 4) + 3) & ~3; }

extern "C" int cg_scale_wavelet_tables(int ntheta, int nz, int nzp, const float *wavelets, const float *A,
                                       const double *prior_var0, const float *circ_corr_t,
                                       const double *err_theta_cov, float dz_ms, float lz_ms, float low_cut,
                                       float high_cut, float wnc, float *tables)
{
  if (ntheta < 1 || nz < 1 || nzp < 2 || !wavelets || !A || !prior_var0 || !circ_corr_t || !err_theta_cov ||
      !tables || !(dz_ms > 0) || !(lz_ms > 0) || !(high_cut > 0)) {
    cg::set_error("cg_scale_wavelet_tables: bad argument");
    return CG_ERR_ARG;
  }
  const int c = nzp / 2 + 1, ts = cg_scale_wavelet_table_size(nzp);
  for (int l = 0; l < ntheta; l++) {
    float *t = tables + (long)l * ts;
    for (int i = 0; i < ts; i++) t[i] = 0.0f;
    std::vector<double> w(nzp), f(nzp), b(nzp), e3(nzp), rc(nzp);
    for (int i = 0; i < nzp; i++) w[i] = wavelets[(long)l * nzp + i];
    const std::vector<cd> W = rfft(w);
    for (int k = 0; k < c; k++) { t[2 * k] = (float)W[k].real(); t[2 * k + 1] = (float)W[k].imag(); }
    for (int i = 0; i < nzp; i++) f[i] = (float)((i == nzp - 1) ? w[0] - w[i] : w[i + 1] - w[i]);
    for (int i = 0; i < nzp; i++) b[i] = (float)((i == 0) ? f[0] - f[nzp - 1] : f[i] - f[i - 1]);
    for (int i = 0; i < nzp; i++) {
      const double v = (i == 0) ? 0.5 * (b[1] - b[nzp - 1]) : (i == nzp - 1) ? 0.5 * (b[0] - b[i - 1]) : 0.5 * (b[i + 1] - b[i - 1]);
      e3[i] = (float)v;
    }
    const std::vector<cd> E = rfft(e3);
    // band-limited norm of E3 (dOmega in float as the reference computes it)
    const float dOmega = 1.0f / ((float)nzp * dz_ms * 0.001f);
    const int loI = std::max(0, (int)std::floor(low_cut / dOmega));
    const int hiI = std::min(c, (int)std::ceil(high_cut / dOmega));
    double n2 = 0.0;
    for (int i = loI; i < hiI; i++) n2 += 2.0 / nzp * std::norm(E[i]);
    if (loI == 0) n2 -= 1.0 / nzp * std::norm(E[0]);
    const double normF3 = std::sqrt(n2);
    float *te = t + 2 * c;
    for (int i = 0; i < 2 * c; i++) {
      const cd v = E[i / 2];
      te[i] = (float)((i % 2 ? v.imag() : v.real()) / normF3);
    }
    // reflection-coefficient time covariance: eiVar * corrT filtered to refk < nz, then 2 c_i - c_{i+1} - c_{i-1}
    double eiVar = 0.0;
    for (int p = 0; p < 3; p++)
      for (int q = 0; q < 3; q++) eiVar += (double)A[l * 3 + p] * prior_var0[p * 3 + q] * (double)A[l * 3 + q];
    std::vector<double> ei(nzp);
    for (int k = 0; k < nzp; k++) {
      const int refk = k < c ? k : nzp - k;
      ei[k] = refk < nz ? eiVar * (double)circ_corr_t[refk] : 0.0;
    }
    for (int i = 0; i < nzp; i++) rc[i] = 2.0 * ei[i] - ei[(i + 1) % nzp] - ei[(i + nzp - 1) % nzp];
    const std::vector<cd> RC = rfft(rc);
    for (int k = 0; k < c; k++) t[4 * c + k] = (float)std::fabs(RC[k].real());
    const float wn = (float)norm2(w);
    float modW = wn * wn;
    const float maxfrequency = (float)((nzp / 2) * 1000.0 * nz) / (float)((double)lz_ms * nzp);
    modW *= maxfrequency / high_cut;
    t[5 * c + 0] = wn * wn;
    t[5 * c + 1] = modW;
    t[5 * c + 2] = (float)err_theta_cov[(long)l * ntheta + l];
    t[5 * c + 3] = wnc;
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
