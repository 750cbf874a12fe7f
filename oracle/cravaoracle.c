/*
 * CPU oracle for the FFT-domain Bayesian AVO inversion path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GPU
 * implementation is compared against, and the CPU baseline timed next to it.
 * It is never linked into, loaded by, or called from the product library.
 *
 * It restates, in plain C, the reference CRAVA algorithm (paths relative to
 * the CRAVA source tree):
 *   - FFTGrid::fftInPlace / invFFTInPlace      src/fftgrid.cpp:1783-1842
 *   - the bin loop of Crava::computePostMeanResidAndFFTCov
 *                                              src/crava.cpp:1084-1247
 *   - Crava::simulate bin loop                 src/crava.cpp:1617-1656
 *   - State4D::merge / mergeCov / split        src/state4d.cpp:140-580
 *   - FFTGrid::fillInParamCorr / fillInErrCorr src/fftgrid.cpp:1018-1119
 *   - FFTGrid::fillInComplexNoise              src/fftgrid.cpp:1191-1241
 *   - RandomGen::unif01 / rnorm01              libs/lib/random.cpp:39-121
 *   - FFTGrid::findClosestFactorableNumber     src/fftgrid.cpp:2857-2885
 * in single precision (same operation order as the reference) and in double
 * precision (the FP64 oracle).  Parity of this restatement is pinned against
 * the reference's own FFTW 2.1.2, lib_matr.c and RandomGen compiled from the
 * reference sources (see ref_harness.cpp and Makefile.ref).
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define OR_DATA 1
#define OR_PARAMETER 2
#define OR_COVARIANCE 3
#define OR_OPERATOR 5
#define OR_TOL 1e-20
#define OR_RMISSING (-99999.000f)

#define R float
#define SFX _f
#include "oracle_impl.inc"
#undef R
#undef SFX

#define R double
#define SFX _d
#include "oracle_impl.inc"
#undef R
#undef SFX

/* ------------------------------------------------------------------------ */
/* RandomGen (libs/lib/random.cpp, libs/lib/random.h:11-14): 32-bit LCG      */
/* seed = 69069*seed + 1, u = seed * 2^-32, Marsaglia-Bray normal draws.     */
/* The state is passed explicitly instead of living in a static.             */
/* ------------------------------------------------------------------------ */
static double or_unif01(unsigned int *seed)
{
  *seed = 69069u * (*seed) + 1u;
  return (double)(*seed) * ((1.0 / (double)(256 * 256 * 256 * 64)) / 4.0);
}

static double or_g(double x)
{
  double a = 17.49731196, b = 2.36785163, c = 2.15787544;
  double absx = fabs(x);
  double result = a * exp(-x * x / 2.0);
  if (absx < 1.0) result -= 2.0 * b * (3.0 - x * x) + c * (1.5 - absx);
  else if (absx < 1.5) result -= b * (3.0 - absx) * (3.0 - absx) + c * (1.5 - absx);
  else result -= b * (3.0 - absx) * (3.0 - absx);
  return result;
}

double or_rnorm01(unsigned int *seed)
{
  double u, u1, u2, u3, c, x, v1, v2, w, s, t;
  u = or_unif01(seed);
  if (u < 0.8638) {
    u1 = or_unif01(seed); u2 = or_unif01(seed); u3 = or_unif01(seed);
    x = 2.0 * (u1 + u2 + u3) - 3.0;
  } else if (u < 0.9745) {
    u1 = or_unif01(seed); u2 = or_unif01(seed);
    x = 1.5 * (u1 + u2 - 1.0);
  } else if (u < 0.9973002039) {
    do {
      u1 = or_unif01(seed); u2 = or_unif01(seed);
      x = 6.0 * u1 - 3.0;
    } while (0.358 * u2 > or_g(x));
  } else {
    do {
      do {
        u1 = or_unif01(seed); u2 = or_unif01(seed);
        v1 = 2.0 * u1 - 1.0; v2 = 2.0 * u2 - 1.0;
        w = v1 * v1 + v2 * v2;
      } while (w >= 1.0);
      c = sqrt((9.0 - 2.0 * log(w)) / w);
      s = c * v1; t = c * v2;
    } while ((fabs(s) <= 3.0) && (fabs(t) <= 3.0));
    x = (fabs(s) > 3.0) ? s : t;
  }
  return x;
}

/* FFTGrid::fillInComplexNoise (src/fftgrid.cpp:1191-1241), including its   */
/* parity test on the flat index for the last x column.                     */
void or_fill_complex_noise(float *cbuf, int nxp, int nyp, int nzp, unsigned int *seed)
{
  int cnxp = nxp / 2 + 1;
  long csize = (long)cnxp * nyp * nzp;
  float sd = (float)(1 / sqrt(2.0));
  for (long i = 0; i < csize; i++) {
    float *v = cbuf + 2 * i;
    if (((i % cnxp) == 0) || (((i % cnxp) == cnxp - 1) && ((i % 2) == 1))) {
      long xshift = i % cnxp;
      long jkind = (i - xshift) / cnxp;
      long jind = jkind % nyp;
      long kind = jkind / nyp;
      long jccind = (jind == 0) ? 0 : nyp - jind;
      long kccind = (kind == 0) ? 0 : nzp - kind;
      long jkccind = jccind + kccind * nyp;
      if (jkccind == jkind) {
        v[0] = (float)or_rnorm01(seed);
        v[1] = 0;
      } else if (jkccind > jkind) {
        v[0] = (float)(sd * or_rnorm01(seed));
        v[1] = (float)(sd * or_rnorm01(seed));
      } else {
        long cci = jkccind * cnxp + xshift;
        v[0] = cbuf[2 * cci];
        v[1] = -cbuf[2 * cci + 1];
      }
    } else {
      v[0] = (float)(sd * or_rnorm01(seed));
      v[1] = (float)(sd * or_rnorm01(seed));
    }
  }
}

/* FFTGrid::findClosestFactorableNumber (src/fftgrid.cpp:2857-2885):       */
/* smallest 2^a 3^b 5^c 7^d >= leastint (11 and 13 are disabled).           */
int or_find_closest_factorable(int leastint)
{
  int m2 = (int)ceil((double)logf((float)leastint) / (double)logf(2.0f));
  int m3 = (int)ceil((double)logf((float)leastint) / (double)logf(3.0f));
  int m5 = (int)ceil((double)logf((float)leastint) / (double)logf(5.0f));
  int m7 = (int)ceil((double)logf((float)leastint) / (double)logf(7.0f));
  int best = (int)pow(2.0f, m2);
  for (int i = 0; i < m2 + 1; i++)
    for (int j = 0; j < m3 + 1; j++)
      for (int k = 0; k < m5 + 1; k++)
        for (int l = 0; l < m7 + 1; l++) {
          int f = (int)(pow(2.0f, i) * pow(3.0f, j) * pow(5.0f, k) * pow(7.0f, l));
          if (f >= leastint && f < best) best = f;
        }
  return best;
}
