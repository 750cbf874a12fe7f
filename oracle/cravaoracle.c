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
 *   - Crava::correctAlphaBetaRho / newPosteriorCovPointwise
 *                                              src/crava.cpp:2345-2569
 *   - the non-constant-thickness data scaling and trace interpolation
 *     (oracle_impl.inc)                        src/crava.cpp:678-968,
 *                                              src/fftgrid.cpp:2576-2738
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

/* ------------------------------------------------------------------------ */
/* Local-noise correction: Crava::correctAlphaBetaRho (src/crava.cpp:       */
/* 2471-2569) and newPosteriorCovPointwise (:2345-2451), double precision.   */
/* The reference takes eigen-decompositions through NRLib::                 */
/* ComputeEigenVectors (LAPACK); every use here is V f(L) V^T, which does    */
/* not depend on eigenvector signs, so a largest-pivot Jacobi restates it.   */
/* G (Crava::computeG, :2261-2343) is an input: it does depend on signs.     */
/* ------------------------------------------------------------------------ */

/* eigen-decomposition of a symmetric n x n matrix a (destroyed; eigenvalues on
   the diagonal), eigenvectors in the columns of v; rotates the largest
   off-diagonal entry each step */
static void or_sym_eig(double *a, double *v, int n)
{
  for (int i = 0; i < n * n; i++) v[i] = 0.0;
  for (int i = 0; i < n; i++) v[i * n + i] = 1.0;
  for (int it = 0; it < 100 * n * n; it++) {
    int p = 0, q = 1;
    double best = -1.0, scale = 0.0;
    for (int i = 0; i < n; i++) {
      scale += fabs(a[i * n + i]);
      for (int j = i + 1; j < n; j++)
        if (fabs(a[i * n + j]) > best) { best = fabs(a[i * n + j]); p = i; q = j; }
    }
    if (n < 2 || best <= 1e-18 * scale || best == 0.0) break;
    double phi = 0.5 * atan2(2.0 * a[p * n + q], a[q * n + q] - a[p * n + p]);
    double c = cos(phi), s = sin(phi);
    for (int k = 0; k < n; k++) {
      double akp = a[k * n + p], akq = a[k * n + q];
      a[k * n + p] = c * akp - s * akq;
      a[k * n + q] = s * akp + c * akq;
    }
    for (int k = 0; k < n; k++) {
      double apk = a[p * n + k], aqk = a[q * n + k];
      a[p * n + k] = c * apk - s * aqk;
      a[q * n + k] = s * apk + c * aqk;
    }
    for (int k = 0; k < n; k++) {
      double vkp = v[k * n + p], vkq = v[k * n + q];
      v[k * n + p] = c * vkp - s * vkq;
      v[k * n + q] = s * vkp + c * vkq;
    }
  }
}

/* out = V diag(f(l)) V^T for symmetric m (n x n): mode 0 sqrt(l > 0), 1 1/sqrt(l > thr), 2 1/l (l > thr) */
static void or_sym_fun(const double *m, double *out, int n, int mode, double thr)
{
  double a[64], v[64], f[8];
  for (int i = 0; i < n * n; i++) a[i] = m[i];
  or_sym_eig(a, v, n);
  for (int i = 0; i < n; i++) {
    double l = a[i * n + i];
    if (mode == 0) f[i] = l > 0.0 ? sqrt(l) : 0.0;
    else if (mode == 1) f[i] = l > thr ? 1.0 / sqrt(l) : 0.0;
    else f[i] = l > thr ? 1.0 / l : 0.0;
  }
  for (int r = 0; r < n; r++)
    for (int c = 0; c < n; c++) {
      double s = 0.0;
      for (int k = 0; k < n; k++) s += v[r * n + k] * f[k] * v[c * n + k];
      out[r * n + c] = s;
    }
}

/* C (n1 x n3) = A (n1 x n2) B (n2 x n3), row-major */
static void or_mm(const double *A, const double *B, int n1, int n2, int n3, double *C)
{
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n3; j++) {
      double s = 0.0;
      for (int k = 0; k < n2; k++) s += A[i * n2 + k] * B[k * n3 + j];
      C[i * n3 + j] = s;
    }
}

/* newPosteriorCovPointwise: sigmanew (3x3) and sigmamdnew (3x3) of one trace */
void or_new_posterior_cov_pointwise(int n, const double *G, const double *etc, const double *sm, const double *smd,
                                    const double *scales, double *sigmanew, double *sigmamdnew)
{
  double D[8], help[64], GT[24], H1[24], GSG[64], hinv[64], H4[24], H2[24], H3[9], delta[9], tmp[9], dsq[9];
  double sdelta[9], sdinv[9];
  for (int l = 0; l < n; l++) D[l] = sqrt(scales[l]);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < 3; j++) GT[j * n + i] = G[i * 3 + j];
  or_mm(G, sm, n, 3, 3, H1);                /* H1 = G Sm */
  or_mm(H1, GT, n, 3, n, GSG);              /* G Sm G^T */
  for (int l = 0; l < n; l++)
    for (int m = 0; m < n; m++) help[l * n + m] = GSG[l * n + m] + D[l] * etc[l * n + m] * D[m];
  or_sym_fun(help, hinv, n, 2, 0.00000001);  /* (G Sm G^T + D Se D)^+ */
  or_mm(sm, GT, 3, 3, n, H4);               /* Sm G^T */
  or_mm(H4, hinv, 3, n, n, H2);
  or_mm(H2, G, 3, n, 3, H3);
  or_mm(H3, sm, 3, 3, 3, delta);            /* Sm G^T H^+ G Sm */
  for (int i = 0; i < 9; i++) tmp[i] = sm[i] - delta[i];
  or_sym_fun(tmp, sigmamdnew, 3, 0, 0.0);   /* sqrt(local posterior covariance) */
  or_sym_fun(delta, dsq, 3, 0, 0.0);
  for (int i = 0; i < 9; i++) sdelta[i] = sm[i] - smd[i];
  or_sym_fun(sdelta, sdinv, 3, 1, 0.0000001);
  or_mm(dsq, sdinv, 3, 3, 3, sigmanew);
}

/* correctAlphaBetaRho on 3 real padded posterior-mean cubes (in place). scale: [n][ny][nx] local noise
   scales (Grid2D<double>, divided here by each grid's minimum over non-RMISSING values). sigmamd (may be
   NULL): [ny][nx][9] sigmamdx * postVar0^-1/2 (Crava::sigmamdnew_). */
void or_correct_alpha_beta_rho(float **post, float **mean, int nx, int ny, int nz, int nxp, int nyp, int n,
                               const double *G, const double *etc, const double *sm, const double *smd,
                               const double *scale, double *sigmamd)
{
  const int rnxp = 2 * (nxp / 2 + 1);
  double minScale[8], sold[9], sigmanew[9], sigmamdnew[9], scales[8];
  for (int l = 0; l < n; l++) {
    const double *g = scale + (size_t)l * nx * ny;
    double m = g[0];
    for (int t = 0; t < nx * ny; t++)
      if ((m == (double)OR_RMISSING || g[t] < m) && g[t] != (double)OR_RMISSING) m = g[t];
    minScale[l] = m;
  }
  or_sym_fun(smd, sold, 3, 1, 0.0);  /* lib_matr_eigen: eigval > 0 -> 1/sqrt */
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      for (int l = 0; l < n; l++) {
        /* a missing scale gives NaN in the reference; here it counts as the minimum */
        double sv = scale[((size_t)l * ny + j) * nx + i];
        scales[l] = sv == (double)OR_RMISSING ? 1.0 : sv / minScale[l];
      }
      or_new_posterior_cov_pointwise(n, G, etc, sm, smd, scales, sigmanew, sigmamdnew);
      if (sigmamd) or_mm(sigmamdnew, sold, 3, 3, 3, sigmamd + ((size_t)j * nx + i) * 9);
      for (int k = 0; k < nz; k++) {
        size_t o = ((size_t)k * nyp + j) * rnxp + i;
        float ad = post[0][o] - mean[0][o], bd = post[1][o] - mean[1][o], rd = post[2][o] - mean[2][o];
        float an = (float)(mean[0][o] + sigmanew[0] * ad + sigmanew[1] * bd + sigmanew[2] * rd);
        float bn = (float)(mean[1][o] + sigmanew[3] * ad + sigmanew[4] * bd + sigmanew[5] * rd);
        float rn = (float)(mean[2][o] + sigmanew[6] * ad + sigmanew[7] * bd + sigmanew[8] * rd);
        post[0][o] = an; post[1][o] = bn; post[2][o] = rn;
      }
    }
}
