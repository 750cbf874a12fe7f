/*
 * Reference harness (test infrastructure only).
 *
 * Built by Makefile.ref into oracle/_ref/libcrava_ref.so together with the
 * reference's own, unmodified sources: the vendored FFTW 2.1.2 (float,
 * libs/fft/{fftw,rfftw}), libs/lib/lib_matr.c and libs/lib/random.cpp.  The
 * reference's Crava/FFTGrid classes need BLAS/LAPACK, flens and most of nrlib,
 * so they are not built; the glue below re-states their loops
 * (src/fftgrid.cpp:1783-1842, src/crava.cpp:1084-1247 and :1617-1656,
 * src/fftgrid.cpp:1191-1241) and hands every transform and every small
 * complex matrix operation to the reference's compiled code.  Its outputs are
 * what the C restatement in cravaoracle.c is pinned against, and what the
 * golden fixtures under tests/golden are generated from.
 */
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <string>

#include "fftw.h"
#include "rfftw.h"
#include "lib/lib_matr.h"
#include "lib/random.h"

/* RandomGen(const std::string&) reads a seed file through NRLib::OpenRead;
 * the harness only uses the integer-seed constructor, so this symbol exists
 * solely to satisfy the linker. */
namespace NRLib {
void OpenRead(std::ifstream &stream, const std::string &filename, std::ios_base::openmode mode)
{
  stream.open(filename.c_str(), mode);
}
}  // namespace NRLib

namespace {
const int kCovariance = 3;
const int kOperator = 5;

fftw_complex **alloc_cpx(int m, int n)
{
  fftw_complex **c = new fftw_complex *[m];
  for (int i = 0; i < m; i++) c[i] = new fftw_complex[n];
  return c;
}
void free_cpx(fftw_complex **c, int m)
{
  for (int i = 0; i < m; i++) delete[] c[i];
  delete[] c;
}
}  // namespace

extern "C" {

/* FFTGrid::fftInPlace, src/fftgrid.cpp:1783-1809 */
void ref_fft3d_r2c(float *buf, int nxp, int nyp, int nzp, int cubetype)
{
  int rsize = 2 * (nxp / 2 + 1) * nyp * nzp;
  if (cubetype != kCovariance && cubetype != kOperator) {
    float s = 1.0f / sqrt(static_cast<float>(nxp * nyp * nzp));
    for (int i = 0; i < rsize; i++) buf[i] *= s;
  }
  rfftwnd_plan plan = rfftw3d_create_plan(nzp, nyp, nxp, FFTW_REAL_TO_COMPLEX, FFTW_ESTIMATE | FFTW_IN_PLACE);
  rfftwnd_one_real_to_complex(plan, buf, reinterpret_cast<fftw_complex *>(buf));
  fftwnd_destroy_plan(plan);
}

/* FFTGrid::invFFTInPlace, src/fftgrid.cpp:1811-1842 */
void ref_fft3d_c2r(float *buf, int nxp, int nyp, int nzp, int cubetype)
{
  int rsize = 2 * (nxp / 2 + 1) * nyp * nzp;
  float scale;
  if (cubetype == kCovariance || cubetype == kOperator)
    scale = float(1.0 / (nxp * nyp * nzp));
  else
    scale = float(1.0 / sqrt(float(nxp * nyp * nzp)));
  rfftwnd_plan plan = rfftw3d_create_plan(nzp, nyp, nxp, FFTW_COMPLEX_TO_REAL, FFTW_ESTIMATE | FFTW_IN_PLACE);
  rfftwnd_one_complex_to_real(plan, reinterpret_cast<fftw_complex *>(buf), buf);
  fftwnd_destroy_plan(plan);
  for (int i = 0; i < rsize; i++) buf[i] *= scale;
}

/* 1D real transform in place (Wavelet::fft1DInPlace, src/wavelet.cpp:246-261) */
void ref_fft1d_r2c(float *buf, int n)
{
  rfftwnd_plan plan = rfftwnd_create_plan(1, &n, FFTW_REAL_TO_COMPLEX, FFTW_ESTIMATE | FFTW_IN_PLACE);
  rfftwnd_one_real_to_complex(plan, buf, reinterpret_cast<fftw_complex *>(buf));
  fftwnd_destroy_plan(plan);
}

/* lib_matrCholCpx on one row-major n x n matrix (lower triangle returned) */
int ref_chol_cpx(int n, float *a)
{
  fftw_complex **m = alloc_cpx(n, n);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) { m[i][j].re = a[2 * (i * n + j)]; m[i][j].im = a[2 * (i * n + j) + 1]; }
  int flag = lib_matrCholCpx(n, m);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) { a[2 * (i * n + j)] = m[i][j].re; a[2 * (i * n + j) + 1] = m[i][j].im; }
  free_cpx(m, n);
  return flag;
}

/*
 * Bin loop of Crava::computePostMeanResidAndFFTCov (src/crava.cpp:1084-1247)
 * with findParameterVariances (src/seismicparametersholder.cpp:357-428),
 * getNextErrorVariance (src/crava.cpp:1442-1469) and invertSeismicData
 * (src/crava.cpp:1389-1438).  Matrix work is the reference's lib_matr.
 */
int ref_invert_bins(int nxp, int nyp, int nzp, int ntheta,
                    float **data, float **mean, float **cov, const float *errcorr,
                    const float *Ktab, const float *em1, const float *em2, const float *em3,
                    const unsigned char *band, const double *errThetaCov,
                    const double *sigma0, float wnc, int is4d, int nthreads)
{
  int cnxp = nxp / 2 + 1;
  int n = ntheta;
  int failed = 0;
  double **etc = new double *[n];
  for (int l = 0; l < n; l++) {
    etc[l] = new double[n];
    for (int m = 0; m < n; m++) etc[l][m] = errThetaCov[l * n + m];
  }
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+:failed)
  for (int k = 0; k < nzp; k++) {
    fftw_complex *errMult1 = new fftw_complex[n];
    fftw_complex *errMult2 = new fftw_complex[n];
    fftw_complex *errMult3 = new fftw_complex[n];
    fftw_complex *ijkData = new fftw_complex[n];
    fftw_complex *ijkDataMean = new fftw_complex[n];
    fftw_complex *ijkRes = new fftw_complex[n];
    fftw_complex *ijkMean = new fftw_complex[3];
    fftw_complex *ijkAns = new fftw_complex[3];
    fftw_complex **K = alloc_cpx(n, 3);
    fftw_complex **KS = alloc_cpx(n, 3);
    fftw_complex **KScc = alloc_cpx(3, n);
    fftw_complex **parVar = alloc_cpx(3, 3);
    fftw_complex **reduceVar = alloc_cpx(3, 3);
    fftw_complex **margVar = alloc_cpx(n, n);
    fftw_complex **errVar = alloc_cpx(n, n);
    for (int l = 0; l < n; l++) {
      for (int p = 0; p < 3; p++) {
        K[l][p].re = Ktab[2 * ((k * n + l) * 3 + p)];
        K[l][p].im = Ktab[2 * ((k * n + l) * 3 + p) + 1];
      }
      errMult1[l].re = em1[2 * (k * n + l)]; errMult1[l].im = em1[2 * (k * n + l) + 1];
      errMult2[l].re = em2[2 * (k * n + l)]; errMult2[l].im = em2[2 * (k * n + l) + 1];
      errMult3[l].re = em3[2 * (k * n + l)]; errMult3[l].im = em3[2 * (k * n + l) + 1];
    }
    for (int j = 0; j < nyp; j++) {
      for (int i = 0; i < cnxp; i++) {
        long b = i + (long)cnxp * j + (long)cnxp * nyp * k;
        for (int p = 0; p < 3; p++) { ijkMean[p].re = mean[p][2 * b]; ijkMean[p].im = mean[p][2 * b + 1]; }
        for (int l = 0; l < n; l++) {
          ijkData[l].re = data[l][2 * b]; ijkData[l].im = data[l][2 * b + 1];
          ijkRes[l] = ijkData[l];
        }
        fftw_complex ijkErrCorr;
        ijkErrCorr.re = errcorr[2 * b]; ijkErrCorr.im = errcorr[2 * b + 1];
        fftw_complex c[6];
        for (int t = 0; t < 6; t++) { c[t].re = cov[t][2 * b]; c[t].im = cov[t][2 * b + 1]; }
        /* findParameterVariances */
        fftw_complex ii = c[0], jj = c[1], kk = c[2], ij = c[3], ik = c[4], jk = c[5];
        if (is4d) {
          ii.re = sqrt(ii.re * ii.re + ii.im * ii.im); ii.im = 0.0f;
          jj.re = sqrt(jj.re * jj.re + jj.im * jj.im); jj.im = 0.0f;
          kk.re = sqrt(kk.re * kk.re + kk.im * kk.im); kk.im = 0.0f;
        } else {
          fftw_complex *v[6] = {&ii, &jj, &kk, &ij, &ik, &jk};
          int pq[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
          for (int t = 0; t < 6; t++) {
            double s = sigma0[pq[t][0] * 3 + pq[t][1]];
            fftw_complex cv = *v[t];
            if (s != 0) cv.re = cv.re / static_cast<float>(s);
            fftw_complex o;
            o.re = float(sqrt(cv.re * cv.re)) * static_cast<float>(s);
            o.im = 0.0f;
            *v[t] = o;
          }
        }
        parVar[0][0] = ii; parVar[1][1] = jj; parVar[2][2] = kk;
        parVar[0][1] = ij; parVar[1][0].re = ij.re; parVar[1][0].im = -ij.im;
        parVar[0][2] = ik; parVar[2][0].re = ik.re; parVar[2][0].im = -ik.im;
        parVar[1][2] = jk; parVar[2][1].re = jk.re; parVar[2][1].im = -jk.im;
        if (band[k]) {
          fftw_complex lam;
          lam.re = static_cast<float>(sqrt(ijkErrCorr.re * ijkErrCorr.re));
          lam.im = 0.0;
          for (int l = 0; l < n; l++)
            for (int m = 0; m < n; m++) {
              errVar[l][m].re = static_cast<float>(0.5 * (1.0 - wnc) * etc[l][m] * lam.re * (errMult1[l].re * errMult1[m].re + errMult1[l].im * errMult1[m].im));
              errVar[l][m].re += static_cast<float>(0.5 * (1.0 - wnc) * etc[l][m] * lam.re * (errMult2[l].re * errMult2[m].re + errMult2[l].im * errMult2[m].im));
              if (l == m) {
                errVar[l][m].re += static_cast<float>(wnc * etc[l][m] * errMult3[l].re * errMult3[l].re);
                errVar[l][m].im = 0.0;
              } else {
                errVar[l][m].im = static_cast<float>(0.5 * (1.0 - wnc) * etc[l][m] * lam.re * (-errMult1[l].re * errMult1[m].im + errMult1[l].im * errMult1[m].re));
                errVar[l][m].im += static_cast<float>(0.5 * (1.0 - wnc) * etc[l][m] * lam.re * (-errMult2[l].re * errMult2[m].im + errMult2[l].im * errMult2[m].re));
              }
            }
          lib_matrProdCpx(K, parVar, n, 3, 3, KS);
          lib_matrProdAdjointCpx(KS, K, n, 3, n, margVar);
          lib_matrAddMatCpx(errVar, n, n, margVar);
          int cholFlag = lib_matrCholCpx(n, margVar);
          if (cholFlag == 0) {
            lib_matrAdjoint(KS, n, 3, KScc);
            lib_matrAXeqBMatCpx(n, margVar, KS, 3);
            lib_matrProdCpx(KScc, KS, 3, n, 3, reduceVar);
            lib_matrSubtMatCpx(reduceVar, 3, 3, parVar);
            lib_matrProdMatVecCpx(K, ijkMean, n, 3, ijkDataMean);
            lib_matrSubtVecCpx(ijkDataMean, n, ijkData);
            lib_matrProdAdjointMatVecCpx(KS, ijkData, 3, n, ijkAns);
            lib_matrAddVecCpx(ijkAns, 3, ijkMean);
            lib_matrProdMatVecCpx(K, ijkMean, n, 3, ijkData);
            lib_matrSubtVecCpx(ijkData, n, ijkRes);
          } else {
            failed++;
          }
        }
        for (int l = 0; l < n; l++) { data[l][2 * b] = ijkRes[l].re; data[l][2 * b + 1] = ijkRes[l].im; }
        for (int p = 0; p < 3; p++) { mean[p][2 * b] = ijkMean[p].re; mean[p][2 * b + 1] = ijkMean[p].im; }
        fftw_complex out6[6] = {parVar[0][0], parVar[1][1], parVar[2][2], parVar[0][1], parVar[0][2], parVar[1][2]};
        for (int t = 0; t < 6; t++) { cov[t][2 * b] = out6[t].re; cov[t][2 * b + 1] = out6[t].im; }
      }
    }
    delete[] errMult1; delete[] errMult2; delete[] errMult3;
    delete[] ijkData; delete[] ijkDataMean; delete[] ijkRes; delete[] ijkMean; delete[] ijkAns;
    free_cpx(K, n); free_cpx(KS, n); free_cpx(KScc, 3); free_cpx(parVar, 3);
    free_cpx(reduceVar, 3); free_cpx(margVar, n); free_cpx(errVar, n);
  }
  for (int l = 0; l < n; l++) delete[] etc[l];
  delete[] etc;
  return failed;
}

/* Crava::simulate bin loop, src/crava.cpp:1617-1656 */
void ref_simulate_bins(long csize, float **cov, float **seed)
{
  fftw_complex **P = alloc_cpx(3, 3);
  fftw_complex s[3];
  for (long b = 0; b < csize; b++) {
    P[0][0].re = cov[0][2 * b]; P[0][0].im = cov[0][2 * b + 1];
    P[1][1].re = cov[1][2 * b]; P[1][1].im = cov[1][2 * b + 1];
    P[2][2].re = cov[2][2 * b]; P[2][2].im = cov[2][2 * b + 1];
    P[0][1].re = cov[3][2 * b]; P[0][1].im = cov[3][2 * b + 1];
    P[0][2].re = cov[4][2 * b]; P[0][2].im = cov[4][2 * b + 1];
    P[1][2].re = cov[5][2 * b]; P[1][2].im = cov[5][2 * b + 1];
    P[1][0].re = P[0][1].re; P[1][0].im = -P[0][1].im;
    P[2][0].re = P[0][2].re; P[2][0].im = -P[0][2].im;
    P[2][1].re = P[1][2].re; P[2][1].im = -P[1][2].im;
    for (int l = 0; l < 3; l++) { s[l].re = seed[l][2 * b]; s[l].im = seed[l][2 * b + 1]; }
    if (lib_matrCholCpx(3, P) == 0) {
      lib_matrProdCholVec(3, P, s);
    } else {
      for (int l = 0; l < 3; l++) { s[l].re = 0.0; s[l].im = 0.0; }
    }
    for (int l = 0; l < 3; l++) { seed[l][2 * b] = s[l].re; seed[l][2 * b + 1] = s[l].im; }
  }
  free_cpx(P, 3);
}

/* n draws of the reference RandomGen::rnorm01 starting from `seed` */
void ref_rnorm01_seq(unsigned int seed, int n, double *out)
{
  RandomGen gen(seed);
  for (int i = 0; i < n; i++) out[i] = gen.rnorm01();
}

/* FFTGrid::fillInComplexNoise loop (src/fftgrid.cpp:1191-1241) driven by the
 * reference RandomGen seeded with `seed`. */
void ref_fill_complex_noise(float *cbuf, int nxp, int nyp, int nzp, unsigned int seed, int ncubes)
{
  RandomGen gen(seed);
  int cnxp = nxp / 2 + 1;
  long csize = (long)cnxp * nyp * nzp;
  float sd = float(1 / sqrt(2.0));
  for (int c = 0; c < ncubes; c++) {
    fftw_complex *cv = reinterpret_cast<fftw_complex *>(cbuf) + c * csize;
    for (long i = 0; i < csize; i++) {
      if (((i % cnxp) == 0) || (((i % cnxp) == cnxp - 1) && ((i % 2) == 1))) {
        long xshift = i % cnxp;
        long jkind = (i - xshift) / cnxp;
        long jind = jkind % nyp;
        long kind = jkind / nyp;
        long jccind = (jind == 0) ? 0 : nyp - jind;
        long kccind = (kind == 0) ? 0 : nzp - kind;
        long jkccind = jccind + kccind * nyp;
        if (jkccind == jkind) {
          cv[i].re = float(gen.rnorm01());
          cv[i].im = 0;
        } else if (jkccind > jkind) {
          cv[i].re = float(sd * gen.rnorm01());
          cv[i].im = float(sd * gen.rnorm01());
        } else {
          long cci = jkccind * cnxp + xshift;
          cv[i].re = cv[cci].re;
          cv[i].im = -cv[cci].im;
        }
      } else {
        cv[i].re = float(sd * gen.rnorm01());
        cv[i].im = float(sd * gen.rnorm01());
      }
    }
  }
}

}  // extern "C"
