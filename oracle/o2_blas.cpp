// The BLAS / LAPACK entry points of the reference's flens layer that the O2
// harness's reference code reaches, bound to the OpenBLAS that ships inside
// scipy (its symbols carry a scipy_ prefix) -- TEST INFRASTRUCTURE ONLY.
// The reference's own wrappers (libs/flens/blas.cc, lapack.cc) need a full
// system CBLAS/LAPACK, which this machine does not have; these restate the
// same one-line mappings (storage order, transposition, side and triangle
// flags to their BLAS/LAPACK characters or enumerations) from the public
// BLAS/LAPACK calling conventions.
#include <complex>

#include "flens/flens.h"

extern "C" {
// CBLAS (the enumerations come from the shim cblas.h the flens headers include)
void scipy_cblas_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy);
void scipy_cblas_dcopy(int n, const double *x, int incx, double *y, int incy);
double scipy_cblas_ddot(int n, const double *x, int incx, const double *y, int incy);
void scipy_cblas_dscal(int n, double alpha, double *x, int incx);
void scipy_cblas_dgemm(CBLAS_ORDER o, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n, int k, double alpha,
                       const double *a, int lda, const double *b, int ldb, double beta, double *c, int ldc);
void scipy_cblas_dgemv(CBLAS_ORDER o, CBLAS_TRANSPOSE t, int m, int n, double alpha, const double *a, int lda,
                       const double *x, int incx, double beta, double *y, int incy);
void scipy_cblas_dsymm(CBLAS_ORDER o, CBLAS_SIDE s, CBLAS_UPLO u, int m, int n, double alpha, const double *a,
                       int lda, const double *b, int ldb, double beta, double *c, int ldc);
// LAPACK (Fortran calling convention)
void scipy_dgeev_(const char *jobvl, const char *jobvr, const int *n, double *a, const int *lda, double *wr,
                  double *wi, double *vl, const int *ldvl, double *vr, const int *ldvr, double *work,
                  const int *lwork, int *info);
void scipy_dgetrf_(const int *m, const int *n, double *a, const int *lda, int *ipiv, int *info);
void scipy_dgetri_(const int *n, double *a, const int *lda, const int *ipiv, double *work, const int *lwork,
                   int *info);
void scipy_dposv_(const char *uplo, const int *n, const int *nrhs, double *a, const int *lda, double *b,
                  const int *ldb, int *info);
void scipy_zposv_(const char *uplo, const int *n, const int *nrhs, std::complex<double> *a, const int *lda,
                  std::complex<double> *b, const int *ldb, int *info);
void scipy_dpotrf_(const char *uplo, const int *n, double *a, const int *lda, int *info);
void scipy_dpotri_(const char *uplo, const int *n, double *a, const int *lda, int *info);
void scipy_dsyev_(const char *jobz, const char *uplo, const int *n, double *a, const int *lda, double *w,
                  double *work, const int *lwork, int *info);
}

namespace {
CBLAS_ORDER order_of(flens::StorageOrder o) { return o == flens::RowMajor ? CblasRowMajor : CblasColMajor; }
CBLAS_TRANSPOSE trans_of(flens::Transpose t) { return t == flens::NoTrans ? CblasNoTrans : CblasTrans; }
char uplo_of(flens::StorageUpLo u) { return u == flens::Upper ? 'U' : 'L'; }
}  // namespace

namespace flens {

void axpy(int n, double alpha, const double *x, int incx, double *y, int incy)
{
  scipy_cblas_daxpy(n, alpha, x, incx, y, incy);
}

void copy(int n, const double *x, int incx, double *y, int incy) { scipy_cblas_dcopy(n, x, incx, y, incy); }

double dot(int n, const double *x, int incx, const double *y, int incy)
{
  return scipy_cblas_ddot(n, x, incx, y, incy);
}

void scal(int n, double alpha, double *x, int incx) { scipy_cblas_dscal(n, alpha, x, incx); }

void gemm(StorageOrder o, Transpose ta, Transpose tb, int m, int n, int k, double alpha, const double *a, int lda,
          const double *b, int ldb, double beta, double *c, const int ldc)
{
  scipy_cblas_dgemm(order_of(o), trans_of(ta), trans_of(tb), m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

void gemv(StorageOrder o, Transpose t, int m, int n, double alpha, const double *a, int lda, const double *x,
          int incx, double beta, double *y, int incy)
{
  scipy_cblas_dgemv(order_of(o), trans_of(t), m, n, alpha, a, lda, x, incx, beta, y, incy);
}

void symm(StorageOrder o, BlasSide s, StorageUpLo u, int m, int n, double alpha, const double *a, const int lda,
          const double *b, const int ldb, const double beta, double *c, const int ldc)
{
  scipy_cblas_dsymm(order_of(o), s == Left ? CblasLeft : CblasRight, u == Upper ? CblasUpper : CblasLower, m, n,
                    alpha, a, lda, b, ldb, beta, c, ldc);
}

int geev(bool jobvl, bool jobvr, int n, double *a, int lda, double *wr, double *wi, double *vl, int ldvl, double *vr,
         int ldvr, double *work, int lwork)
{
  int info;
  const char jl = jobvl ? 'V' : 'N', jr = jobvr ? 'V' : 'N';
  scipy_dgeev_(&jl, &jr, &n, a, &lda, wr, wi, vl, &ldvl, vr, &ldvr, work, &lwork, &info);
  return info;
}

int getrf(int m, int n, double *a, int lda, int *ipiv)
{
  int info;
  scipy_dgetrf_(&m, &n, a, &lda, ipiv, &info);
  return info;
}

int getri(int n, double *a, int lda, const int *ipiv, double *work, int lwork)
{
  int info;
  scipy_dgetri_(&n, a, &lda, ipiv, work, &lwork, &info);
  return info;
}

int posv(StorageUpLo u, int n, int nrhs, double *a, int lda, double *b, int ldb)
{
  int info;
  const char c = uplo_of(u);
  scipy_dposv_(&c, &n, &nrhs, a, &lda, b, &ldb, &info);
  return info;
}

int posv(StorageUpLo u, int n, int nrhs, std::complex<double> *a, int lda, std::complex<double> *b, int ldb)
{
  int info;
  const char c = uplo_of(u);
  scipy_zposv_(&c, &n, &nrhs, a, &lda, b, &ldb, &info);
  return info;
}

int potrf(StorageUpLo u, int n, double *a, int lda)
{
  int info;
  const char c = uplo_of(u);
  scipy_dpotrf_(&c, &n, a, &lda, &info);
  return info;
}

int potri(StorageUpLo u, int n, double *a, int lda)
{
  int info;
  const char c = uplo_of(u);
  scipy_dpotri_(&c, &n, a, &lda, &info);
  return info;
}

int syev(bool jobz, StorageUpLo u, int n, double *a, int lda, double *w, double *work, int lwork)
{
  int info;
  const char jz = jobz ? 'V' : 'N', c = uplo_of(u);
  scipy_dsyev_(&jz, &c, &n, a, &lda, w, work, &lwork, &info);
  return info;
}

}  // namespace flens
