/* Enumerations of the C interface to the BLAS, enough for the reference's
 * flens headers to compile (their blas.h includes <cblas.h>).  The O2
 * harness does not compile flens's BLAS wrappers (blas.cc, lapack.cc), so no
 * BLAS routine is declared or linked here. */
#ifndef CRAVA_O2_CBLAS_SHIM_H
#define CRAVA_O2_CBLAS_SHIM_H
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 };
#endif
