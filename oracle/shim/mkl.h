/*
 * MKL CBLAS stand-in used ONLY to compile the reference program as a CPU
 * checker.  The reference links MKL (UVaTRMM/Makefile:20) and calls
 * cblas_dgemm / cblas_dtrmm (UVaTRMM/src/mm_triangular.c:347, :374).  Here
 * those names resolve to the CBLAS entry points of the OpenBLAS build that
 * scipy bundles (exported with a `scipy_` prefix, LP64 ints).
 *
 * Enum values are the CBLAS standard ones (RowMajor=101 ... Right=142).
 */
#ifndef UVATRMM_ORACLE_MKL_SHIM_H
#define UVATRMM_ORACLE_MKL_SHIM_H

typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef enum { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;

void scipy_cblas_dgemm(CBLAS_LAYOUT, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, int, int, int, double,
                       const double *, int, const double *, int, double, double *, int);
void scipy_cblas_dtrmm(CBLAS_LAYOUT, CBLAS_SIDE, CBLAS_UPLO, CBLAS_TRANSPOSE, CBLAS_DIAG, int, int,
                       double, const double *, int, double *, int);

#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dtrmm scipy_cblas_dtrmm

#endif
