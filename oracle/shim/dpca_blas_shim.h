/*
 * BLAS/LAPACK declarations for the CPU oracle (test infrastructure only).
 *
 * The oracle links the OpenBLAS build that ships inside the scipy wheel
 * (LP64, every exported symbol carries a "scipy_" prefix), or, where scipy
 * carries none, the ILP64 one inside the numpy wheel (DPCA_ORACLE_ILP64).  This header maps
 * the unprefixed CBLAS/LAPACKE names that the reference sources and the C
 * restatement call onto those exports, and supplies the few MKL service
 * calls the reference uses on x86 (dsecnd, mkl_set_num_threads,
 * mkl_dimatcopy).
 */
#ifndef DPCA_ORACLE_BLAS_SHIM_H
#define DPCA_ORACLE_BLAS_SHIM_H

#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifdef DPCA_ORACLE_ILP64
/* numpy's bundled OpenBLAS: 64-bit integers, names suffixed "64_" */
typedef long long lapack_int;
typedef long long blas_int;
#define DPCA_SCIPY(name) scipy_##name##64_
#else
typedef int lapack_int;
typedef int blas_int;
#define DPCA_SCIPY(name) scipy_##name
#endif

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

void DPCA_SCIPY(cblas_dgemm)(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE, blas_int m, blas_int n,
                             blas_int k, double alpha, const double *a, blas_int lda, const double *b, blas_int ldb,
                             double beta, double *c, blas_int ldc);
lapack_int DPCA_SCIPY(LAPACKE_dgeqrf)(int layout, lapack_int m, lapack_int n, double *a, lapack_int lda, double *tau);
lapack_int DPCA_SCIPY(LAPACKE_dorgqr)(int layout, lapack_int m, lapack_int n, lapack_int k, double *a,
                                      lapack_int lda, const double *tau);
lapack_int DPCA_SCIPY(LAPACKE_dsyev)(int layout, char jobz, char uplo, lapack_int n, double *a, lapack_int lda,
                                     double *w);
lapack_int DPCA_SCIPY(LAPACKE_dgesvd)(int layout, char jobu, char jobvt, lapack_int m, lapack_int n, double *a,
                                      lapack_int lda, double *s, double *u, lapack_int ldu, double *vt,
                                      lapack_int ldvt, double *superb);
void DPCA_SCIPY(openblas_set_num_threads)(int);

#define cblas_dgemm DPCA_SCIPY(cblas_dgemm)
#define LAPACKE_dgeqrf DPCA_SCIPY(LAPACKE_dgeqrf)
#define LAPACKE_dorgqr DPCA_SCIPY(LAPACKE_dorgqr)
#define LAPACKE_dsyev DPCA_SCIPY(LAPACKE_dsyev)
#define LAPACKE_dgesvd DPCA_SCIPY(LAPACKE_dgesvd)
#define scipy_openblas_set_num_threads DPCA_SCIPY(openblas_set_num_threads)

#ifdef __cplusplus
}
#endif

#endif
