/*
 * MKL service calls for building the reference as a CPU oracle on x86
 * (test infrastructure only).  Dense math goes to scipy's OpenBLAS through
 * dpca_blas_shim.h.
 */
#ifndef DPCA_ORACLE_SHIM_MKL_H
#define DPCA_ORACLE_SHIM_MKL_H

#include "dpca_blas_shim.h"

/* Wall-clock seconds, as MKL's dsecnd() is used by the reference's timers. */
static inline double dsecnd(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static inline void mkl_set_num_threads(int n) { scipy_openblas_set_num_threads(n); }

/* In-place out-of-place-buffered transpose for ordering 'R', trans 'T':
 * AB (rows x cols, leading dim lda) becomes cols x rows with leading dim ldb. */
static inline void mkl_dimatcopy(char, char, size_t rows, size_t cols, double alpha, double *ab, size_t lda,
                                 size_t ldb) {
    double *t = (double *)malloc(rows * cols * sizeof(double));
    for (size_t i = 0; i < rows; ++i)
        for (size_t j = 0; j < cols; ++j) t[j * ldb + i] = alpha * ab[i * lda + j];
    memcpy(ab, t, rows * cols * sizeof(double));
    free(t);
}

#endif
