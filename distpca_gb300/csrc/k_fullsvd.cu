// -fullSVD on the device: the dense SVD of the standardized matrix for the accuracy check
// (distpca.cpp:449-635).  The reference runs LAPACKE_dgesvd on the n_ind x n_snp matrix; here
// its left singular vectors and values come from the symmetric eigendecomposition of the FP64
// Gram matrix G = X^T X (n_ind x n_ind): sigma_j = sqrt(lambda_j), u_j = the eigenvector.  G is
// built 128 columns at a time by the plain FP64 pass kernels (Y = the decoded columns, then
// X^T Y); the eigensolve is cuSOLVER's dsyevd.  This is an off-path accuracy check, limited to
// n_ind <= 20,000.
#include <cusolverDn.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "dpca_internal.h"

namespace dpca {

// y[s][c] = standardized value of (SNP s, individual c0 + c), 0 past the last individual.
__global__ void decode_columns_kernel(const uint8_t *__restrict__ P, int64_t pitch, const double *__restrict__ lut,
                                      int n_ind, int n_snp, int c0, int cols, double *__restrict__ y) {
    const int64_t total = (int64_t)n_snp * cols;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = e / cols;
        const int c = (int)(e - s * cols), i = c0 + c;
        double v = 0.0;
        if (i < n_ind) {
            const uint32_t code = (P[s * pitch + (i >> 2)] >> (2 * (i & 3))) & 3u;
            v = lut[4 * s + code];
        }
        y[e] = v;
    }
}

// Leading nsv singular values and left singular vectors (host, row-major n_ind x nsv) of the
// resident FP64 handle h, which must have been created with nrhs = 128.
dpca_status full_svd_device(Handle *h, int nsv, double *sigma, double *u, int *info) {
    const int n = h->n_ind;
    if (h->k != 128 || h->streamed || h->precision != DPCA_PREC_FP64) {
        set_error("internal: full SVD needs a resident FP64 handle of width 128");
        return DPCA_ERR_INVALID;
    }
    double *G = nullptr, *W = nullptr, *work = nullptr;
    int *dinfo = nullptr;
    cusolverDnHandle_t sol = nullptr;
    dpca_status st = DPCA_OK;
    auto fail = [&](dpca_status s) {
        st = s;
        return s;
    };
    do {
        if (cudaMalloc(&G, (size_t)n * n * 8) != cudaSuccess || cudaMalloc(&W, (size_t)n * 8) != cudaSuccess ||
            cudaMalloc(&dinfo, sizeof(int)) != cudaSuccess) {
            set_error("full SVD: cannot allocate the %d x %d Gram matrix", n, n);
            fail(DPCA_ERR_NOMEM);
            break;
        }
        // G[:, c0:c0+128] = X^T (decoded columns c0..c0+127): Z (n x 128) copied into G's columns
        for (int c0 = 0; c0 < n && st == DPCA_OK; c0 += 128) {
            const int cols = std::min(128, n - c0);
            const int64_t total = (int64_t)h->n_snp * 128;
            const int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)h->sm_count * 16);
            decode_columns_kernel<<<grid, 256, 0, h->stream>>>(h->P, h->pitch, h->lut, n, h->n_snp, c0, 128, h->y);
            if (cudaGetLastError() != cudaSuccess) {
                set_error("full SVD: column decode launch failed");
                fail(DPCA_ERR_CUDA);
                break;
            }
            if ((st = launch_fp64_xty(h, h->y, h->z)) != DPCA_OK) break;
            if (cudaMemcpy2DAsync(G + c0, (size_t)n * 8, h->z, 128 * 8, (size_t)cols * 8, n, cudaMemcpyDeviceToDevice,
                                  h->stream) != cudaSuccess) {
                set_error("full SVD: Gram copy failed");
                fail(DPCA_ERR_CUDA);
            }
        }
        if (st != DPCA_OK) break;
        if (cusolverDnCreate(&sol) != CUSOLVER_STATUS_SUCCESS || cusolverDnSetStream(sol, h->stream) !=
                                                                      CUSOLVER_STATUS_SUCCESS) {
            set_error("full SVD: cusolverDnCreate failed");
            fail(DPCA_ERR_CUDA);
            break;
        }
        int lwork = 0;
        if (cusolverDnDsyevd_bufferSize(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n, G, n, W, &lwork) !=
                CUSOLVER_STATUS_SUCCESS ||
            cudaMalloc(&work, (size_t)std::max(lwork, 1) * 8) != cudaSuccess) {
            set_error("full SVD: eigensolver workspace");
            fail(DPCA_ERR_NOMEM);
            break;
        }
        if (cusolverDnDsyevd(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n, G, n, W, work, lwork, dinfo) !=
            CUSOLVER_STATUS_SUCCESS) {
            set_error("full SVD: dsyevd failed");
            fail(DPCA_ERR_CUDA);
            break;
        }
        std::vector<double> w(n);
        if (cudaMemcpyAsync(w.data(), W, (size_t)n * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
            cudaMemcpyAsync(info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) {
            fail(DPCA_ERR_CUDA);
            break;
        }
        // eigenvalues ascending; eigenvector j is column j of the column-major result, i.e. row j
        // of the row-major buffer: the leading ones are the last nsv rows
        std::vector<double> rows((size_t)nsv * n);
        if (cudaMemcpyAsync(rows.data(), G + (size_t)(n - nsv) * n, (size_t)nsv * n * 8, cudaMemcpyDeviceToHost,
                            h->stream) != cudaSuccess ||
            cudaStreamSynchronize(h->stream) != cudaSuccess) {
            set_error("full SVD: result copy failed");
            fail(DPCA_ERR_CUDA);
            break;
        }
        for (int t = 0; t < nsv; ++t) {
            const double lam = w[n - 1 - t];
            sigma[t] = lam > 0 ? std::sqrt(lam) : 0.0;
            const double *vec = rows.data() + (size_t)(nsv - 1 - t) * n;
            for (int i = 0; i < n; ++i) u[(size_t)i * nsv + t] = vec[i];
        }
    } while (false);
    if (sol) cusolverDnDestroy(sol);
    for (void *p : {(void *)G, (void *)W, (void *)work, (void *)dinfo})
        if (p) cudaFree(p);
    return st;
}

}  // namespace dpca
