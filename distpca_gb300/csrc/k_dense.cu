// Small dense FP64 steps of the subspace iteration (methods.cpp:944-1063):
//   launch_qr         thin QR of the n x k panel by shifted CholeskyQR3: atb_kernel (Gram),
//                     the k x k Cholesky factor's inverse on the host (eig_host.cpp), and
//                     apply_w_kernel (A R^-1), three times (methods.cpp:947-961, see launch_qr).
//   atb_kernel        C = A^T B over the n rows (B = Q^T Z, methods.cpp:972-973; the in-core
//                     Gram (XQ)^T (XQ), methods.cpp:141-142).
//   launch_eig_desc   the k x k eigenproblem (dsyev 'V','U', methods.cpp:981-1000) on the host.
//   apply_w_kernel    Omega = Q W (methods.cpp:1006-1007).
//   coldots_kernel + criterion_kernel: sigma = sqrt(w), sum, and crit 0/1/2
//                     (methods.cpp:1012-1063).
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "dpca_internal.h"

namespace dpca {

// ------------------------------------------------------------------ C = A^T B (k x k)
// Block b accumulates rows [b*rpb, ...) into red[b][k*k]; outputs are spread over threads.
__global__ void __launch_bounds__(256) atb_kernel(const double *__restrict__ A, const double *__restrict__ B, int n,
                                                  int k, int rpb, double *__restrict__ part) {
    extern __shared__ double tile[];  // [2][32][k]
    double *ta = tile, *tb = tile + 32 * k;
    const int r0 = blockIdx.x * rpb, r1 = min(n, r0 + rpb);
    const int kk = k * k;
    for (int o0 = 0; o0 < kk; o0 += 256 * 8) {
        double acc[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) acc[m] = 0.0;
        for (int i0 = r0; i0 < r1; i0 += 32) {
            __syncthreads();
            for (int e = threadIdx.x; e < 32 * k; e += 256) {
                int ii = e / k, c = e - ii * k;
                int i = i0 + ii;
                ta[e] = i < r1 ? A[(size_t)i * k + c] : 0.0;
                tb[e] = i < r1 ? B[(size_t)i * k + c] : 0.0;
            }
            __syncthreads();
#pragma unroll
            for (int m = 0; m < 8; ++m) {
                int o = o0 + threadIdx.x + 256 * m;
                if (o < kk) {
                    int a = o / k, c = o - a * k;
                    double s = acc[m];
                    for (int ii = 0; ii < 32; ++ii) s = fma(ta[ii * k + a], tb[ii * k + c], s);
                    acc[m] = s;
                }
            }
        }
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            int o = o0 + threadIdx.x + 256 * m;
            if (o < kk) part[(size_t)blockIdx.x * kk + o] = acc[m];
        }
    }
}

// out[e] = sum over p of part[p][e]: one warp per element, its lanes taking every 32nd part, then
// a fixed-order shuffle reduction (deterministic).  With one thread per element the k^2 sums ran
// on k^2 / 256 blocks, each thread walking all parts: ~36 us per Gram at 12,919 x 40, more than
// the Gram itself.
__global__ void __launch_bounds__(256) sum_parts_kernel(const double *__restrict__ part, int nparts, int elems,
                                                        double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < elems; e += warps) {
        double s = 0.0;
        for (int p = lane; p < nparts; p += 32) s += part[(size_t)p * elems + e];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) out[e] = s;
    }
}

// A^T B over n rows in two launches (block partials, then their sum), timed under the given names.
static dpca_status atb_timed(Handle *h, const double *a, const double *b, int n, double *out, const char *name,
                             const char *sum_name) {
    int k = h->k;
    int kk = k * k;
    // FP64 is a small fraction of this GPU's arithmetic: spread the n k^2 FMAs over as many SMs
    // as there are 32-row tiles (up to two blocks per SM)
    int nparts = std::max(1, std::min(2 * h->sm_count, ceil_div(n, 32)));
    nparts = (int)std::min<int64_t>(nparts, (int64_t)(h->red_elems / kk));
    int rpb = ceil_div(n, nparts);
    nparts = ceil_div(n, rpb);
    size_t smem = (size_t)2 * 32 * k * sizeof(double);
    DPCA_TRY(allow_max_smem((const void *)atb_kernel));
    {
        ScopedLaunch t(&h->clock, h->stream, name);
        atb_kernel<<<nparts, 256, smem, h->stream>>>(a, b, n, k, rpb, h->red);
        DPCA_CUDA(cudaGetLastError());
    }
    {
        ScopedLaunch t(&h->clock, h->stream, sum_name);
        sum_parts_kernel<<<std::min(ceil_div(kk * 32, 256), 8 * h->sm_count), 256, 0, h->stream>>>(h->red, nparts, kk,
                                                                                                 out);
        DPCA_CUDA(cudaGetLastError());
    }
    return DPCA_OK;
}

dpca_status launch_atb(Handle *h, const double *a, const double *b, int n, double *out) {
    return atb_timed(h, a, b, n, out, "atb", "atb_sum");
}

// The k x k eigenproblem goes to the host (eig_host.cpp): B down, W and w (adjacent in the small
// block) back up.  The event pair brackets the copies and the host solve.
dpca_status launch_eig_desc(Handle *h) {
    ScopedLaunch t(&h->clock, h->stream, "sym_eig");
    const int k = h->k;
    const SmallLayout L{k};
    DPCA_CUDA(cudaMemcpyAsync(h->host_small + L.B(), h->small + L.B(), (size_t)k * k * sizeof(double),
                              cudaMemcpyDeviceToHost, h->stream));
    DPCA_CUDA(cudaStreamSynchronize(h->stream));
    DPCA_TRY(check_device_flag(h));
    DPCA_TRY(host_sym_eig_desc(k, h->host_small + L.B(), h->host_small + L.w(), h->host_small + L.W()));
    DPCA_CUDA(cudaMemcpyAsync(h->small + L.W(), h->host_small + L.W(), ((size_t)k * k + k) * sizeof(double),
                              cudaMemcpyHostToDevice, h->stream));
    return DPCA_OK;
}

// ------------------------------------------------------------------ Omega = Q W
__global__ void __launch_bounds__(256) apply_w_kernel(const double *__restrict__ Q, const double *__restrict__ W, int n,
                                                      int k, double *__restrict__ out) {
    extern __shared__ double ws[];
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) ws[e] = W[e];
    __syncthreads();
    int64_t total = (int64_t)n * k;
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < total; o += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = o / k;
        int c = (int)(o - i * k);
        const double *q = Q + i * k;
        double s = 0.0;
        for (int a = 0; a < k; ++a) s = fma(q[a], ws[a * k + c], s);
        out[o] = s;
    }
}

dpca_status launch_apply_w(Handle *h, const double *q, double *out) {
    ScopedLaunch t(&h->clock, h->stream, "apply_w");
    int k = h->k;
    size_t smem = (size_t)k * k * sizeof(double);
    DPCA_TRY(allow_max_smem((const void *)apply_w_kernel));
    int64_t total = (int64_t)h->n_ind * k;
    int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)h->sm_count * 4);
    apply_w_kernel<<<grid, 256, smem, h->stream>>>(q, h->small + SmallLayout{k}.W(), h->n_ind, k, out);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

// ------------------------------------------------------------------ shifted CholeskyQR3
// Thin QR of the n x k panel A (in place, Q only) by three CholeskyQR steps (Fukaya, Kannan,
// Nakatsukasa, Yamamoto, Yanagisawa, "Shifted Cholesky QR for computing the QR factorization of
// ill-conditioned matrices", SIAM J. Sci. Comput. 42 (2020)): G = A^T A, R = chol(G + s I),
// A <- A R^-1, with the shift s = 11 (n k + k (k + 1)) u ||A||_F^2 in the first step, which keeps
// the Cholesky factorization defined for condition numbers up to ~1/u (the reference's start
// block has ~5e9), and then two plain steps (CholeskyQR2) that restore orthogonality to O(u).
// The panel is read three times and written three times; no step needs a grid-wide barrier, so
// the QR costs a dozen short launches instead of ~4k barriers of a column-by-column Householder
// QR.  Q spans the same column space as the reference's dgeqrf + dorgqr (methods.cpp:947-961);
// its columns may differ in sign, which the Rayleigh-Ritz step (methods.cpp:972-1007) absorbs:
// the Ritz vectors come out with the eigensolver's signs either way.
//
dpca_status launch_qr(Handle *h, double *a) {
    const int n = h->n_ind, k = h->k;
    const SmallLayout L{k};
    double *G = h->small + L.B(), *Rinv = h->small + L.W();  // free until the Rayleigh-Ritz step
    DPCA_TRY(allow_max_smem((const void *)apply_w_kernel));
    const size_t smem_g = (size_t)k * k * sizeof(double);
    const int64_t total = (int64_t)n * k;
    const int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)h->sm_count * 4);
    double *src = a, *dst = h->work;
    // the k x k factorization on the host: a k-step FP64 dependency chain runs ~5x faster on a CPU
    // core than on the one SM a device launch of it can use (84 us at k = 40, measured)
    double *hG = h->host_small + L.B(), *hR = h->host_small + L.W();
    for (int step = 0; step < 3; ++step) {
        DPCA_TRY(atb_timed(h, src, src, n, G, "qr_gram", "qr_gram_sum"));
        {
            ScopedLaunch t(&h->clock, h->stream, "qr_chol");
            DPCA_CUDA(cudaMemcpyAsync(hG, G, (size_t)k * k * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            DPCA_CUDA(cudaStreamSynchronize(h->stream));
            host_chol_inv(k, n, hG, step == 0, hR);
            DPCA_CUDA(cudaMemcpyAsync(Rinv, hR, (size_t)k * k * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        }
        {
            ScopedLaunch t(&h->clock, h->stream, "qr_apply");
            apply_w_kernel<<<grid, 256, smem_g, h->stream>>>(src, Rinv, n, k, dst);
            DPCA_CUDA(cudaGetLastError());
        }
        std::swap(src, dst);
    }
    // three steps: a -> work -> a -> work
    DPCA_CUDA(cudaMemcpyAsync(a, src, (size_t)total * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    return DPCA_OK;
}

// ------------------------------------------------------------------ convergence
// part[b][j] = sum over block b's rows of old[i][j] * cur[i][j], j < nsv.
__global__ void __launch_bounds__(256) coldots_kernel(const double *__restrict__ a, const double *__restrict__ b, int n,
                                                      int k, int nsv, int rpb, double *__restrict__ part) {
    __shared__ double red[32];
    int r0 = blockIdx.x * rpb, r1 = min(n, r0 + rpb);
    for (int j = 0; j < nsv; ++j) {
        double s = 0.0;
        for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) s = fma(a[(size_t)i * k + j], b[(size_t)i * k + j], s);
        s = block_sum(s, red);
        if (threadIdx.x == 0) part[(size_t)blockIdx.x * nsv + j] = s;
    }
}

// Single block: sigma_j = sqrt(w_j) (j < nsv), delta = sum sigma, then crit 0/1/2 when ii > 0.
// small.crit: [0] criterion value (NaN at ii = 0), [1] stop flag, [2] delta, [3] previous delta.
__global__ void criterion_kernel(double *__restrict__ small_, int k, int nsv, int crit, double tol, int ii,
                                 const double *__restrict__ dots_part, int nparts) {
    SmallLayout L{k};
    double *w = small_ + L.w(), *sig = small_ + L.sigma(), *old = small_ + L.sigma_old(), *cr = small_ + L.crit();
    if (threadIdx.x != 0) return;
    double delta = 0.0;
    for (int j = 0; j < nsv; ++j) {
        sig[j] = sqrt(w[j]);
        delta += sig[j];
    }
    double val = nan(""), stop = 0.0;
    if (ii > 0) {
        if (crit == 0) {
            val = fabs(cr[3] - delta) / delta;
            stop = val <= tol ? 1.0 : 0.0;
        } else if (crit == 1) {
            int conv = 0;
            for (int j = 0; j < nsv; ++j)
                if (fabs((sig[j] - old[j]) / sig[j]) <= tol) conv++;
            val = conv;
            stop = conv == nsv ? 1.0 : 0.0;
        } else if (crit == 2) {
            double mev = 0.0;
            for (int j = 0; j < nsv; ++j) {
                double d = 0.0;
                for (int p = 0; p < nparts; ++p) d += dots_part[(size_t)p * nsv + j];
                mev += d * d;
            }
            mev /= nsv;
            val = 1.0 - mev;
            stop = val <= tol ? 1.0 : 0.0;
        }
    }
    cr[0] = val;
    cr[1] = stop;
    cr[2] = delta;
    cr[3] = delta;
    for (int j = 0; j < nsv; ++j) old[j] = sig[j];
}

dpca_status launch_sigma_and_criterion(Handle *h, int nsv, int crit, double tol, int ii, const double *old,
                                       const double *omega) {
    int nparts = 0;
    if (crit == 2 && ii > 0) {
        ScopedLaunch t(&h->clock, h->stream, "coldots");
        nparts = std::max(1, std::min(2 * h->sm_count, ceil_div(h->n_ind, 256)));
        nparts = (int)std::min<int64_t>(nparts, (int64_t)(h->red_elems / std::max(1, nsv)));
        int rpb = ceil_div(h->n_ind, nparts);
        nparts = ceil_div(h->n_ind, rpb);
        coldots_kernel<<<nparts, 256, 0, h->stream>>>(old, omega, h->n_ind, h->k, nsv, rpb, h->red);
        DPCA_CUDA(cudaGetLastError());
    }
    ScopedLaunch t(&h->clock, h->stream, "criterion");
    criterion_kernel<<<1, 32, 0, h->stream>>>(h->small, h->k, nsv, crit, tol, ii, h->red, nparts);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

}  // namespace dpca
