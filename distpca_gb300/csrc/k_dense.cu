// Small dense FP64 kernels of the subspace iteration (methods.cpp:944-1063):
//   hh_qr_kernel      thin Householder QR with explicit Q, the semantics of LAPACKE_dgeqrf +
//                     LAPACKE_dorgqr (methods.cpp:947-948, 960-961): reflector
//                     beta = -sign(alpha)*||x||, tau = (beta-alpha)/beta, Q = H_0 ... H_{k-1} I.
//                     One cooperative launch; rows are partitioned over the blocks and the
//                     column reductions are exchanged through global memory between grid
//                     barriers (partials summed in block order: deterministic).
//   atb_kernel        C = A^T B over the n rows (B = Q^T Z, methods.cpp:972-973; the in-core
//                     Gram (XQ)^T (XQ), methods.cpp:141-142).
//   jacobi_eig_kernel symmetric eigensolve of the upper triangle (dsyev 'V','U',
//                     methods.cpp:981-989) by parallel cyclic Jacobi, sorted descending
//                     (the column reversal of methods.cpp:994-1000).
//   apply_w_kernel    Omega = Q W (methods.cpp:1006-1007).
//   coldots_kernel + criterion_kernel: sigma = sqrt(w), sum, and crit 0/1/2
//                     (methods.cpp:1012-1063).
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "dpca_internal.h"

namespace cg = cooperative_groups;

namespace dpca {

// ------------------------------------------------------------------ Householder QR
constexpr int kQrThreads = 256;

__global__ void __launch_bounds__(kQrThreads) hh_qr_kernel(double *__restrict__ A, int n, int k,
                                                           double *__restrict__ tau_out, double *__restrict__ part,
                                                           int rows_per_block) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double red[32];
    __shared__ double wsh[kMaxNrhs + 1];
    __shared__ double sc[4];
    const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5, nwarps = kQrThreads / 32;
    const int r0 = b * rows_per_block, r1 = min(n, r0 + rows_per_block);
    const int stride = k + 1;

    // ---- factorization (dgeqr2) ----
    for (int j = 0; j < k; ++j) {
        double *buf = part + (size_t)(j & 1) * G * stride;
        double s = 0.0;
        for (int i = max(r0, j + 1) + tid; i < r1; i += kQrThreads) {
            double v = A[(size_t)i * k + j];
            s += v * v;
        }
        s = block_sum(s, red);
        if (tid == 0) buf[(size_t)b * stride] = s;
        grid.sync();
        if (tid == 0) {
            double xn2 = 0.0;
            for (int p = 0; p < G; ++p) xn2 += buf[(size_t)p * stride];
            double alpha = A[(size_t)j * k + j];
            double beta = alpha, tau = 0.0, scal = 0.0;
            if (xn2 > 0.0) {
                beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
                tau = (beta - alpha) / beta;
                scal = 1.0 / (alpha - beta);
            }
            sc[0] = beta;
            sc[1] = tau;
            sc[2] = scal;
        }
        __syncthreads();
        const double beta = sc[0], tau = sc[1], scal = sc[2];
        if (tau != 0.0)
            for (int i = max(r0, j + 1) + tid; i < r1; i += kQrThreads) A[(size_t)i * k + j] *= scal;
        __syncthreads();
        // partial w[c] = sum_{i >= j} v_i A[i][c], v_j = 1
        for (int c = j + 1 + warp; c < k; c += nwarps) {
            double acc = 0.0;
            for (int i = max(r0, j) + lane; i < r1; i += 32) {
                double v = (i == j) ? 1.0 : A[(size_t)i * k + j];
                acc += v * A[(size_t)i * k + c];
            }
            acc = warp_sum(acc);
            if (lane == 0) buf[(size_t)b * stride + 1 + c] = acc;
        }
        grid.sync();
        for (int c = j + 1 + tid; c < k; c += kQrThreads) {
            double w = 0.0;
            for (int p = 0; p < G; ++p) w += buf[(size_t)p * stride + 1 + c];
            wsh[c] = w;
        }
        __syncthreads();
        if (tau != 0.0) {
            int nc = k - j - 1;
            for (int e = tid; e < (r1 - max(r0, j)) * nc; e += kQrThreads) {
                int i = max(r0, j) + e / nc, c = j + 1 + e % nc;
                double v = (i == j) ? 1.0 : A[(size_t)i * k + j];
                A[(size_t)i * k + c] -= tau * v * wsh[c];
            }
        }
        if (j >= r0 && j < r1 && tid == 0) A[(size_t)j * k + j] = beta;
        if (b == 0 && tid == 0) tau_out[j] = tau;
        __syncthreads();
    }
    grid.sync();
    // ---- explicit Q (dorg2r) ----
    for (int j = k - 1; j >= 0; --j) {
        const double tau = tau_out[j];
        double *buf = part + (size_t)(j & 1) * G * stride;
        if (j < k - 1) {
            for (int c = j + 1 + warp; c < k; c += nwarps) {
                double acc = 0.0;
                for (int i = max(r0, j) + lane; i < r1; i += 32) {
                    double v = (i == j) ? 1.0 : A[(size_t)i * k + j];
                    acc += v * A[(size_t)i * k + c];
                }
                acc = warp_sum(acc);
                if (lane == 0) buf[(size_t)b * stride + 1 + c] = acc;
            }
            grid.sync();
            for (int c = j + 1 + tid; c < k; c += kQrThreads) {
                double w = 0.0;
                for (int p = 0; p < G; ++p) w += buf[(size_t)p * stride + 1 + c];
                wsh[c] = w;
            }
            __syncthreads();
            int nc = k - j - 1;
            for (int e = tid; e < (r1 - max(r0, j)) * nc; e += kQrThreads) {
                int i = max(r0, j) + e / nc, c = j + 1 + e % nc;
                double v = (i == j) ? 1.0 : A[(size_t)i * k + j];
                A[(size_t)i * k + c] -= tau * v * wsh[c];
            }
            __syncthreads();
        }
        for (int i = r0 + tid; i < r1; i += kQrThreads) {
            double *a = A + (size_t)i * k + j;
            if (i > j) *a = -tau * *a;
            else if (i == j) *a = 1.0 - tau;
            else *a = 0.0;
        }
        __syncthreads();
    }
}

dpca_status launch_qr_householder(Handle *h, double *a) {
    ScopedLaunch t(&h->clock, h->stream, "hh_qr");
    int n = h->n_ind, k = h->k;
    // one block per SM at most (every block sums all G partials after each barrier), and only
    // if the kernel fits an SM at all; the query runs once, thread-safely (handles of the
    // serving loop launch from several host threads)
    static const int max_blocks_per_sm = [] {
        int v = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, hh_qr_kernel, kQrThreads, 0) != cudaSuccess) {
            cudaGetLastError();
            v = 1;
        }
        return v;
    }();
    int maxg = std::min(std::max(1, max_blocks_per_sm), 1) * h->sm_count;
    if (h->coop_blocks > 0) maxg = std::min(maxg, h->coop_blocks);
    int G = std::max(1, std::min(maxg, ceil_div(n, 64)));
    int rpb = ceil_div(n, G);
    G = ceil_div(n, rpb);
    if ((size_t)2 * G * (k + 1) > h->red_elems) {
        set_error("QR scratch too small");
        return DPCA_ERR_INVALID;
    }
    double *tau = h->small + SmallLayout{k}.tau();
    double *part = h->red;
    void *args[] = {&a, &n, &k, &tau, &part, &rpb};
    DPCA_CUDA(cudaLaunchCooperativeKernel((void *)hh_qr_kernel, dim3(G), dim3(kQrThreads), args, 0, h->stream));
    return DPCA_OK;
}

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

__global__ void sum_parts_kernel(const double *__restrict__ part, int nparts, int elems, double *__restrict__ out) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < elems; e += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int p = 0; p < nparts; ++p) s += part[(size_t)p * elems + e];
        out[e] = s;
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
        sum_parts_kernel<<<ceil_div(kk, 256), 256, 0, h->stream>>>(h->red, nparts, kk, out);
        DPCA_CUDA(cudaGetLastError());
    }
    return DPCA_OK;
}

dpca_status launch_atb(Handle *h, const double *a, const double *b, int n, double *out) {
    return atb_timed(h, a, b, n, out, "atb", "atb_sum");
}

// ------------------------------------------------------------------ Jacobi eigensolver
// B (k x k, upper triangle used) -> eigenvalues w (descending) and eigenvectors W (columns).
// Parallel cyclic Jacobi with round-robin pairing: per round, every disjoint pair (p,q) computes
// its rotation from the current matrix, then all column rotations, then all row rotations.
// vwork: k*k global scratch for the accumulated rotations.
__global__ void __launch_bounds__(512) jacobi_eig_kernel(const double *__restrict__ Bin, int k,
                                                         double *__restrict__ Wout, double *__restrict__ wout,
                                                         double *__restrict__ V, int max_sweeps) {
    extern __shared__ double sm[];
    const int ld = k + 1;
    double *B = sm;                          // k x ld
    double *cs = B + (size_t)k * ld;         // [64][2]
    int *pos = reinterpret_cast<int *>(cs + 2 * 64);  // m entries
    __shared__ int rotated;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int m = (k + 1) & ~1;  // even number of slots (slot k is a dummy when k is odd)
    for (int e = tid; e < k * k; e += nt) {
        int i = e / k, j = e - i * k;
        B[i * ld + j] = (i <= j) ? Bin[i * k + j] : Bin[j * k + i];
        V[e] = (i == j) ? 1.0 : 0.0;
    }
    for (int e = tid; e < m; e += nt) pos[e] = e;
    __syncthreads();
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        if (tid == 0) rotated = 0;
        __syncthreads();
        for (int round = 0; round < m - 1; ++round) {
            int np = m / 2;
            if (tid < np) {
                int p = pos[tid], q = pos[m - 1 - tid];
                if (p > q) { int t = p; p = q; q = t; }
                double c = 1.0, s = 0.0;
                if (q < k) {
                    double app = B[p * ld + p], aqq = B[q * ld + q], apq = B[p * ld + q];
                    if (apq != 0.0 && fabs(apq) > 1e-300 &&
                        fabs(apq) > 1e-17 * sqrt(fabs(app)) * sqrt(fabs(aqq))) {
                        double theta = (aqq - app) / (2.0 * apq);
                        double t = copysign(1.0, theta) / (fabs(theta) + sqrt(theta * theta + 1.0));
                        c = 1.0 / sqrt(t * t + 1.0);
                        s = t * c;
                        rotated = 1;
                    }
                }
                cs[2 * tid] = c;
                cs[2 * tid + 1] = s;
            }
            __syncthreads();
            // column rotations B <- B J, V <- V J
            for (int e = tid; e < np * k; e += nt) {
                int pr = e / k, i = e - pr * k;
                double c = cs[2 * pr], s = cs[2 * pr + 1];
                if (s == 0.0) continue;
                int p = pos[pr], q = pos[m - 1 - pr];
                if (p > q) { int t = p; p = q; q = t; }
                double bp = B[i * ld + p], bq = B[i * ld + q];
                B[i * ld + p] = c * bp - s * bq;
                B[i * ld + q] = s * bp + c * bq;
                double vp = V[i * k + p], vq = V[i * k + q];
                V[i * k + p] = c * vp - s * vq;
                V[i * k + q] = s * vp + c * vq;
            }
            __syncthreads();
            // row rotations B <- J^T B
            for (int e = tid; e < np * k; e += nt) {
                int pr = e / k, j = e - pr * k;
                double c = cs[2 * pr], s = cs[2 * pr + 1];
                if (s == 0.0) continue;
                int p = pos[pr], q = pos[m - 1 - pr];
                if (p > q) { int t = p; p = q; q = t; }
                double bp = B[p * ld + j], bq = B[q * ld + j];
                B[p * ld + j] = c * bp - s * bq;
                B[q * ld + j] = s * bp + c * bq;
            }
            __syncthreads();
            // round-robin: slot 0 fixed, the others rotate by one
            if (tid == 0) {
                int last = pos[m - 1];
                for (int e = m - 1; e > 1; --e) pos[e] = pos[e - 1];
                pos[1] = last;
            }
            __syncthreads();
        }
        if (!rotated) break;
        __syncthreads();
    }
    // sort descending by eigenvalue (selection by rank; ties keep index order)
    for (int j = tid; j < k; j += nt) {
        double wj = B[j * ld + j];
        int rank = 0;
        for (int i = 0; i < k; ++i) {
            double wi = B[i * ld + i];
            if (wi > wj || (wi == wj && i < j)) rank++;
        }
        wout[rank] = wj;
        for (int i = 0; i < k; ++i) Wout[i * k + rank] = V[i * k + j];
    }
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
// chol_inv_kernel (one block): G (k x k, from the Gram launch) -> R^-1 (upper triangular,
// row-major k x k).  A non-positive or non-finite pivot in a plain step restarts that step with
// the shift; a pivot that still fails (a panel with a zero or non-finite column) is replaced by 1,
// which leaves that column unnormalised instead of dividing by zero.
constexpr int kCholThreads = 256;

__global__ void __launch_bounds__(kCholThreads) chol_inv_kernel(const double *__restrict__ G, int k, int n,
                                                                int always_shift, double *__restrict__ Rinv) {
    extern __shared__ double g[];  // k x k, upper triangle -> R
    __shared__ double sh_inv[kMaxNrhs];
    __shared__ double sh_shift;
    __shared__ int broke;
    const int tid = threadIdx.x;
    // FP64 is a small fraction of this GPU's arithmetic: scalar work (trace, pivots) is done once
    // by thread 0 and broadcast through shared memory
    if (tid == 0) {
        double tr = 0.0;
        for (int i = 0; i < k; ++i) tr += G[(size_t)i * k + i];
        sh_shift = 11.0 * ((double)n * k + (double)k * (k + 1)) * 0x1p-53 * tr;
    }
    __syncthreads();
    const double shift = sh_shift;
    for (int attempt = always_shift ? 1 : 0; attempt < 2; ++attempt) {
        for (int e = tid; e < k * k; e += kCholThreads) {
            const int i = e / k, c = e - i * k;
            g[e] = G[e] + (attempt == 1 && i == c ? shift : 0.0);
        }
        if (tid == 0) broke = 0;
        __syncthreads();
        const int tx = tid & 15, ty = tid >> 4;  // 16 x 16 map of the trailing block
        for (int j = 0; j < k; ++j) {
            if (tid == 0) {
                double d = g[(size_t)j * k + j];
                if (!(d > 0.0) || !isfinite(d)) {
                    broke = 1;
                    d = 1.0;
                }
                const double inv = rsqrt(d);
                g[(size_t)j * k + j] = d * inv;
                sh_inv[j] = inv;
            }
            __syncthreads();
            const double inv = sh_inv[j];
            for (int c = j + 1 + tid; c < k; c += kCholThreads) g[(size_t)j * k + c] *= inv;
            __syncthreads();
            // trailing update of the upper triangle: g[a][b] -= r[j][a] r[j][b], j < a <= b
            for (int a = j + 1 + ty; a < k; a += 16) {
                const double rja = g[(size_t)j * k + a];
                for (int b = a + tx; b < k; b += 16) g[(size_t)a * k + b] -= rja * g[(size_t)j * k + b];
            }
            __syncthreads();
        }
        if (!broke) break;
        __syncthreads();
    }
    // R^-1 in place, column by column (the order of LAPACK's dtrti2): with the leading j x j block
    // already inverted, column j above the diagonal is -(R^-1)_{0:j,0:j} R_{0:j,j} / R_jj; thread i
    // computes row i (i < j <= k <= kMaxNrhs < kCholThreads)
    for (int j = 0; j < k; ++j) {
        double x = 0.0;
        if (tid < j)
            for (int l = tid; l < j; ++l) x = fma(g[(size_t)tid * k + l], g[(size_t)l * k + j], x);
        __syncthreads();
        if (tid < j) g[(size_t)tid * k + j] = -x * sh_inv[j];
        if (tid == j) g[(size_t)j * k + j] = sh_inv[j];
        __syncthreads();
    }
    for (int e = tid; e < k * k; e += kCholThreads) {
        const int i = e / k, c = e - i * k;
        Rinv[e] = c >= i ? g[e] : 0.0;
    }
}

dpca_status launch_qr(Handle *h, double *a) {
    const int n = h->n_ind, k = h->k;
    const SmallLayout L{k};
    double *G = h->small + L.B(), *Rinv = h->small + L.W();  // free until the Rayleigh-Ritz step
    DPCA_TRY(allow_max_smem((const void *)chol_inv_kernel));
    DPCA_TRY(allow_max_smem((const void *)apply_w_kernel));
    const size_t smem_g = (size_t)k * k * sizeof(double);
    const int64_t total = (int64_t)n * k;
    const int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)h->sm_count * 4);
    double *src = a, *dst = h->work;
    for (int step = 0; step < 3; ++step) {
        DPCA_TRY(atb_timed(h, src, src, n, G, "qr_gram", "qr_gram_sum"));
        {
            ScopedLaunch t(&h->clock, h->stream, "qr_chol");
            chol_inv_kernel<<<1, kCholThreads, smem_g, h->stream>>>(G, k, n, step == 0 ? 1 : 0, Rinv);
            DPCA_CUDA(cudaGetLastError());
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
