// Batched local PCA over SNP windows (dpca_windows_* in dpca.h).
//
// The reference solves one PCA per run (src/distpca.cpp:83-405).  Here W independent PCAs that
// share the individuals -- window w is a consecutive range of m_w SNP rows of one packed
// matrix, standardized on its own (1/sqrt(m_w) in place of 1/sqrt(n_snp), utilities.cpp:294-305)
// -- advance together: each step of the subspace iteration (methods.cpp:941-1066) is one launch
// over every window still iterating.
//
// Layout.  One mixed-precision handle holds all windows' rows, each window padded to whole
// 512-row blocks (the transposed operand's K tiles), padding rows with zero coefficients; a
// 128-row tile or a 64-SNP K-block therefore never straddles two windows.  The tcgen05 products
// run over all windows in one launch each (k_mixed.cu mixed_win_pass): X Omega reads each tile's
// window's Omega slices, X^T Y runs one grid row per window.  The n x k FP64 state of every
// window ([W][n][k]), its QR (shifted CholeskyQR3 in one block per window), Rayleigh-Ritz and
// convergence test are batched kernels below, one block per window.  A window that passes its
// convergence test is marked inactive: every later launch skips it, so its result stays where it
// was written.  The host reads W flags once per outer iteration.
//
// Each window's iteration is dpca_solve's with bsize < n_snp (a full pass for the Rayleigh
// quotient Q^T Z, methods.cpp:972-973) on the mixed path, so a window's result is the one a
// handle of its rows alone gives, within the mixed-path tolerance.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "common.cuh"
#include "dpca_internal.h"

namespace dpca {
namespace {

constexpr int kWinRowAlign = 512;  // rows per 128-byte K tile of the transposed operand
constexpr int kWinThreads = 256;
constexpr int kWinMaxNrhs = 48;    // the mixed path's limit
constexpr int kWinMaxSweeps = 60;

// ------------------------------------------------------------------ small per-window kernels
__global__ void win_replicate_kernel(const double *__restrict__ om, int64_t nk, int W, double *__restrict__ all) {
    const int64_t total = nk * W;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
        all[e] = om[e % nk];
}

__global__ void win_copy_kernel(const double *__restrict__ src, double *__restrict__ dst, int64_t per, int W,
                                const int *__restrict__ active) {
    const int64_t total = per * W;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
        if (!active || active[e / per]) dst[e] = src[e];
}

// Host rows [h0, h0 + cnt) staged at `stride` -> device rows dst_row[h] (one warp per row).
__global__ void win_scatter_kernel(const uint8_t *__restrict__ stage, int64_t stride, int cnt, int h0,
                                   const int *__restrict__ dst_row, uint8_t *__restrict__ P, int64_t pitch,
                                   int64_t np) {
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < cnt; r += warps) {
        const uint8_t *s = stage + (int64_t)r * stride;
        uint8_t *d = P + (int64_t)dst_row[h0 + r] * pitch;
        for (int64_t b = threadIdx.x & 31; b < np; b += 32) d[b] = s[b];
    }
}

// Sum over the n rows of a[i][ca] * b[i][cb] for every pair (ca <= cb), into out[ca * k + cb]
// (and the mirrored entry): block partials by row groups in shared memory, summed in a fixed
// order (deterministic).  part holds max(1, kWinThreads / k^2) * k^2 doubles.
__device__ void block_atb_upper(const double *__restrict__ a, const double *__restrict__ b, int n, int k,
                                double *part, double *out) {
    const int kk = k * k, tid = threadIdx.x;
    const int groups = kk <= kWinThreads ? kWinThreads / kk : 1;
    for (int t = tid; t < groups * kk; t += kWinThreads) {
        const int pr = t % kk, g = t / kk;
        const int ca = pr / k, cb = pr - ca * k;
        double s = 0.0;
        if (ca <= cb)
            for (int i = g; i < n; i += groups) s = fma(a[(size_t)i * k + ca], b[(size_t)i * k + cb], s);
        part[t] = s;
    }
    __syncthreads();
    for (int pr = tid; pr < kk; pr += kWinThreads) {
        const int ca = pr / k, cb = pr - ca * k;
        if (ca <= cb) {
            double s = 0.0;
            for (int g = 0; g < groups; ++g) s += part[(size_t)g * kk + pr];
            out[ca * k + cb] = s;
            out[cb * k + ca] = s;
        }
    }
    __syncthreads();
}

// Thread 0: R = chol(G [+ shift I]) then R^-1 in place (upper, row-major), as host_chol_inv.
__device__ void chol_inv_serial(const double *G, double *R, int k, int n, bool always_shift, double *sinv) {
    double tr = 0.0;
    for (int i = 0; i < k; ++i) tr += G[i * k + i];
    const double shift = 11.0 * ((double)n * k + (double)k * (k + 1)) * 0x1p-53 * tr;
    for (int attempt = always_shift ? 1 : 0; attempt < 2; ++attempt) {
        bool broke = false;
        for (int e = 0; e < k * k; ++e) R[e] = G[e] + (attempt == 1 && e / k == e % k ? shift : 0.0);
        for (int j = 0; j < k; ++j) {
            double d = R[j * k + j];
            if (!(d > 0.0) || !isfinite(d)) {
                broke = true;
                d = 1.0;
            }
            const double inv = rsqrt(d);
            R[j * k + j] = d * inv;
            sinv[j] = inv;
            for (int c = j + 1; c < k; ++c) R[j * k + c] *= inv;
            for (int a = j + 1; a < k; ++a)
                for (int c = a; c < k; ++c) R[a * k + c] -= R[j * k + a] * R[j * k + c];
        }
        if (!broke) break;
    }
    for (int j = 0; j < k; ++j) {
        for (int i = 0; i < j; ++i) {
            double x = 0.0;
            for (int l = i; l < j; ++l) x = fma(R[i * k + l], R[l * k + j], x);
            sinv[k + i] = -x * sinv[j];  // column j of the inverse, rows < j (R[l][j], l < j, still R)
        }
        for (int i = 0; i < j; ++i) R[i * k + j] = sinv[k + i];
        R[j * k + j] = sinv[j];
    }
    for (int i = 1; i < k; ++i)
        for (int c = 0; c < i; ++c) R[i * k + c] = 0.0;
}

// Shifted CholeskyQR3 of each active window: out_w = Q of in_w (n x k); tmp is scratch (in may
// be out).  Steps: in -> tmp -> out -> tmp, then tmp -> out.
__global__ void __launch_bounds__(kWinThreads) win_qr_kernel(const double *in_all, double *out_all, double *tmp_all,
                                                             int n, int k, const int *__restrict__ active) {
    extern __shared__ double sm[];
    const int w = blockIdx.x;
    if (active && !active[w]) return;
    const int kk = k * k;
    double *G = sm, *R = G + kk, *sinv = R + kk, *part = sinv + 2 * k;
    const size_t off = (size_t)w * n * k;
    const double *in = in_all + off;
    double *out = out_all + off, *tmp = tmp_all + off;
    for (int step = 0; step < 3; ++step) {
        const double *src = step == 0 ? in : (step == 1 ? tmp : out);
        double *dst = step == 1 ? out : tmp;
        block_atb_upper(src, src, n, k, part, G);
        if (threadIdx.x == 0) chol_inv_serial(G, R, k, n, step == 0, sinv);
        __syncthreads();
        for (int e = threadIdx.x; e < n * k; e += kWinThreads) {
            const int i = e / k, c = e - i * k;
            double s = 0.0;
            for (int a = 0; a <= c; ++a) s = fma(src[(size_t)i * k + a], R[a * k + c], s);
            dst[e] = s;
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < n * k; e += kWinThreads) out[e] = tmp[e];
}

// Rayleigh-Ritz and the convergence test of each active window (methods.cpp:972-1063):
// B = Q^T Z (upper triangle), eigenpairs by cyclic Jacobi in descending order, Omega = Q W,
// sigma_j = sqrt(w_j) (j < nsv), then crit 0/1/2 when ii > 0; a window that stops is marked
// inactive with its iteration count.  crit 2 compares with old_w (replaced by the new Omega).
__global__ void __launch_bounds__(kWinThreads) win_rr_kernel(const double *__restrict__ Q_all,
                                                             const double *__restrict__ Z_all, double *Om_all,
                                                             double *old_all, int n, int k, int nsv, int crit,
                                                             double tol, int ii, int *active, int *its,
                                                             double *sig_all, double *delta_old) {
    extern __shared__ double sm[];
    __shared__ double red[32];
    __shared__ double cs[2];
    __shared__ int rotated, stop;
    const int w = blockIdx.x, tid = threadIdx.x;
    if (!active[w]) return;
    const int kk = k * k;
    double *B = sm, *V = B + kk, *Wm = V + kk, *ev = Wm + kk, *part = ev + k;
    int *order = reinterpret_cast<int *>(part + (kk > kWinThreads ? kk : kWinThreads));
    const size_t off = (size_t)w * n * k;
    const double *Q = Q_all + off, *Z = Z_all + off;
    double *Om = Om_all + off;
    block_atb_upper(Q, Z, n, k, part, B);  // symmetric from the upper triangle ('U')
    for (int e = tid; e < kk; e += kWinThreads) V[e] = e / k == e % k ? 1.0 : 0.0;
    __syncthreads();
    for (int sweep = 0; sweep < kWinMaxSweeps; ++sweep) {
        if (tid == 0) rotated = 0;
        __syncthreads();
        for (int p = 0; p < k - 1; ++p)
            for (int q = p + 1; q < k; ++q) {
                if (tid == 0) {
                    const double app = B[p * k + p], aqq = B[q * k + q], apq = B[p * k + q];
                    double c = 1.0, s = 0.0;
                    if (apq != 0.0 && fabs(apq) > 1e-300 && fabs(apq) > 1e-17 * sqrt(fabs(app)) * sqrt(fabs(aqq))) {
                        const double theta = (aqq - app) / (2.0 * apq);
                        const double t = copysign(1.0, theta) / (fabs(theta) + sqrt(theta * theta + 1.0));
                        c = 1.0 / sqrt(t * t + 1.0);
                        s = t * c;
                        rotated = 1;
                    }
                    cs[0] = c;
                    cs[1] = s;
                }
                __syncthreads();
                const double c = cs[0], s = cs[1];
                if (s != 0.0) {
                    for (int i = tid; i < k; i += kWinThreads) {  // columns: B J, V J
                        const double bp = B[i * k + p], bq = B[i * k + q];
                        B[i * k + p] = c * bp - s * bq;
                        B[i * k + q] = s * bp + c * bq;
                        const double vp = V[i * k + p], vq = V[i * k + q];
                        V[i * k + p] = c * vp - s * vq;
                        V[i * k + q] = s * vp + c * vq;
                    }
                    __syncthreads();
                    for (int j = tid; j < k; j += kWinThreads) {  // rows: J^T B
                        const double bp = B[p * k + j], bq = B[q * k + j];
                        B[p * k + j] = c * bp - s * bq;
                        B[q * k + j] = s * bp + c * bq;
                    }
                }
                __syncthreads();
            }
        if (!rotated) break;
        __syncthreads();
    }
    if (tid == 0) {  // descending order (ties keep index order)
        for (int j = 0; j < k; ++j) {
            int rank = 0;
            for (int i = 0; i < k; ++i)
                if (B[i * k + i] > B[j * k + j] || (B[i * k + i] == B[j * k + j] && i < j)) rank++;
            order[rank] = j;
        }
    }
    __syncthreads();
    for (int e = tid; e < kk; e += kWinThreads) {
        const int i = e / k, c = e - i * k;
        Wm[e] = V[i * k + order[c]];
    }
    for (int c = tid; c < k; c += kWinThreads) ev[c] = B[order[c] * k + order[c]];
    __syncthreads();
    for (int e = tid; e < n * k; e += kWinThreads) {  // Omega = Q W
        const int i = e / k, c = e - i * k;
        double s = 0.0;
        for (int a = 0; a < k; ++a) s = fma(Q[(size_t)i * k + a], Wm[a * k + c], s);
        Om[e] = s;
    }
    __syncthreads();
    double mev = 0.0;
    if (crit == 2 && ii > 0) {
        const double *old = old_all + off;
        for (int j = 0; j < nsv; ++j) {
            double d = 0.0;
            for (int i = tid; i < n; i += kWinThreads) d = fma(old[(size_t)i * k + j], Om[(size_t)i * k + j], d);
            d = block_sum(d, red);
            mev += d * d;
        }
    }
    if (tid == 0) {
        double *sig = sig_all + (size_t)w * k;
        double delta = 0.0;
        int conv = 0;
        for (int j = 0; j < nsv; ++j) {
            const double sj = sqrt(ev[j]);
            if (fabs((sj - sig[j]) / sj) <= tol) conv++;
            sig[j] = sj;
            delta += sj;
        }
        int st = 0;
        if (ii > 0) {
            if (crit == 0) st = fabs(delta_old[w] - delta) / delta <= tol;
            else if (crit == 1) st = conv == nsv;
            else if (crit == 2) st = 1.0 - mev / nsv <= tol;
        }
        delta_old[w] = delta;
        stop = st;
        if (st) {
            active[w] = 0;
            its[w] = ii + 1;
        }
    }
    __syncthreads();
    if (crit == 2 && !stop) {
        double *old = old_all + off;
        for (int e = tid; e < n * k; e += kWinThreads) old[e] = Om[e];
    }
}

size_t qr_smem(int k) { return (size_t)(2 * k * k + 2 * k + std::max(kWinThreads, k * k)) * sizeof(double); }
size_t rr_smem(int k) {
    return (size_t)(3 * k * k + k + std::max(kWinThreads, k * k)) * sizeof(double) + (size_t)k * sizeof(int);
}

int grid_for(int64_t elems, int sm) { return (int)std::max<int64_t>(1, std::min<int64_t>((elems + 255) / 256, (int64_t)sm * 8)); }

}  // namespace
}  // namespace dpca

using namespace dpca;

struct dpca_windows {
    dpca_handle *hh = nullptr;
    int W = 0, n = 0, k = 0, rows = 0;
    int64_t host_rows = 0;
    std::vector<int> m, row0;  // per window: SNPs, first device row
    int *tile_win = nullptr, *win_kb0 = nullptr, *win_nkb = nullptr, *active = nullptr, *its = nullptr;
    int *dst_row = nullptr, *row_src = nullptr;  // host row -> device row; device row -> host row (-1)
    double *row_inv = nullptr;                    // per device row 1/sqrt(m_w), 0 on padding rows
    double *omega = nullptr, *z = nullptr, *q = nullptr, *tmp = nullptr, *old = nullptr, *partial = nullptr;
    double *scales = nullptr, *sig = nullptr, *delta_old = nullptr;
    unsigned int *colmax = nullptr;
    long long *colsumq = nullptr, *rq = nullptr;
    __half *omega_s = nullptr;
    CUtensorMap map_om;
    WinPass pass;
};

namespace {

void free_windows(dpca_windows *w) {
    void *ptrs[] = {w->tile_win, w->win_kb0, w->win_nkb, w->active, w->its,     w->dst_row, w->row_src,
                    w->row_inv,  w->omega,   w->z,       w->q,      w->tmp,     w->old,     w->partial,
                    w->scales,   w->sig,     w->delta_old, w->colmax, w->colsumq, w->rq,    w->omega_s};
    if (w->hh) cudaStreamSynchronize(w->hh->h.stream);
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (w->hh) dpca_destroy(w->hh);
    delete w;
}

template <typename T>
dpca_status walloc(T **p, size_t elems) {
    *p = nullptr;
    cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(elems, 1) * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("windows: device allocation of %zu bytes: %s", elems * sizeof(T), cudaGetErrorString(e));
        *p = nullptr;
        return DPCA_ERR_NOMEM;
    }
    return DPCA_OK;
}

dpca_status after_rows(dpca_windows *w) {
    Handle *h = &w->hh->h;
    {
        ScopedLaunch t(&h->clock, h->stream, "snp_stats");
        launch_snp_stats_raw(h->P, h->pitch, h->n_ind, h->n_snp, 1.0, h->counts, h->avg, h->sd, h->lut, h->coef,
                             h->stream, w->row_inv);
        DPCA_CUDA(cudaGetLastError());
    }
    {
        ScopedLaunch t(&h->clock, h->stream, "transpose_packed");
        launch_transpose_raw(h->P, h->pitch, h->PT, h->pitchT, h->n_ind, h->n_snp, h->stream);
        DPCA_CUDA(cudaGetLastError());
    }
    DPCA_CUDA(cudaStreamSynchronize(h->stream));
    h->stats_ready = true;
    return DPCA_OK;
}

dpca_status win_qr(dpca_windows *w, const double *in, double *out) {
    Handle *h = &w->hh->h;
    ScopedLaunch t(&h->clock, h->stream, "win_qr");
    win_qr_kernel<<<w->W, kWinThreads, qr_smem(w->k), h->stream>>>(in, out, w->tmp, w->n, w->k, w->active);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

dpca_status win_pass(dpca_windows *w, const double *in, double *out) {
    w->pass.omega = in;
    w->pass.z = out;
    return mixed_win_pass(&w->hh->h, w->pass);
}

}  // namespace

extern "C" {

dpca_status dpca_windows_create(dpca_windows **out, int n_ind, int n_win, const int *win_snps, int nrhs, int device,
                                void *stream) {
    clear_error();
    if (!out || !win_snps || n_ind <= 0 || n_win <= 0 || nrhs <= 0) {
        set_error("dpca_windows_create: bad arguments");
        return DPCA_ERR_INVALID;
    }
    *out = nullptr;
    if (nrhs > kWinMaxNrhs) {
        set_error("dpca_windows_create: nrhs=%d above the mixed-precision limit %d", nrhs, kWinMaxNrhs);
        return DPCA_ERR_UNSUPPORTED;
    }
    if (n_win > 65535) {
        set_error("dpca_windows_create: at most 65535 windows");
        return DPCA_ERR_UNSUPPORTED;
    }
    dpca_windows *w = new (std::nothrow) dpca_windows();
    if (!w) return DPCA_ERR_NOMEM;
    w->W = n_win;
    w->n = n_ind;
    w->k = nrhs;
    w->m.assign(win_snps, win_snps + n_win);
    int64_t rows = 0, hrows = 0;
    for (int i = 0; i < n_win; ++i) {
        if (w->m[i] <= 0) {
            delete w;
            set_error("dpca_windows_create: window %d has %d SNPs", i, w->m[i]);
            return DPCA_ERR_INVALID;
        }
        w->row0.push_back((int)rows);
        rows += (w->m[i] + kWinRowAlign - 1) / kWinRowAlign * kWinRowAlign;
        hrows += w->m[i];
    }
    if (rows > (int64_t)1 << 30) {
        delete w;
        set_error("dpca_windows_create: %lld padded rows is too many", (long long)rows);
        return DPCA_ERR_UNSUPPORTED;
    }
    w->rows = (int)rows;
    w->host_rows = hrows;
    dpca_status st = dpca_create(&w->hh, n_ind, w->rows, nrhs, DPCA_PREC_MIXED, device, stream);
    if (st != DPCA_OK) {
        delete w;
        return st;
    }
    Handle *h = &w->hh->h;
    const size_t nk = (size_t)n_ind * nrhs, Wnk = nk * n_win;
    const int N = 2 * ((nrhs + 7) / 8 * 8);
    if ((st = walloc(&w->tile_win, rows / 128)) || (st = walloc(&w->win_kb0, n_win)) ||
        (st = walloc(&w->win_nkb, n_win)) || (st = walloc(&w->active, n_win)) || (st = walloc(&w->its, n_win)) ||
        (st = walloc(&w->dst_row, hrows)) || (st = walloc(&w->row_src, rows)) || (st = walloc(&w->row_inv, rows)) ||
        (st = walloc(&w->omega, Wnk)) || (st = walloc(&w->z, Wnk)) || (st = walloc(&w->q, Wnk)) ||
        (st = walloc(&w->tmp, Wnk)) || (st = walloc(&w->old, Wnk)) || (st = walloc(&w->partial, Wnk)) ||
        (st = walloc(&w->scales, (size_t)4 * nrhs * n_win)) || (st = walloc(&w->sig, (size_t)nrhs * n_win)) ||
        (st = walloc(&w->delta_old, n_win)) || (st = walloc(&w->colmax, (size_t)nrhs * n_win)) ||
        (st = walloc(&w->colsumq, (size_t)nrhs * n_win)) || (st = walloc(&w->rq, (size_t)nrhs * n_win)) ||
        (st = walloc(&w->omega_s, (size_t)n_win * N * h->n_ind_pad))) {
        free_windows(w);
        return st;
    }
    // tables (host-built, copied once)
    std::vector<int> tw(rows / 128), kb0(n_win), nkb(n_win), rsrc(rows, -1), drow(hrows);
    std::vector<double> rinv(rows, 0.0);
    int64_t hr = 0;
    for (int i = 0; i < n_win; ++i) {
        const int r0 = w->row0[i], mp = (w->m[i] + kWinRowAlign - 1) / kWinRowAlign * kWinRowAlign;
        for (int t = r0 / 128; t < (r0 + mp) / 128; ++t) tw[t] = i;
        kb0[i] = r0 / 64;
        nkb[i] = mp / 64;
        const double inv = 1.0 / sqrt((double)w->m[i]);
        for (int j = 0; j < w->m[i]; ++j, ++hr) {
            rsrc[r0 + j] = (int)hr;
            drow[hr] = r0 + j;
            rinv[r0 + j] = inv;
        }
    }
    cudaStream_t s = h->stream;
    if (cudaMemcpyAsync(w->tile_win, tw.data(), tw.size() * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(w->win_kb0, kb0.data(), kb0.size() * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(w->win_nkb, nkb.data(), nkb.size() * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(w->row_src, rsrc.data(), rsrc.size() * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(w->dst_row, drow.data(), drow.size() * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(w->row_inv, rinv.data(), rinv.size() * 8, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        set_error("dpca_windows_create: table upload: %s", cudaGetErrorString(cudaGetLastError()));
        free_windows(w);
        return DPCA_ERR_CUDA;
    }
    if ((st = allow_max_smem((const void *)win_qr_kernel)) != DPCA_OK ||
        (st = allow_max_smem((const void *)win_rr_kernel)) != DPCA_OK) {
        free_windows(w);
        return st;
    }
    WinPass &p = w->pass;
    p.W = n_win;
    p.tile_win = w->tile_win;
    p.win_kb0 = w->win_kb0;
    p.win_nkb = w->win_nkb;
    p.active = w->active;
    p.omega_s = w->omega_s;
    p.scales = w->scales;
    p.colmax = w->colmax;
    p.colsumq = w->colsumq;
    p.rq = w->rq;
    p.partial = w->partial;
    p.map_om = &w->map_om;
    *out = w;
    return DPCA_OK;
}

dpca_handle *dpca_windows_handle(dpca_windows *w) { return w ? w->hh : nullptr; }

dpca_status dpca_windows_destroy(dpca_windows *w) {
    if (w) free_windows(w);
    return DPCA_OK;
}

dpca_status dpca_windows_upload(dpca_windows *w, const uint8_t *packed, int64_t row_stride) {
    clear_error();
    if (!w || !packed) return DPCA_ERR_INVALID;
    Handle *h = &w->hh->h;
    if (row_stride < h->np) {
        set_error("row_stride %lld < ceil(n_ind/4) = %lld", (long long)row_stride, (long long)h->np);
        return DPCA_ERR_INVALID;
    }
    DPCA_CUDA(cudaSetDevice(h->device));
    const int64_t per = std::max<int64_t>(1, std::min<int64_t>(w->host_rows, ((int64_t)256 << 20) / row_stride));
    uint8_t *stage = nullptr;
    DPCA_TRY(walloc(&stage, (size_t)per * row_stride));
    dpca_status st = DPCA_OK;
    for (int64_t h0 = 0; h0 < w->host_rows && st == DPCA_OK; h0 += per) {
        const int cnt = (int)std::min<int64_t>(per, w->host_rows - h0);
        cudaError_t e = cudaMemcpyAsync(stage, packed + h0 * row_stride, (size_t)cnt * row_stride,
                                        cudaMemcpyHostToDevice, h->stream);
        if (e == cudaSuccess) {
            win_scatter_kernel<<<grid_for((int64_t)cnt * 32, h->sm_count), 256, 0, h->stream>>>(
                stage, row_stride, cnt, (int)h0, w->dst_row, h->P, h->pitch, h->np);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) {
            set_error("dpca_windows_upload: %s", cudaGetErrorString(e));
            st = DPCA_ERR_CUDA;
        }
    }
    cudaStreamSynchronize(h->stream);
    cudaFree(stage);
    DPCA_TRY(st);
    return after_rows(w);
}

dpca_status dpca_windows_synth_fill(dpca_windows *w, uint64_t key, const uint8_t *pop, const uint32_t *miss_thr,
                                    const uint32_t *snp_thr, int n_pop) {
    clear_error();
    if (!w || !pop || !miss_thr || !snp_thr || n_pop <= 0) return DPCA_ERR_INVALID;
    Handle *h = &w->hh->h;
    DPCA_CUDA(cudaSetDevice(h->device));
    uint8_t *d_pop = nullptr;
    uint32_t *d_miss = nullptr, *d_thr = nullptr;
    dpca_status st = walloc(&d_pop, w->n);
    if (st == DPCA_OK) st = walloc(&d_miss, w->n);
    if (st == DPCA_OK) st = walloc(&d_thr, (size_t)w->host_rows * n_pop);
    if (st == DPCA_OK &&
        (cudaMemcpyAsync(d_pop, pop, (size_t)w->n, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
         cudaMemcpyAsync(d_miss, miss_thr, (size_t)w->n * 4, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
         cudaMemcpyAsync(d_thr, snp_thr, (size_t)w->host_rows * n_pop * 4, cudaMemcpyHostToDevice, h->stream) !=
             cudaSuccess)) {
        set_error("dpca_windows_synth_fill: copy: %s", cudaGetErrorString(cudaGetLastError()));
        st = DPCA_ERR_CUDA;
    }
    if (st == DPCA_OK) st = launch_synth_fill(h, key, d_pop, d_miss, d_thr, n_pop, w->row_src);
    cudaStreamSynchronize(h->stream);
    if (d_pop) cudaFree(d_pop);
    if (d_miss) cudaFree(d_miss);
    if (d_thr) cudaFree(d_thr);
    DPCA_TRY(st);
    return after_rows(w);
}

dpca_status dpca_windows_solve(dpca_windows *w, const dpca_config *cfg, const double *omega0, double *sigma,
                               double *u, int *its_out) {
    clear_error();
    if (!w || !cfg || !sigma) return DPCA_ERR_INVALID;
    Handle *h = &w->hh->h;
    const int n = w->n, k = w->k, W = w->W, nsv = cfg->nsv, power = cfg->power, miter = cfg->miter;
    if (nsv <= 0 || nsv > k || power < 1 || miter < 1 || cfg->crit < 0 || cfg->crit > 2) {
        set_error("dpca_windows_solve: need 0 < nsv <= nrhs, power >= 1, miter >= 1, crit in 0..2");
        return DPCA_ERR_INVALID;
    }
    if (!h->stats_ready) {
        set_error("dpca_windows_solve: no genotype data on the device");
        return DPCA_ERR_INVALID;
    }
    DPCA_CUDA(cudaSetDevice(h->device));
    cudaStream_t s = h->stream;
    const int64_t nk = (int64_t)n * k;
    std::vector<double> om0((size_t)nk);
    if (omega0)
        std::memcpy(om0.data(), omega0, om0.size() * sizeof(double));
    else
        DPCA_TRY(dpca_start_block(n, k, om0.data()));
    std::vector<int> ones(W, 1), itsv(W, miter);
    DPCA_CUDA(cudaMemcpyAsync(w->q, om0.data(), (size_t)nk * 8, cudaMemcpyHostToDevice, s));
    win_replicate_kernel<<<grid_for(nk * W, h->sm_count), 256, 0, s>>>(w->q, nk, W, w->omega);
    DPCA_CUDA(cudaGetLastError());
    DPCA_CUDA(cudaMemcpyAsync(w->active, ones.data(), (size_t)W * 4, cudaMemcpyHostToDevice, s));
    DPCA_CUDA(cudaMemcpyAsync(w->its, itsv.data(), (size_t)W * 4, cudaMemcpyHostToDevice, s));
    DPCA_CUDA(cudaMemsetAsync(w->sig, 0, (size_t)W * k * 8, s));
    DPCA_CUDA(cudaMemsetAsync(w->delta_old, 0, (size_t)W * 8, s));
    if (cfg->crit == 2)
        win_copy_kernel<<<grid_for(nk * W, h->sm_count), 256, 0, s>>>(w->omega, w->old, nk, W, nullptr);
    // the start block orthonormalised first, as dpca_solve does on the mixed path
    DPCA_TRY(win_qr(w, w->omega, w->omega));
    std::vector<int> act(W, 1);
    int ii = 0;
    for (ii = 0; ii < miter; ++ii) {
        DPCA_TRY(win_pass(w, w->omega, w->z));
        for (int kk = 0; kk < power - 1; ++kk) {
            DPCA_TRY(win_qr(w, w->z, w->omega));
            DPCA_TRY(win_pass(w, w->omega, w->z));
        }
        DPCA_TRY(win_qr(w, w->z, w->q));
        DPCA_TRY(win_pass(w, w->q, w->z));
        {
            ScopedLaunch t(&h->clock, s, "win_rr");
            win_rr_kernel<<<W, kWinThreads, rr_smem(k), s>>>(w->q, w->z, w->omega, w->old, n, k, nsv, cfg->crit,
                                                               cfg->tol, ii, w->active, w->its, w->sig, w->delta_old);
            DPCA_CUDA(cudaGetLastError());
        }
        DPCA_CUDA(cudaMemcpyAsync(act.data(), w->active, (size_t)W * 4, cudaMemcpyDeviceToHost, s));
        DPCA_CUDA(cudaStreamSynchronize(s));
        DPCA_TRY(check_device_flag(h));
        if (std::none_of(act.begin(), act.end(), [](int a) { return a != 0; })) break;
    }
    std::vector<double> sg((size_t)W * k);
    DPCA_CUDA(cudaMemcpyAsync(sg.data(), w->sig, sg.size() * 8, cudaMemcpyDeviceToHost, s));
    DPCA_CUDA(cudaMemcpyAsync(itsv.data(), w->its, (size_t)W * 4, cudaMemcpyDeviceToHost, s));
    std::vector<double> om;
    if (u) {
        om.resize((size_t)nk * W);
        DPCA_CUDA(cudaMemcpyAsync(om.data(), w->omega, om.size() * 8, cudaMemcpyDeviceToHost, s));
    }
    DPCA_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < W; ++i) {
        for (int j = 0; j < nsv; ++j) {
            const double v = sg[(size_t)i * k + j];
            if (!std::isfinite(v)) {
                set_error("window %d: non-finite singular value %d", i, j);
                return DPCA_ERR_NUMERIC;
            }
            sigma[(size_t)i * nsv + j] = v;
        }
        if (its_out) its_out[i] = itsv[i];
        if (u)
            for (int r = 0; r < n; ++r)
                for (int j = 0; j < nsv; ++j)
                    u[((size_t)i * n + r) * nsv + j] = om[(size_t)i * nk + (size_t)r * k + j];
    }
    return DPCA_OK;
}

}  // extern "C"
