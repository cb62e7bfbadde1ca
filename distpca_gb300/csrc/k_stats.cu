// Per-SNP decode statistics, the synthetic-cohort fill, and the individual-major
// transposed copy of the packed matrix.
//
// snp_counts_kernel + snp_moments_kernel restate, on the device and bit-exactly,
//   decode_plink_sse2 (utilities.cpp:351-414): code 00 -> 0, 01 -> missing, 10 -> 1, 11 -> 2;
//   standardize (utilities.cpp:272-292): avg = sum/ctr over non-missing, p = avg/2,
//     sd = sqrt(2p(1-p)) -- all in IEEE FP64 with explicit round-to-nearest ops so that no
//     contraction can change a bit;
//   the LUT cache (methods.cpp:819-843): value per code = ((g - avg)/sd) * (1/sqrt(n_snp)),
//     zero for missing codes and for SNPs with sd <= 1e-9.
// The streaming pass (counts) is separate from the per-SNP FP64 arithmetic (moments), so that
// the divisions and square roots stay off the HBM-bound loop: one warp streams one SNP row with
// 128-bit coalesced loads and three population counts per pair of words, reduced with shuffles.
#include <algorithm>

#include "common.cuh"
#include "dpca_internal.h"

namespace dpca {

// Pass 1: counts only.  One warp per SNP row streams the row with 16-byte loads; per pair of
// words three population counts give popc(hi) = c10 + c11, popc(lo) = c01 + c11 and
// popc(hi & lo) = c11 (two words' even-position bits interleaved into one word).
__global__ void __launch_bounds__(256) snp_counts_kernel(const uint8_t *__restrict__ P, int64_t pitch, int n_ind,
                                                         int n_snp, int64_t np, int32_t *__restrict__ counts) {
    int lane = threadIdx.x & 31;
    int64_t s = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= n_snp) return;
    const uint4 *row = reinterpret_cast<const uint4 *>(P + s * pitch);
    int nchunk = (int)((np + 15) >> 4);
    int n_hi = 0, n_lo = 0, n_11 = 0, n_valid = 0;
#pragma unroll 8
    for (int c = lane; c < nchunk; c += 32) {
        uint4 v = __ldg(row + c);
        uint32_t ws[4] = {v.x, v.y, v.z, v.w};
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int base = c * 64 + j * 16;  // first individual of this word
            int valid = n_ind - base;
            uint32_t m = valid >= 16 ? 0x55555555u : (valid <= 0 ? 0u : (((1u << (2 * valid)) - 1u) & 0x55555555u));
            hi[j] = (ws[j] >> 1) & m;
            lo[j] = ws[j] & m;
            n_valid += valid >= 16 ? 16 : (valid <= 0 ? 0 : valid);
        }
#pragma unroll
        for (int j = 0; j < 4; j += 2) {
            const uint32_t h2 = hi[j] | (hi[j + 1] << 1), l2 = lo[j] | (lo[j + 1] << 1);
            n_hi += __popc(h2);
            n_lo += __popc(l2);
            n_11 += __popc(h2 & l2);
        }
    }
    n_hi = warp_sum_int(n_hi);
    n_lo = warp_sum_int(n_lo);
    n_11 = warp_sum_int(n_11);
    n_valid = warp_sum_int(n_valid);
    if (lane != 0) return;
    const int c11 = n_11, c10 = n_hi - n_11, c01 = n_lo - n_11, c00 = n_valid - c01 - c10 - c11;
    counts[4 * s + 0] = c00;
    counts[4 * s + 1] = c01;
    counts[4 * s + 2] = c10;
    counts[4 * s + 3] = c11;
}

// Pass 2: one thread per SNP turns its counts into mean, sd, the LUT and the mixed-path
// coefficients (the FP64 divisions stay off the streaming pass).  row_inv_sqrt (optional) gives
// each row its own 1/sqrt(n_snp): batched windows standardize each window on its own, and a
// padding row gets 0 (zero LUT and coefficients).
__global__ void __launch_bounds__(256) snp_moments_kernel(int n_snp, double inv_sqrt_all,
                                                          const int32_t *__restrict__ counts, double *__restrict__ avg,
                                                          double *__restrict__ sd, double *__restrict__ lut,
                                                          double *__restrict__ coef,
                                                          const double *__restrict__ row_inv_sqrt) {
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n_snp; s += (int64_t)gridDim.x * blockDim.x) {
        const double inv_sqrt_nsnp = row_inv_sqrt ? row_inv_sqrt[s] : inv_sqrt_all;
        const int c00 = counts[4 * s + 0], c10 = counts[4 * s + 2], c11 = counts[4 * s + 3];
        double sum = (double)c10 + 2.0 * (double)c11;  // exact: small integers
        unsigned int ctr = (unsigned int)(c00 + c10 + c11);
        double mean = __ddiv_rn(sum, (double)ctr);
        double p = __ddiv_rn(mean, 2.0);
        double sdev = __dsqrt_rn(__dmul_rn(__dmul_rn(2.0, p), __dsub_rn(1.0, p)));
        avg[s] = mean;
        sd[s] = sdev;
        double v00 = 0.0, v10 = 0.0, v11 = 0.0, b = 0.0, a = 0.0;
        if (sdev > 1e-9) {
            v00 = __dmul_rn(__ddiv_rn(__dsub_rn(0.0, mean), sdev), inv_sqrt_nsnp);
            v10 = __dmul_rn(__ddiv_rn(__dsub_rn(1.0, mean), sdev), inv_sqrt_nsnp);
            v11 = __dmul_rn(__ddiv_rn(__dsub_rn(2.0, mean), sdev), inv_sqrt_nsnp);
            b = inv_sqrt_nsnp / sdev;
            a = -mean * b;
        }
        lut[4 * s + 0] = v00;
        lut[4 * s + 1] = 0.0;
        lut[4 * s + 2] = v10;
        lut[4 * s + 3] = v11;
        if (coef) {
            coef[2 * s + 0] = b;
            coef[2 * s + 1] = a;
        }
    }
}

dpca_status launch_snp_stats(Handle *h) {
    ScopedLaunch t(&h->clock, h->stream, "snp_stats");
    launch_snp_stats_raw(h->P, h->pitch, h->n_ind, h->n_snp, h->inv_sqrt_nsnp, h->counts, h->avg, h->sd, h->lut,
                         h->coef, h->stream);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

// The statistics kernel on caller-given buffers: used by the allocation-free pass and by the
// streaming sweep, whose rows are one block of the matrix (inv_sqrt_nsnp is then the whole
// matrix's 1/sqrt(n_snp)).
void launch_snp_stats_raw(const uint8_t *P, int64_t pitch, int n_ind, int n_snp, double inv_sqrt_nsnp,
                          int32_t *counts, double *avg, double *sd, double *lut, double *coef, cudaStream_t stream,
                          const double *row_inv_sqrt) {
    const int64_t np = ((int64_t)n_ind + 3) / 4;
    snp_counts_kernel<<<ceil_div(n_snp, 8), 256, 0, stream>>>(P, pitch, n_ind, n_snp, np, counts);
    snp_moments_kernel<<<std::min(ceil_div(n_snp, 256), 4096), 256, 0, stream>>>(n_snp, inv_sqrt_nsnp, counts, avg,
                                                                                  sd, lut, coef, row_inv_sqrt);
}

// One thread writes one 32-bit word (16 individuals) of one SNP row; the
// genotype of (snp s, individual i) is a pure function of (key, s, i), as in
// distpca_gb300/synth.py::genotype_codes.
// row_src (optional): the cohort SNP drawn into each device row, -1 for a padding row (zero codes).
__global__ void __launch_bounds__(256) synth_fill_kernel(uint8_t *__restrict__ P, int64_t pitch, int n_ind,
                                                         int n_snp, int64_t words_per_row, uint64_t key,
                                                         const uint8_t *__restrict__ pop,
                                                         const uint32_t *__restrict__ miss_thr,
                                                         const uint32_t *__restrict__ thr, int n_pop,
                                                         const int *__restrict__ row_src) {
    int64_t total = words_per_row * (int64_t)n_snp;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = t / words_per_row;
        int64_t w = t - row * words_per_row;
        const int64_t s = row_src ? (int64_t)row_src[row] : row;
        if (s < 0) {
            *reinterpret_cast<uint32_t *>(P + row * pitch + 4 * w) = 0u;
            continue;
        }
        const uint32_t *ts = thr + s * n_pop;
        uint32_t word = 0;
#pragma unroll 4
        for (int j = 0; j < 16; ++j) {
            int64_t i = w * 16 + j;
            if (i >= n_ind) break;
            uint64_t x = (((uint64_t)s) << 32 | (uint64_t)i) ^ key;
            uint64_t hg = fmix64(x + kGold);
            uint64_t hm = fmix64(x ^ kMissSalt);
            uint32_t th = __ldg(ts + __ldg(pop + i));
            uint32_t g = ((uint32_t)hg < th ? 1u : 0u) + ((uint32_t)(hg >> 32) < th ? 1u : 0u);
            uint32_t code = g == 0 ? 0u : (g == 1 ? 2u : 3u);
            if ((uint32_t)hm < __ldg(miss_thr + i)) code = 1u;
            word |= code << (2 * j);
        }
        *reinterpret_cast<uint32_t *>(P + row * pitch + 4 * w) = word;
    }
}

dpca_status launch_synth_fill(Handle *h, uint64_t key, const uint8_t *d_pop, const uint32_t *d_miss,
                              const uint32_t *d_thr, int n_pop, const int *d_row_src) {
    int64_t wpr = (h->np + 3) / 4;
    int64_t total = wpr * h->n_snp;
    int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)h->sm_count * 32);
    synth_fill_kernel<<<grid, 256, 0, h->stream>>>(h->P, h->pitch, h->n_ind, h->n_snp, wpr, key, d_pop, d_miss,
                                                    d_thr, n_pop, d_row_src);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

// Individual-major copy: PT[i][s/4] holds the codes of SNPs s..s+3 of individual i (low bits
// first), the same 2-bit codes as P.  A block transposes a tile of 64 SNPs x 256 individuals
// through shared memory (one byte per code), reading 64 B per SNP row and writing 16 B per
// individual row.
constexpr int kTS = 64;   // SNPs per tile
constexpr int kTI = 256;  // individuals per tile

__global__ void __launch_bounds__(256) transpose_packed_kernel(const uint8_t *__restrict__ P, int64_t pitch,
                                                               uint8_t *__restrict__ PT, int64_t pitchT, int n_ind,
                                                               int n_snp, int s_base) {
    __shared__ uint8_t codes[kTS][kTI + 4];
    // SNP blocks on grid x (up to 2^31 - 1), individual blocks on y: matrices of more than
    // 65,535 SNP blocks stay launchable
    int s0 = blockIdx.x * kTS, i0 = blockIdx.y * kTI;
    int tid = threadIdx.x;
    // load: 64 rows x 64 bytes; thread -> (row, 16-byte chunk): 256 threads = 64 rows x 4 chunks
    {
        int r = tid >> 2, ch = tid & 3;
        int s = s0 + r;
        uint4 v = make_uint4(0, 0, 0, 0);
        int64_t byte0 = (int64_t)(i0 >> 2) + ch * 16;
        if (s < n_snp && byte0 < pitch) v = *reinterpret_cast<const uint4 *>(P + (int64_t)s * pitch + byte0);
        uint32_t ws[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 16; ++q) codes[r][ch * 64 + j * 16 + q] = (uint8_t)((ws[j] >> (2 * q)) & 3u);
    }
    __syncthreads();
    // store: 256 individual rows x 16 bytes (64 SNPs); thread -> one individual row
    int i = i0 + tid;
    if (i < n_ind) {
        uint32_t out[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            uint32_t w = 0;
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                int s = s0 + j * 16 + q;
                uint32_t c = s < n_snp ? (uint32_t)codes[j * 16 + q][tid] : 0u;
                w |= c << (2 * q);
            }
            out[j] = w;
        }
        // tile-blocked layout: 128 individuals x 128 bytes (512 SNPs) per contiguous 16 KB tile,
        // tiles of one row block consecutive along the SNPs, so that a TMA tile load touches one
        // contiguous range instead of 128 rows a whole matrix row apart
        const int64_t byte0 = (int64_t)((s0 + s_base) >> 2), nkt = pitchT / 128;
        uint8_t *dst = PT + (((int64_t)(i >> 7) * nkt + (byte0 >> 7)) * 128 + (i & 127)) * 128 + (byte0 & 127);
        *reinterpret_cast<uint4 *>(dst) = make_uint4(out[0], out[1], out[2], out[3]);
    }
}

// Rows [0, n_snp) of P are SNPs s_base + [0, n_snp) of PT (s_base a multiple of 64).
void launch_transpose_raw(const uint8_t *P, int64_t pitch, uint8_t *PT, int64_t pitchT, int n_ind, int n_snp,
                          cudaStream_t stream, int s_base) {
    dim3 grid(ceil_div(n_snp, kTS), ceil_div(n_ind, kTI));
    transpose_packed_kernel<<<grid, 256, 0, stream>>>(P, pitch, PT, pitchT, n_ind, n_snp, s_base);
}

dpca_status launch_transpose_packed(Handle *h) {
    ScopedLaunch t(&h->clock, h->stream, "transpose_packed");
    dim3 grid(ceil_div(h->n_snp, kTS), ceil_div(h->n_ind, kTI));
    transpose_packed_kernel<<<grid, 256, 0, h->stream>>>(h->P, h->pitch, h->PT, h->pitchT, h->n_ind, h->n_snp, 0);
    DPCA_CUDA(cudaGetLastError());
    return DPCA_OK;
}

}  // namespace dpca
